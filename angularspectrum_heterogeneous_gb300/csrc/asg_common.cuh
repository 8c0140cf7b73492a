// Shared device helpers for the angular-spectrum march kernels (sm_103a).
//
// Complex numbers are float2 (x = re, y = im).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "asg_gb300.h"

#define ASG_DEV __device__ __forceinline__

// ---------------------------------------------------------------------------
// complex arithmetic.  ASG_PACKED_F32X2 selects the Blackwell FP32x2
// instructions (FADD2/FMUL2/FFMA2); the scalar form is the default (fewer
// register-pair moves for the twiddle products).
// ---------------------------------------------------------------------------
#ifdef ASG_PACKED_F32X2
ASG_DEV float2 cadd(float2 a, float2 b) { return __fadd2_rn(a, b); }
ASG_DEV float2 csub(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
ASG_DEV float2 cscale(float2 a, float s) { return __fmul2_rn(a, make_float2(s, s)); }
// a * b
ASG_DEV float2 cmul(float2 a, float2 b) {
  float2 t = __fmul2_rn(make_float2(a.x, a.x), b);                   // (ar br, ar bi)
  return __ffma2_rn(make_float2(-a.y, a.y), make_float2(b.y, b.x), t);  // -ai bi, ai br
}
// a * conj(b)
ASG_DEV float2 cmulc(float2 a, float2 b) {
  float2 t = __fmul2_rn(make_float2(a.x, a.x), make_float2(b.x, -b.y));
  return __ffma2_rn(make_float2(a.y, a.y), make_float2(b.y, b.x), t);
}
#else
ASG_DEV float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
ASG_DEV float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
ASG_DEV float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
ASG_DEV float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
ASG_DEV float2 cmulc(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.y, b.x, -a.x * b.y));
}
#endif
ASG_DEV float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
// multiply by -i (forward) or +i (inverse)
template <bool INV>
ASG_DEV float2 mul_mi(float2 a) {
  return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// ---------------------------------------------------------------------------
// Roots of unity for the in-register DFTs.  c_w192[j] = exp(-2 pi i j / 192),
// filled by the host from FP64 values.  Every small DFT size used here divides
// 192 or 64 (sizes 2,3,4,6,8,12,16,24,32,48,64 -> W_N^j = W_192^(j*192/N)
// for N | 192; N = 64 uses c_w64).
// ---------------------------------------------------------------------------
// Each translation unit that includes this header holds its own copy of the
// tables (no relocatable device code); the host fills every copy once through
// the per-unit uploader that ASG_DEFINE_ROOT_UPLOADER defines.
static __constant__ float2 c_w192[192];
static __constant__ float2 c_w64[64];

#define ASG_DEFINE_ROOT_UPLOADER(name)                                              \
  int name(const float2* w192, const float2* w64) {                                 \
    if (cudaMemcpyToSymbol(c_w192, w192, sizeof(float2) * 192) != cudaSuccess)     \
      return -1;                                                                    \
    if (cudaMemcpyToSymbol(c_w64, w64, sizeof(float2) * 64) != cudaSuccess)         \
      return -1;                                                                    \
    return 0;                                                                       \
  }

template <int N, bool INV>
ASG_DEV float2 twiddle_const(int j) {
  // j is a compile-time constant after unrolling; the table index folds into
  // a constant-bank operand.
  float2 w;
  if constexpr (192 % N == 0) {
    w = c_w192[((j % N) * (192 / N)) % 192];
  } else {
    static_assert(64 % N == 0, "unsupported in-register DFT size");
    w = c_w64[((j % N) * (64 / N)) % 64];
  }
  return INV ? cconj(w) : w;
}

template <int N, bool INV>
ASG_DEV float2 twiddle_mul(float2 v, int j) {
  const int e = ((j % N) + N) % N;
  if (e == 0) return v;
  if (4 * e == N) return mul_mi<INV>(v);            // W^(N/4) = -i
  if (2 * e == N) return make_float2(-v.x, -v.y);   // W^(N/2) = -1
  if (4 * e == 3 * N) return mul_mi<!INV>(v);       // W^(3N/4) = +i
  return cmul(v, twiddle_const<N, INV>(e));
}

// ---------------------------------------------------------------------------
// In-register DFT of size N (natural order in, natural order out),
// forward sign exp(-2 pi i nk/N), inverse exp(+2 pi i nk/N), unnormalised.
// Recursive Cooley-Tukey split N = P*Q with compile-time indices only.
// ---------------------------------------------------------------------------
template <int N>
struct DftSplit {
  static constexpr int P = (N % 4 == 0 && N > 4) ? ((N % 8 == 0 && N >= 64) ? 8 : 4)
                                                 : ((N % 2 == 0) ? 2 : 3);
  static constexpr int Q = N / P;
};

template <int N, bool INV>
ASG_DEV void dft(float2 (&v)[N]) {
  if constexpr (N == 1) {
    return;
  } else if constexpr (N == 2) {
    float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  } else if constexpr (N == 3) {
    // exp(-2 pi i/3) = -1/2 - i sqrt(3)/2
    const float s3 = INV ? 0.86602540378443864676f : -0.86602540378443864676f;
    float2 a = v[0], b = v[1], c = v[2];
    float2 t = cadd(b, c);
    float2 d = csub(b, c);
    v[0] = cadd(a, t);
    float2 m = make_float2(a.x - 0.5f * t.x, a.y - 0.5f * t.y);
    // (b - c) * i * s3
    float2 r = make_float2(-s3 * d.y, s3 * d.x);
    v[1] = cadd(m, r);
    v[2] = csub(m, r);
  } else if constexpr (N == 4) {
    float2 a = v[0], b = v[1], c = v[2], d = v[3];
    float2 s0 = cadd(a, c), d0 = csub(a, c);
    float2 s1 = cadd(b, d), d1 = mul_mi<INV>(csub(b, d));
    v[0] = cadd(s0, s1);
    v[2] = csub(s0, s1);
    v[1] = cadd(d0, d1);
    v[3] = csub(d0, d1);
  } else {
    constexpr int P = DftSplit<N>::P;
    constexpr int Q = DftSplit<N>::Q;
    // input n = Q*p + q ; output k = ka + P*kb.  Stage 1 runs in place on v
    // (stride-Q subsequences), stage 2 writes each block straight into its
    // output positions; with compile-time indices the final permutation is a
    // register renaming, so about N complex values are live at any time.
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      float2 t[P];
#pragma unroll
      for (int p = 0; p < P; ++p) t[p] = v[Q * p + q];
      dft<P, INV>(t);
#pragma unroll
      for (int ka = 0; ka < P; ++ka) v[Q * ka + q] = twiddle_mul<N, INV>(t[ka], q * ka);
    }
    float2 o[N];
#pragma unroll
    for (int ka = 0; ka < P; ++ka) {
      float2 t[Q];
#pragma unroll
      for (int q = 0; q < Q; ++q) t[q] = v[Q * ka + q];
      dft<Q, INV>(t);
#pragma unroll
      for (int kb = 0; kb < Q; ++kb) o[ka + P * kb] = t[kb];
    }
#pragma unroll
    for (int i = 0; i < N; ++i) v[i] = o[i];
  }
}

// ---------------------------------------------------------------------------
// Two-level line FFT of length N = N1*N2 in shared memory ("four-step").
//   forward, step A: for each b in [0,N2): DFT_N1 over a of x[b + N2 a],
//                    times W_N^(b ka), stored at slot b + N2 ka
//   forward, step B: for each ka in [0,N1): DFT_N2 over b of slots b + N2 ka,
//                    stored at slot kb + N2 ka  -> frequency ka + N1 kb
// The inverse runs B^-1 then A^-1 and takes the permuted slots back to
// natural order.  Slots are padded by two complex every N2 slots
// (position s + 2*(s/N2)): step A's strided 8-byte accesses and step B's
// contiguous 16-byte accesses are both free of bank conflicts, and an even
// slot stays 16-byte aligned.
// ---------------------------------------------------------------------------
template <int N1_, int N2_>
struct LinePlan {
  static constexpr int N1 = N1_;
  static constexpr int N2 = N2_;
  static constexpr int N = N1 * N2;
  static constexpr int PADDED = N + 2 * N1;  // padded slots per line
  ASG_DEV static int pos(int s) { return s + 2 * (s / N2); }
  // slot holding frequency k
  __host__ __device__ static int slot_of_freq(int k) { return (k / N1) + N2 * (k % N1); }
  __host__ __device__ static int freq_of_slot(int s) { return (s / N2) + N1 * (s % N2); }
};

// Fast sizes: N -> (N1, N2)
template <int N> struct FastPlan;
template <> struct FastPlan<32> : LinePlan<4, 8> {};
template <> struct FastPlan<64> : LinePlan<8, 8> {};
template <> struct FastPlan<96> : LinePlan<8, 12> {};
template <> struct FastPlan<128> : LinePlan<8, 16> {};
template <> struct FastPlan<192> : LinePlan<12, 16> {};
template <> struct FastPlan<256> : LinePlan<16, 16> {};
template <> struct FastPlan<384> : LinePlan<16, 24> {};
template <> struct FastPlan<512> : LinePlan<16, 32> {};
template <> struct FastPlan<768> : LinePlan<24, 32> {};
template <> struct FastPlan<1024> : LinePlan<32, 32> {};

// step A on one subline (column b) of a line starting at `line` (padded
// layout); tw = W_N^j table (N entries, smem or global)
template <class PL, bool INV>
ASG_DEV void stepA_fwd_smem(float2* line, int b, const float2* tw) {
  float2 v[PL::N1];
#pragma unroll
  for (int a = 0; a < PL::N1; ++a) v[a] = line[PL::pos(b + PL::N2 * a)];
  dft<PL::N1, false>(v);
#pragma unroll
  for (int ka = 0; ka < PL::N1; ++ka) {
    // b*ka <= (N2-1)(N1-1) < N: no reduction needed
    line[PL::pos(b + PL::N2 * ka)] = ka == 0 ? v[0] : cmul(v[ka], tw[b * ka]);
  }
}

template <class PL, bool INV>
ASG_DEV void stepB_smem(float2* line, int ka) {
  static_assert(PL::N2 % 2 == 0, "step B reads complex pairs");
  float2 v[PL::N2];
  float4* p = reinterpret_cast<float4*>(line + ka * (PL::N2 + 2));  // pos(N2*ka)
#pragma unroll
  for (int b = 0; b < PL::N2 / 2; ++b) {
    const float4 q = p[b];
    v[2 * b] = make_float2(q.x, q.y);
    v[2 * b + 1] = make_float2(q.z, q.w);
  }
  dft<PL::N2, INV>(v);
#pragma unroll
  for (int b = 0; b < PL::N2 / 2; ++b)
    p[b] = make_float4(v[2 * b].x, v[2 * b].y, v[2 * b + 1].x, v[2 * b + 1].y);
}

// inverse step A: twiddle conj(W^(b ka)) then inverse DFT_N1 over ka -> a
template <class PL>
ASG_DEV void stepA_inv_smem(float2* line, int b, const float2* tw) {
  float2 v[PL::N1];
#pragma unroll
  for (int ka = 0; ka < PL::N1; ++ka) {
    float2 x = line[PL::pos(b + PL::N2 * ka)];
    v[ka] = ka == 0 ? x : cmulc(x, tw[b * ka]);
  }
  dft<PL::N1, true>(v);
#pragma unroll
  for (int a = 0; a < PL::N1; ++a) line[PL::pos(b + PL::N2 * a)] = v[a];
}

// ---------------------------------------------------------------------------
// misc
// ---------------------------------------------------------------------------
ASG_DEV unsigned int float_as_ordered(float f) {
  // non-negative floats order as unsigned ints; NaN payloads sort above inf
  return __float_as_uint(f);
}

template <typename T>
ASG_DEV T warp_sum(T v, unsigned mask = 0xffffffffu) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o);
  return v;
}
ASG_DEV float warp_max(float v, unsigned mask = 0xffffffffu) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(mask, v, o));
  return v;
}
ASG_DEV float warp_min(float v, unsigned mask = 0xffffffffu) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(mask, v, o));
  return v;
}
