// t-column kernels: per (x,y) column, the inverse real FFT along t, the
// column phase (taper, Burgers step, sources, accumulators) and the forward
// real FFT along t, with the spectrum planes in HBM between passes.
//
// Spectrum layout in HBM: spec[plane][x*Y + y] (complex64).  One plane per
// rfft bin; the fast kernels keep the planes in their permuted slot order
// (plane = slot holding bin f, Nyquist bin in the last plane), the generic
// kernels in natural order.  The xy kernels get the bin of each plane from
// a host-built table.
//
// Reference semantics: rfft/irfft along t of angular_spectrum_solver.py
// (:215, :272, :662-664, :679, :685), the analytic-signal step of :652-654
// (realised as r2c/c2r, see the xy kernels), and numpy's irfft rule that
// drops the imaginary part of the DC and Nyquist bins.
#include "asg_internal.h"
#include "asg_column.cuh"
#include "asg_generic.cuh"

ASG_DEFINE_ROOT_UPLOADER(asg_roots_upload_t)

// ---------------------------------------------------------------------------
// fast kernel: nT = 2M, M = N1*N2 (register-resident four-step FFT)
// C columns per block, one warp per column
// ---------------------------------------------------------------------------
template <class PL, int C>
__global__ void __launch_bounds__(32 * C) tk_fast(TParams p) {
  if (*p.status != 0) return;
  constexpr int M = PL::N;
  constexpr int N1 = PL::N1;
  constexpr int N2 = PL::N2;
  constexpr int CH = (2 * M + 31) / 32;
  const int nT = 2 * M;
  extern __shared__ float4 smraw[];
  float2* lines = reinterpret_cast<float2*>(smraw);
  float2* twM = lines + C * PL::PADDED;
  float2* twT = twM + M;
  __shared__ float red_max[C];

  const int tid = threadIdx.x, nthr = blockDim.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int c0 = blockIdx.x * C;
  const int ncols = p.ncols;
  for (int i = tid; i < M; i += nthr) twM[i] = p.twM[i];
  for (int i = tid; i <= M; i += nthr) twT[i] = p.tw[i];

  float2* myline = lines + warp * PL::PADDED;
  const int mycol = c0 + warp;
  const bool active = mycol < ncols;

  // ---------------- phase 1: input ----------------
  if (p.in_real) {
    __syncthreads();
    if (active) {
      const float2* src = reinterpret_cast<const float2*>(p.real_in + (size_t)mycol * nT);
      for (int j = lane; j < M; j += 32) myline[PL::pos(j)] = src[j];
    }
    __syncwarp();
  } else {
    __syncthreads();
    const float inv2M = 0.5f / (float)M;
    const int npairs = M / 2 + 1;
    for (int it = tid; it < npairs * C; it += nthr) {
      const int cc = it % C, k = it / C;
      const int c = c0 + cc;
      if (c >= ncols) continue;
      float2* line = lines + cc * PL::PADDED;
      if (k == 0) {
        const float a = p.spec[c].x;                           // DC (imag dropped)
        const float b = p.spec[(size_t)M * ncols + c].x;       // Nyquist (imag dropped)
        line[PL::pos(0)] = make_float2((a + b) * inv2M, (a - b) * inv2M);
      } else {
        const int k2 = M - k;
        const int sk = PL::slot_of_freq(k), sk2 = PL::slot_of_freq(k2);
        const float2 xk = p.spec[(size_t)sk * ncols + c];
        const float2 xm = p.spec[(size_t)sk2 * ncols + c];
        const float2 E = make_float2(0.5f * (xk.x + xm.x), 0.5f * (xk.y - xm.y));
        const float2 D = make_float2(0.5f * (xk.x - xm.x), 0.5f * (xk.y + xm.y));
        const float2 O = cmulc(D, twT[k]);
        // Z[k] = E + iO ; Z[M-k] = conj(E) + i conj(O)
        line[PL::pos(sk)] = make_float2((E.x - O.y) * (2.f * inv2M), (E.y + O.x) * (2.f * inv2M));
        line[PL::pos(sk2)] = make_float2((E.x + O.y) * (2.f * inv2M), (-E.y + O.x) * (2.f * inv2M));
      }
    }
    __syncthreads();
    // inverse four-step on my column: B^-1 then A^-1
    if (active) {
      for (int ka = lane; ka < N1; ka += 32) stepB_smem<PL, true>(myline, ka);
      __syncwarp();
      for (int b = lane; b < N2; b += 32) stepA_inv_smem<PL>(myline, b, twM);
      __syncwarp();
    }
  }

  // ---------------- phase 2: column work ----------------
  float am = 0.f;
  if (active) {
    PaddedColumn<N2> col{reinterpret_cast<float*>(myline)};
    am = column_phase<CH>(col, mycol, nT, p.op, p.stats != 0);
    if (p.write_real) {
      float2* dst = reinterpret_cast<float2*>(p.real_out + (size_t)mycol * nT);
      for (int j = lane; j < M; j += 32) dst[j] = myline[PL::pos(j)];
    }
  }
  if (p.stats) {
    if (lane == 0) red_max[warp] = am;
    __syncthreads();
    if (tid == 0) {
      float m = 0.f;
      bool bad = false;
      for (int w = 0; w < C; ++w) {
        float v = red_max[w];
        bad |= (v != v);
        m = fmaxf(m, v);
      }
      if (bad) m = __uint_as_float(0x7fc00000u);
      atomicMax(p.op.max_next, float_as_ordered(m));
    }
  }
  if (!p.do_r2c) return;

  // ---------------- phase 3: forward real FFT ----------------
  if (active) {
    for (int b = lane; b < N2; b += 32) stepA_fwd_smem<PL, false>(myline, b, twM);
    __syncwarp();
    for (int ka = lane; ka < N1; ka += 32) stepB_smem<PL, false>(myline, ka);
  }
  __syncthreads();
  {
    const int npairs = M / 2 + 1;
    for (int it = tid; it < npairs * C; it += nthr) {
      const int cc = it % C, k = it / C;
      const int c = c0 + cc;
      if (c >= ncols) continue;
      const float2* line = lines + cc * PL::PADDED;
      if (k == 0) {
        const float2 z = line[PL::pos(0)];
        p.spec[c] = make_float2(z.x + z.y, 0.f);
        p.spec[(size_t)M * ncols + c] = make_float2(z.x - z.y, 0.f);
      } else {
        const int k2 = M - k;
        const int sk = PL::slot_of_freq(k), sk2 = PL::slot_of_freq(k2);
        const float2 zk = line[PL::pos(sk)];
        const float2 zm = line[PL::pos(sk2)];
        const float2 E = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
        // O = -i/2 (zk - conj zm)
        const float2 D = make_float2(0.5f * (zk.x - zm.x), 0.5f * (zk.y + zm.y));
        const float2 O = make_float2(D.y, -D.x);
        const float2 WO = cmul(O, twT[k]);
        p.spec[(size_t)sk * ncols + c] = make_float2(E.x + WO.x, E.y + WO.y);
        p.spec[(size_t)sk2 * ncols + c] = make_float2(E.x - WO.x, -(E.y - WO.y));
      }
    }
  }
}

// ---------------------------------------------------------------------------
// generic kernel: any nT, complex FFT of length nT on real data
// ---------------------------------------------------------------------------
template <int CH>
__global__ void __launch_bounds__(128) tk_generic(TParams p, GenPlan pl) {
  if (*p.status != 0) return;
  constexpr int C = 4;
  const int nT = p.nT;
  const int F = nT / 2 + 1;
  extern __shared__ float4 smraw[];
  float2* A = reinterpret_cast<float2*>(smraw);
  float2* B = A + C * nT;
  float2* tw = B + C * nT;
  __shared__ float red_max[C];
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int c0 = blockIdx.x * C;
  const int ncols = p.ncols;
  for (int i = tid; i < nT; i += nthr) tw[i] = p.tw[i];
  const int mycol = c0 + warp;
  const bool active = mycol < ncols;

  float* re;  // real samples, column cc at re + cc*nT
  if (p.in_real) {
    re = reinterpret_cast<float*>(B);
    for (int it = tid; it < C * nT; it += nthr) {
      const int cc = it / nT, t = it - (it / nT) * nT;
      const int c = c0 + cc;
      re[cc * nT + t] = (c < ncols) ? p.real_in[(size_t)c * nT + t] : 0.f;
    }
    __syncthreads();
  } else {
    for (int it = tid; it < C * F; it += nthr) {
      const int cc = it % C, f = it / C;
      const int c = c0 + cc;
      float2 x = (c < ncols) ? p.spec[(size_t)f * ncols + c] : make_float2(0.f, 0.f);
      float2* a = A + cc * nT;
      if (f == 0 || (2 * f == nT)) {
        a[f] = make_float2(x.x, 0.f);
      } else {
        a[f] = x;
        a[nT - f] = cconj(x);
      }
    }
    __syncthreads();
    float2* res = gen_fft<true>(A, B, C, nT, 1, pl, tw);
    float2* other = (res == A) ? B : A;
    re = reinterpret_cast<float*>(other);
    const float s = 1.0f / (float)nT;
    for (int it = tid; it < C * nT; it += nthr) re[it] = res[it].x * s;
    __syncthreads();
  }

  float am = 0.f;
  if (active) {
    PlainColumn col{re + warp * nT};
    am = column_phase<CH>(col, mycol, nT, p.op, p.stats != 0);
    if (p.write_real) {
      for (int t = lane; t < nT; t += 32) p.real_out[(size_t)mycol * nT + t] = col.get(t);
    }
  }
  if (p.stats) {
    if (lane == 0) red_max[warp] = am;
    __syncthreads();
    if (tid == 0) {
      float m = 0.f;
      bool bad = false;
      for (int w = 0; w < C; ++w) {
        float v = red_max[w];
        bad |= (v != v);
        m = fmaxf(m, v);
      }
      if (bad) m = __uint_as_float(0x7fc00000u);
      atomicMax(p.op.max_next, float_as_ordered(m));
    }
  }
  if (!p.do_r2c) return;
  __syncthreads();
  // real -> complex in the buffer that does not hold `re`
  float2* X = (reinterpret_cast<float2*>(re) == A) ? B : A;
  float2* Y = (X == A) ? B : A;
  for (int it = tid; it < C * nT; it += nthr) X[it] = make_float2(re[it], 0.f);
  __syncthreads();
  float2* res = gen_fft<false>(X, Y, C, nT, 1, pl, tw);
  for (int it = tid; it < C * F; it += nthr) {
    const int cc = it % C, f = it / C;
    const int c = c0 + cc;
    if (c < ncols) p.spec[(size_t)f * ncols + c] = res[cc * nT + f];
  }
}

// ---------------------------------------------------------------------------
// host-side launchers
// ---------------------------------------------------------------------------
template <int M>
static int launch_fast_t(const TParams& p, cudaStream_t st) {
  using PL = FastPlan<M>;
  constexpr int C = 8;
  const size_t smem = (size_t)(C * PL::PADDED + M + M + 1) * sizeof(float2);
  static bool attr_done = false;
  if (!attr_done) {
    if (cudaFuncSetAttribute(tk_fast<PL, C>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess)
      return ASG_ERR_CUDA;
    attr_done = true;
  }
  const int grid = (p.ncols + C - 1) / C;
  tk_fast<PL, C><<<grid, 32 * C, smem, st>>>(p);
  return cudaPeekAtLastError() == cudaSuccess ? ASG_OK : ASG_ERR_CUDA;
}

bool asg_t_fast_supported(int nT) {
  if (nT % 2) return false;
  switch (nT / 2) {
    case 64: case 96: case 128: case 192: case 256: case 384: case 512: case 768: case 1024:
      return true;
    default:
      return false;
  }
}

// generic: C = 4 columns of nT complex, ping-pong
size_t asg_t_generic_smem(int nT) { return (size_t)(2 * 4 * nT + nT) * sizeof(float2); }

template <int CH>
static int launch_generic_t_ch(const TParams& p, const GenPlan& pl, cudaStream_t st) {
  const size_t smem = asg_t_generic_smem(p.nT);
  if (cudaFuncSetAttribute(tk_generic<CH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return ASG_ERR_CUDA;
  const int grid = (p.ncols + 3) / 4;
  tk_generic<CH><<<grid, 128, smem, st>>>(p, pl);
  return cudaPeekAtLastError() == cudaSuccess ? ASG_OK : ASG_ERR_CUDA;
}

int asg_launch_t(const TParams& p, bool fast, const GenPlan& pl, cudaStream_t st) {
  if (fast) {
    switch (p.nT / 2) {
      case 64: return launch_fast_t<64>(p, st);
      case 96: return launch_fast_t<96>(p, st);
      case 128: return launch_fast_t<128>(p, st);
      case 192: return launch_fast_t<192>(p, st);
      case 256: return launch_fast_t<256>(p, st);
      case 384: return launch_fast_t<384>(p, st);
      case 512: return launch_fast_t<512>(p, st);
      case 768: return launch_fast_t<768>(p, st);
      case 1024: return launch_fast_t<1024>(p, st);
      default: return ASG_ERR_SHAPE;
    }
  }
  const int ch = (p.nT + 31) / 32;
  if (ch <= 4) return launch_generic_t_ch<4>(p, pl, st);
  if (ch <= 8) return launch_generic_t_ch<8>(p, pl, st);
  if (ch <= 16) return launch_generic_t_ch<16>(p, pl, st);
  if (ch <= 32) return launch_generic_t_ch<32>(p, pl, st);
  if (ch <= 64) return launch_generic_t_ch<64>(p, pl, st);
  return ASG_ERR_SHAPE;
}
