// Learned KT corrector: a 1-D convolutional network along t that corrects one
// coarse KT step of a column towards the fully sub-cycled KT step.
//
//   h1 = GELU(conv(x,  W1[64,1,5])  + b1)      CUDA cores (GELU in its tanh form)
//   h2 = GELU(conv(h1, W2[64,64,5]) + b2)      BF16 tensor cores, FP32 accumulation
//   h3 = GELU(conv(h2, W3[64,64,5]) + b3)      BF16 tensor cores, FP32 accumulation
//   y  =      conv(h3, W4[1,64,5])  + b4       CUDA cores
//   conv(x, W)[o, t] = sum_i sum_j W[o, i, j] x[i, t + j - 2], zero outside the column
//
// The reference solver has no learned part; its KT scheme (_kt_flux /
// _kt_flux_adaptive, angular_spectrum_solver.py:833-859) produces the
// training targets through the column kernels of this library.
//
// Data layout: a batch of ncols columns of nT samples (nT % 128 == 0), position
// pos = column * nT + t.  Activations are position-major [pos][64 channels]
// (BF16, 128 B per position); pre-activations z are kept in FP32 for the
// backward pass.  Parameters live in one FP32 vector theta (layout below);
// the two 64x64 layers are packed to BF16 GEMM operands Wg[o][j*64 + i] (and
// their transposes for the backward data pass) after every update.
//
// The 64x64 layers are GEMMs with M = 64 output channels, N = positions,
// K = 5 taps x 64 input channels, issued as mma.sync.m16n8k16 BF16 tiles.
#include <math.h>
#include <stdio.h>
#include <stdint.h>
#include <string.h>

#include <cuda_bf16.h>

#include <vector>

#include "asg_internal.h"

namespace {

typedef unsigned short bf16_t;  // raw bfloat16 bits

constexpr int NCH = 64, KT5 = 5, KDIM = NCH * KT5;  // 320
// theta layout (floats)
constexpr int OFF_W1 = 0;                     // [64][5]        (o, j)
constexpr int OFF_B1 = OFF_W1 + NCH * KT5;    // [64]
constexpr int OFF_W2 = OFF_B1 + NCH;          // [64][64][5]    (o, i, j)
constexpr int OFF_B2 = OFF_W2 + NCH * KDIM;
constexpr int OFF_W3 = OFF_B2 + NCH;
constexpr int OFF_B3 = OFF_W3 + NCH * KDIM;
constexpr int OFF_W4 = OFF_B3 + NCH;          // [64][5]        (i, j)
constexpr int OFF_B4 = OFF_W4 + NCH * KT5;    // [1]
constexpr int NPARAM = OFF_B4 + 1;            // 41793

__device__ __forceinline__ bf16_t f2bf(float f) {
  // round to nearest even: one cvt.rn.bf16.f32
  return __bfloat16_as_ushort(__float2bfloat16_rn(f));
}
__device__ __forceinline__ float bf2f(bf16_t h) { return __uint_as_float(((unsigned)h) << 16); }

// GELU in its tanh form, 0.5 z (1 + tanh(sqrt(2/pi) (z + 0.044715 z^3))), with
// the hardware tanh (relative error ~2^-11, below the BF16 rounding of the
// activations); the derivative uses the same tanh value.
__device__ __forceinline__ float tanh_hw(float u) {
  float t;
  asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(u));
  return t;
}
__device__ __forceinline__ float gelu_f(float z) {
  const float t = tanh_hw(0.7978845608028654f * fmaf(0.044715f * z * z, z, z));
  return 0.5f * z * (1.f + t);
}
__device__ __forceinline__ float gelu_grad_f(float z) {
  const float t = tanh_hw(0.7978845608028654f * fmaf(0.044715f * z * z, z, z));
  return 0.5f * (1.f + t) +
         0.5f * z * (1.f - t * t) * 0.7978845608028654f * fmaf(0.134145f, z * z, 1.f);
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], unsigned a0, unsigned a1, unsigned a2,
                                         unsigned a3, unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// ---------------------------------------------------------------------------
// 64 -> 64 channel convolution as a tensor-core GEMM.
//   acc[pos][o] = sum_{j,i} Wg[o][j*64 + i] X[pos + j - 2][i]   (zero outside the column)
// MODE 0 (forward):  z = acc + bias[o];  Z[pos][o] = z (if Z), H[pos][o] = bf16(GELU(z))
// MODE 1 (backward data): d = acc * GELU'(Zin[pos][o]);  H[pos][o] = bf16(d)
// A block of 4 warps owns 64 positions x 64 channels per tile (persistent over
// tiles); warp w computes positions w*16 .. w*16+15 for all 64 channels.
// ---------------------------------------------------------------------------
constexpr int WS = KDIM + 8;   // row stride of the weight tile (bf16): conflict-free ldmatrix rows
constexpr int XS = NCH + 8;    // row stride of the activation tile
constexpr int TP = 64;         // positions per chunk of the weight-gradient kernel
constexpr int TPC = 128;       // positions per tile of the convolution kernel
constexpr size_t CONV_SMEM =
    (size_t)(NCH * WS + (TPC + 4) * XS) * sizeof(bf16_t) + (TPC + 8) * sizeof(float);

__device__ __forceinline__ void ldsm_x4(unsigned (&r)[4], const void* p) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(a));
}

// A block of 4 warps owns 128 positions x 64 channels per tile (persistent
// over tiles); warp w computes positions w*32 .. w*32+31 (4 n-tiles) for all
// 64 channels (4 m-tiles): per k-step of 16, four ldmatrix.x4 for the weight
// fragments, two for the activation fragments, sixteen MMAs.
// FUSE_L1 (inference): X is the FP32 network input x; the staged rows are the
// first layer's output h1 = GELU(b1 + conv(x, W1)), computed in place of a
// load (zero outside the column), so h1 never goes to memory.
template <int MODE, bool FUSE_L1 = false>
__global__ void __launch_bounds__(128) k_conv64(const void* __restrict__ Xv,
                                                const bf16_t* __restrict__ Wg,
                                                const float* __restrict__ bias,
                                                const float* __restrict__ Zin,
                                                float* __restrict__ Zout,
                                                bf16_t* __restrict__ H, int npos, int nT,
                                                const float* __restrict__ th = nullptr) {
  extern __shared__ uint4 smem_u4[];
  bf16_t* Ws = reinterpret_cast<bf16_t*>(smem_u4);
  bf16_t* Xs = Ws + NCH * WS;  // input rows pos0-2 .. pos0+TPC+1; reused for the output tile
  float* xs = reinterpret_cast<float*>(Xs + (TPC + 4) * XS);  // FUSE_L1: x[pos0-4 .. pos0+TPC+3]
  const bf16_t* X = static_cast<const bf16_t*>(Xv);
  const float* xin = static_cast<const float*>(Xv);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int gid = lane >> 2, tig = lane & 3;
  const int lm = lane >> 3, lr = lane & 7;  // ldmatrix: matrix and row this lane addresses
  float w1[KT5], b1 = 0.f;  // FUSE_L1: the first layer's weights of channel tid % 64
  if (FUSE_L1) {
#pragma unroll
    for (int j = 0; j < KT5; ++j) w1[j] = th[OFF_W1 + (tid & 63) * KT5 + j];
    b1 = th[OFF_B1 + (tid & 63)];
  }
  // weights once per block: 64 rows of 320 bf16 = 40 uint4 each
  for (int i = tid; i < NCH * (KDIM / 8); i += blockDim.x) {
    const int o = i / (KDIM / 8), c = i - o * (KDIM / 8);
    *reinterpret_cast<uint4*>(Ws + o * WS + c * 8) =
        *reinterpret_cast<const uint4*>(Wg + (size_t)o * KDIM + c * 8);
  }
  const int ntiles = npos / TPC;
  const int nb = warp * 32;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int pos0 = tile * TPC;
    const int cbeg = (pos0 / nT) * nT, cend = cbeg + nT;
    __syncthreads();  // previous tile's readers are done (and the weights are in)
    if (FUSE_L1) {
      for (int i = tid; i < TPC + 8; i += blockDim.x) {
        const int pos = pos0 - 4 + i;
        xs[i] = (pos >= cbeg && pos < cend) ? xin[pos] : 0.f;
      }
      __syncthreads();
      const int o = tid & 63;
      for (int r = tid >> 6; r < TPC + 4; r += 2) {
        const int pos = pos0 - 2 + r;
        float v = 0.f;
        if (pos >= cbeg && pos < cend) {
          float z = b1;
#pragma unroll
          for (int j = 0; j < KT5; ++j) z = fmaf(w1[j], xs[r + j], z);  // x[pos + j - 2]
          v = gelu_f(z);
        }
        Xs[r * XS + o] = f2bf(v);
      }
    } else {
      for (int i = tid; i < (TPC + 4) * (NCH / 8); i += blockDim.x) {
        const int r = i / (NCH / 8), c = i - r * (NCH / 8);
        const int pos = pos0 - 2 + r;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (pos >= cbeg && pos < cend) v = *reinterpret_cast<const uint4*>(X + (size_t)pos * NCH + c * 8);
        *reinterpret_cast<uint4*>(Xs + r * XS + c * 8) = v;
      }
    }
    __syncthreads();
    float acc[4][4][4];
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
      for (int n = 0; n < 4; ++n)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[m][n][q] = 0.f;
#pragma unroll 1
    for (int j = 0; j < KT5; ++j) {
#pragma unroll
      for (int cb = 0; cb < 4; ++cb) {
        const int k0 = j * NCH + cb * 16;
        // B fragments of n-tiles (0,1) and (2,3): matrices (nt, k 0-7), (nt, k 8-15)
        unsigned b[2][4];
#pragma unroll
        for (int h = 0; h < 2; ++h)
          ldsm_x4(b[h], Xs + (nb + h * 16 + (lm >> 1) * 8 + lr + j) * XS + cb * 16 + (lm & 1) * 8);
#pragma unroll
        for (int m = 0; m < 4; ++m) {
          unsigned a[4];  // matrices (rows 0-7, k 0-7), (8-15, 0-7), (0-7, 8-15), (8-15, 8-15)
          ldsm_x4(a, Ws + (m * 16 + (lm & 1) * 8 + lr) * WS + k0 + (lm >> 1) * 8);
#pragma unroll
          for (int n = 0; n < 4; ++n)
            mma_bf16(acc[m][n], a[0], a[1], a[2], a[3], b[n >> 1][(n & 1) * 2],
                     b[n >> 1][(n & 1) * 2 + 1]);
        }
      }
    }
    // epilogue: acc[m][n][q] -> channel o = m*16 + gid (+8 for q >= 2),
    //           position nb + n*8 + tig*2 (+1 for odd q)
    if (MODE == 0 && Zout == nullptr) {
      // inference: GELU into the (now free) input tile, then 16-byte stores
      __syncthreads();
#pragma unroll
      for (int m = 0; m < 4; ++m)
#pragma unroll
        for (int n = 0; n < 4; ++n)
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int o = m * 16 + gid + (q >= 2 ? 8 : 0);
            const int pl = nb + n * 8 + tig * 2 + (q & 1);
            Xs[pl * XS + o] = f2bf(gelu_f(acc[m][n][q] + bias[o]));
          }
      __syncthreads();
      for (int i = tid; i < TPC * (NCH / 8); i += blockDim.x) {
        const int r = i / (NCH / 8), c = i - r * (NCH / 8);
        *reinterpret_cast<uint4*>(H + (size_t)(pos0 + r) * NCH + c * 8) =
            *reinterpret_cast<const uint4*>(Xs + r * XS + c * 8);
      }
      continue;
    }
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
      for (int n = 0; n < 4; ++n)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int o = m * 16 + gid + (q >= 2 ? 8 : 0);
          const size_t pos = (size_t)pos0 + nb + n * 8 + tig * 2 + (q & 1);
          const size_t idx = pos * NCH + o;
          if (MODE == 0) {
            const float z = acc[m][n][q] + bias[o];
            if (Zout) Zout[idx] = z;
            H[idx] = f2bf(gelu_f(z));
          } else {
            H[idx] = f2bf(acc[m][n][q] * gelu_grad_f(Zin[idx]));
          }
        }
  }
}

// ---------------------------------------------------------------------------
// 64 -> 64 convolution for inference on the 5th-generation tensor cores
// (tcgen05.mma, BF16 operands from shared memory, FP32 accumulator in TMEM).
//   D[pos][o] = sum_j sum_i X[pos + j - 2][i] W[o][i][j]
// A tile of 128 positions is one M = 128, N = 64 GEMM accumulated over 5 taps x
// 4 channel blocks (K = 16 each): 20 MMAs issued by one thread.  Operands are
// K-major without swizzle: the activation tile is stored K-chunk-major
// (8 channels x 132 rows of 16 B per chunk, rows contiguous), so the tap shift
// j is a 16 j-byte offset of the descriptor's start address and one staged
// tile serves all five taps.  The weights of each tap are stored the same way
// (8 chunks x 64 rows), once per CTA.  The epilogue reads the accumulator
// with tcgen05.ld (warp w: TMEM lanes = positions 32w .. 32w+31), applies bias
// and GELU and writes BF16 rows.  Every wait is bounded; on a timeout the
// kernel sets *err, frees its TMEM and returns.
// ---------------------------------------------------------------------------
constexpr int TC_ROWS = TPC + 4;                 // staged rows pos0-2 .. pos0+129
constexpr int TC_LBO_X = TC_ROWS * 16;           // bytes between 8-channel chunks of the tile
constexpr int TC_W_BYTES = KT5 * 8 * NCH * 16;   // 40 KB of weights
constexpr int TC_X_BYTES = 8 * TC_LBO_X;         // 16.5 KB of activations
constexpr size_t TC_SMEM =
    (size_t)TC_W_BYTES + 2 * ((size_t)TC_X_BYTES + (TPC + 8) * sizeof(float) + 64);

__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  // shared-memory matrix descriptor: start, leading (K) and stride (8-row group)
  // byte offsets in 16-byte units, descriptor version 1, no swizzle
  return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

// instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N = 64, M = 128
constexpr uint32_t TC_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(NCH >> 3) << 17) |
                              ((uint32_t)(TPC >> 4) << 24);

// barrier of one warpgroup (128 threads) of the CTA
__device__ __forceinline__ void wg_sync(int half) {
  asm volatile("bar.sync %0, 128;\n" ::"r"(1 + half) : "memory");
}
__device__ __forceinline__ bool wg_any(int half, bool v) {
  uint32_t r;
  asm volatile(
      "{\n.reg .pred p, q;\nsetp.ne.u32 p, %1, 0;\nbar.red.or.pred q, %2, 128, p;\n"
      "selp.u32 %0, 1, 0, q;\n}\n"
      : "=r"(r)
      : "r"((uint32_t)v), "r"(1 + half)
      : "memory");
  return r != 0;
}

// Two warpgroups per CTA, each with its own tile stream, staging buffer,
// mbarrier and 64 TMEM columns; the weights are shared.
template <bool FUSE_L1>
__global__ void __launch_bounds__(256) k_conv64_tc(const void* __restrict__ Xv,
                                                   const bf16_t* __restrict__ Wtc,
                                                   const float* __restrict__ bias,
                                                   bf16_t* __restrict__ H, int npos, int nT,
                                                   const float* __restrict__ th,
                                                   int* __restrict__ err) {
  extern __shared__ uint4 smem_u4[];
  unsigned char* sm = reinterpret_cast<unsigned char*>(smem_u4);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int half = warp >> 2, ht = tid & 127;
  unsigned char* Ws = sm;                       // [tap][chunk][64 rows][16 B]
  unsigned char* mine = sm + TC_W_BYTES + half * (TC_X_BYTES + (TPC + 8) * sizeof(float) + 64);
  unsigned char* Xs = mine;                     // [chunk][132 rows][16 B]
  float* xs = reinterpret_cast<float*>(Xs + TC_X_BYTES);  // FUSE_L1: x[pos0-4 .. pos0+131]
  uint64_t* mbar = reinterpret_cast<uint64_t*>(xs + TPC + 8);
  __shared__ uint32_t tslot;
  const bf16_t* X = static_cast<const bf16_t*>(Xv);
  const float* xin = static_cast<const float*>(Xv);
  for (int i = tid; i < TC_W_BYTES / 16; i += blockDim.x)
    reinterpret_cast<uint4*>(Ws)[i] = reinterpret_cast<const uint4*>(Wtc)[i];
  float w1[KT5], b1 = 0.f;
  if (FUSE_L1) {
#pragma unroll
    for (int j = 0; j < KT5; ++j) w1[j] = th[OFF_W1 + (ht & 63) * KT5 + j];
    b1 = th[OFF_B1 + (ht & 63)];
  }
  const uint32_t mbar_a = (uint32_t)__cvta_generic_to_shared(mbar);
  if (ht == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mbar_a));
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;\n" ::"r"(
        (uint32_t)__cvta_generic_to_shared(&tslot)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tslot + (uint32_t)(half * 64);  // my 64 accumulator columns
  const uint32_t xs_a = (uint32_t)__cvta_generic_to_shared(Xs);
  const uint32_t ws_a = (uint32_t)__cvta_generic_to_shared(Ws);
  const int ntiles = npos / TPC;
  uint32_t phase = 0;
  for (int tile = 2 * blockIdx.x + half; tile < ntiles; tile += 2 * gridDim.x) {
    const int pos0 = tile * TPC;
    const int cbeg = (pos0 / nT) * nT, cend = cbeg + nT;
    // ---- stage the tile (rows pos0-2 .. pos0+129, zero outside the column) ----
    if (FUSE_L1) {
      for (int i = ht; i < TPC + 8; i += 128) {
        const int pos = pos0 - 4 + i;
        xs[i] = (pos >= cbeg && pos < cend) ? xin[pos] : 0.f;
      }
      wg_sync(half);
      const int o = ht & 63;
      for (int r = ht >> 6; r < TC_ROWS; r += 2) {
        const int pos = pos0 - 2 + r;
        float v = 0.f;
        if (pos >= cbeg && pos < cend) {
          float z = b1;
#pragma unroll
          for (int j = 0; j < KT5; ++j) z = fmaf(w1[j], xs[r + j], z);
          v = gelu_f(z);
        }
        *reinterpret_cast<bf16_t*>(Xs + (o >> 3) * TC_LBO_X + r * 16 + (o & 7) * 2) = f2bf(v);
      }
    } else {
      for (int i = ht; i < TC_ROWS * 8; i += 128) {
        const int r = i >> 3, c = i & 7;
        const int pos = pos0 - 2 + r;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (pos >= cbeg && pos < cend) v = *reinterpret_cast<const uint4*>(X + (size_t)pos * NCH + c * 8);
        *reinterpret_cast<uint4*>(Xs + c * TC_LBO_X + r * 16) = v;
      }
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    wg_sync(half);
    // ---- 20 MMAs by one thread of the warpgroup, completion to its mbarrier ----
    if (ht == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
#pragma unroll
      for (int j = 0; j < KT5; ++j)
#pragma unroll
        for (int cb = 0; cb < 4; ++cb) {
          const uint64_t da = tc_desc(xs_a + (2 * cb) * TC_LBO_X + j * 16, TC_LBO_X, 128);
          const uint64_t db = tc_desc(ws_a + (j * 8 + 2 * cb) * (NCH * 16), NCH * 16, 128);
          const uint32_t acc = (j | cb) ? 1u : 0u;
          asm volatile(
              "{\n.reg .pred p;\nsetp.ne.u32 p, %4, 0;\n"
              "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
              "l"(da), "l"(db), "r"(TC_IDESC), "r"(acc));
        }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar_a)
          : "memory");
    }
    // ---- bounded wait for the accumulator ----
    int ok = 0;
    for (int it = 0; it < (1 << 20); ++it) {
      uint32_t done;
      asm volatile(
          "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
          "selp.u32 %0, 1, 0, p;\n}\n"
          : "=r"(done)
          : "r"(mbar_a), "r"(phase)
          : "memory");
      if (done) {
        ok = 1;
        break;
      }
    }
    phase ^= 1u;
    if (wg_any(half, !ok)) {
      if (ht == 0) atomicExch(err, 1);
      break;
    }
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    // ---- epilogue: my position's 64 channels ----
    const int row = (warp & 3) * 32 + lane;
    const size_t pos = (size_t)pos0 + row;
#pragma unroll
    for (int c0 = 0; c0 < NCH; c0 += 16) {
      uint32_t r[16];
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
          "[%16];\n"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
            "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
            "=r"(r[14]), "=r"(r[15])
          : "r"(tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)c0));
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
      unsigned pk[8];
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        const float lo = gelu_f(__uint_as_float(r[2 * e]) + bias[c0 + 2 * e]);
        const float hi = gelu_f(__uint_as_float(r[2 * e + 1]) + bias[c0 + 2 * e + 1]);
        pk[e] = (unsigned)f2bf(lo) | ((unsigned)f2bf(hi) << 16);
      }
      uint4* dst = reinterpret_cast<uint4*>(H + pos * NCH + c0);
      dst[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
      dst[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    wg_sync(half);  // accumulator read and tile consumed before the next tile
  }
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;\n" ::"r"(tslot));
}

// ---------------------------------------------------------------------------
// Last layer (64 -> 1) on the tensor cores for inference:
//   y[pos] = b4 + sum_{j,i} W4[i][j] h3[pos + j - 2][i]
// as a GEMM whose A operand has two non-zero rows, the BF16 high and low parts
// of W4 (so the weights keep ~16 bits), and whose sum the epilogue forms.
// Same tile scheme as k_conv64 with one m-tile.
// ---------------------------------------------------------------------------
constexpr size_t OUT_SMEM = (size_t)(16 * WS + (TPC + 4) * XS) * sizeof(bf16_t);

__global__ void __launch_bounds__(128) k_conv_out(const bf16_t* __restrict__ X,
                                                  const bf16_t* __restrict__ Wg4,
                                                  const float* __restrict__ th,
                                                  float* __restrict__ y, int npos, int nT) {
  extern __shared__ uint4 smem_u4[];
  bf16_t* Ws = reinterpret_cast<bf16_t*>(smem_u4);
  bf16_t* Xs = Ws + 16 * WS;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int gid = lane >> 2, tig = lane & 3;
  const int lm = lane >> 3, lr = lane & 7;
  for (int i = tid; i < 16 * (KDIM / 8); i += blockDim.x) {
    const int o = i / (KDIM / 8), c = i - o * (KDIM / 8);
    *reinterpret_cast<uint4*>(Ws + o * WS + c * 8) =
        *reinterpret_cast<const uint4*>(Wg4 + (size_t)o * KDIM + c * 8);
  }
  const float b4 = th[OFF_B4];
  const int ntiles = npos / TPC;
  const int nb = warp * 32;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int pos0 = tile * TPC;
    const int cbeg = (pos0 / nT) * nT, cend = cbeg + nT;
    __syncthreads();
    for (int i = tid; i < (TPC + 4) * (NCH / 8); i += blockDim.x) {
      const int r = i / (NCH / 8), c = i - r * (NCH / 8);
      const int pos = pos0 - 2 + r;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (pos >= cbeg && pos < cend) v = *reinterpret_cast<const uint4*>(X + (size_t)pos * NCH + c * 8);
      *reinterpret_cast<uint4*>(Xs + r * XS + c * 8) = v;
    }
    __syncthreads();
    float acc[4][4];
#pragma unroll
    for (int n = 0; n < 4; ++n)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[n][q] = 0.f;
#pragma unroll 1
    for (int j = 0; j < KT5; ++j) {
#pragma unroll
      for (int cb = 0; cb < 4; ++cb) {
        const int k0 = j * NCH + cb * 16;
        unsigned b[2][4], a[4];
#pragma unroll
        for (int h = 0; h < 2; ++h)
          ldsm_x4(b[h], Xs + (nb + h * 16 + (lm >> 1) * 8 + lr + j) * XS + cb * 16 + (lm & 1) * 8);
        ldsm_x4(a, Ws + ((lm & 1) * 8 + lr) * WS + k0 + (lm >> 1) * 8);
#pragma unroll
        for (int n = 0; n < 4; ++n)
          mma_bf16(acc[n], a[0], a[1], a[2], a[3], b[n >> 1][(n & 1) * 2], b[n >> 1][(n & 1) * 2 + 1]);
      }
    }
    // rows 0 (high part) and 1 (low part) sit in lanes gid = 0 and gid = 1
#pragma unroll
    for (int n = 0; n < 4; ++n)
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const float lo = __shfl_down_sync(0xffffffffu, acc[n][q], 4);
        if (gid == 0) y[(size_t)pos0 + nb + n * 8 + tig * 2 + q] = acc[n][q] + lo + b4;
      }
  }
}

// ---------------------------------------------------------------------------
// Weight gradient of a 64 -> 64 layer:
//   dW[o][i][j] += sum_pos D[pos][o] X[pos + j - 2][i]
// GEMM with M = o (64), N = (j, i) (320, split in 4 slabs of 80 over
// blockIdx.y), K = positions (64 per chunk).  Tiles are staged
// channel-major so that A fragments pair consecutive positions.
// ---------------------------------------------------------------------------
constexpr int WG_SLAB = 80;
constexpr int DT_S = TP + 8;       // stride of the staged D^T tile [64][TP]
constexpr int XT_S = TP + 4 + 4;   // stride of the staged X^T tile [64][TP + 4]
constexpr size_t WGRAD_SMEM = (size_t)(NCH * DT_S + NCH * XT_S) * sizeof(bf16_t);

__global__ void __launch_bounds__(128) k_conv64_wgrad(const bf16_t* __restrict__ D,
                                                      const bf16_t* __restrict__ X,
                                                      float* __restrict__ dW, int npos, int nT) {
  extern __shared__ uint4 smem_u4[];
  bf16_t* Dt = reinterpret_cast<bf16_t*>(smem_u4);
  bf16_t* Xt = Dt + NCH * DT_S;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int gid = lane >> 2, tig = lane & 3;
  const int slab = blockIdx.y;      // n-range [slab*80, +80)
  const int m0 = warp * 16;         // output channels of this warp
  float acc[10][4];
#pragma unroll
  for (int n = 0; n < 10; ++n)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[n][q] = 0.f;
  const int nchunks = npos / TP;
  for (int ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
    const int pos0 = ch * TP;
    const int cbeg = (pos0 / nT) * nT, cend = cbeg + nT;
    __syncthreads();
    for (int i = tid; i < TP * NCH; i += blockDim.x) {
      const int p = i / NCH, o = i - p * NCH;
      Dt[o * DT_S + p] = D[(size_t)(pos0 + p) * NCH + o];
    }
    for (int i = tid; i < (TP + 4) * NCH; i += blockDim.x) {
      const int r = i / NCH, c = i - r * NCH;
      const int pos = pos0 - 2 + r;
      Xt[c * XT_S + r] = (pos >= cbeg && pos < cend) ? X[(size_t)pos * NCH + c] : (bf16_t)0;
    }
    __syncthreads();
#pragma unroll
    for (int ks = 0; ks < TP / 16; ++ks) {
      const int p0 = ks * 16;
      const bf16_t* ar = Dt + (m0 + gid) * DT_S + p0 + tig * 2;
      const unsigned a0 = *reinterpret_cast<const unsigned*>(ar);
      const unsigned a1 = *reinterpret_cast<const unsigned*>(ar + 8 * DT_S);
      const unsigned a2 = *reinterpret_cast<const unsigned*>(ar + 8);
      const unsigned a3 = *reinterpret_cast<const unsigned*>(ar + 8 * DT_S + 8);
#pragma unroll
      for (int n = 0; n < 10; ++n) {
        const int kk = slab * WG_SLAB + n * 8 + gid;  // column (j, i) of this lane's B values
        const int j = kk / NCH, i = kk - j * NCH;
        // B[k = position][n = (j, i)] = X[p + j - 2][i] = Xt[i][p + j]
        const bf16_t* xr = Xt + i * XT_S + p0 + tig * 2 + j;
        const unsigned b0 = (unsigned)xr[0] | ((unsigned)xr[1] << 16);
        const unsigned b1 = (unsigned)xr[8] | ((unsigned)xr[9] << 16);
        mma_bf16(acc[n], a0, a1, a2, a3, b0, b1);
      }
    }
  }
  // acc[n][q]: o = m0 + gid (+8 for q >= 2), k = slab*80 + n*8 + tig*2 (+1 for odd q)
#pragma unroll
  for (int n = 0; n < 10; ++n)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int o = m0 + gid + (q >= 2 ? 8 : 0);
      const int kk = slab * WG_SLAB + n * 8 + tig * 2 + (q & 1);
      const int j = kk / NCH, i = kk - j * NCH;
      atomicAdd(dW + (size_t)o * KDIM + i * KT5 + j, acc[n][q]);
    }
}

// bias gradient: db[o] += sum_pos D[pos][o]
__global__ void k_bias_grad(const bf16_t* __restrict__ D, float* __restrict__ db, int npos) {
  __shared__ float part[256];
  const int o = threadIdx.x & 63, lane4 = threadIdx.x >> 6;  // 4 position lanes x 64 channels
  float s = 0.f;
  for (int p = blockIdx.x * 4 + lane4; p < npos; p += gridDim.x * 4) s += bf2f(D[(size_t)p * NCH + o]);
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x < 64) atomicAdd(db + o, part[o] + part[o + 64] + part[o + 128] + part[o + 192]);
}

// ---------------------------------------------------------------------------
// first layer (1 -> 64) and its weight gradient, last layer (64 -> 1) with the
// loss, and its backward: CUDA cores
// ---------------------------------------------------------------------------
__global__ void k_layer1_fwd(const float* __restrict__ x, const float* __restrict__ th,
                             float* __restrict__ Z, bf16_t* __restrict__ H, int npos, int nT) {
  const size_t n = (size_t)npos * NCH;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n;
       idx += (size_t)gridDim.x * blockDim.x) {
    const int pos = (int)(idx / NCH), o = (int)(idx - (size_t)pos * NCH);
    const int t = pos % nT;
    float z = th[OFF_B1 + o];
#pragma unroll
    for (int j = 0; j < KT5; ++j) {
      const int tt = t + j - 2;
      if (tt >= 0 && tt < nT) z = fmaf(th[OFF_W1 + o * KT5 + j], x[pos + j - 2], z);
    }
    if (Z) Z[idx] = z;
    H[idx] = f2bf(gelu_f(z));
  }
}

// y = b4 + sum_{j,i} W4[i][j] h3[pos + j - 2][i]; with a target: the masked
// squared error goes to loss_acc[0] (sum) and dy = 2 (y - target) mask / nmask
__global__ void k_layer4_fwd(const bf16_t* __restrict__ H3, const float* __restrict__ th,
                             float* __restrict__ y, const float* __restrict__ target,
                             const float* __restrict__ mask, float inv_nmask,
                             float* __restrict__ dy, double* __restrict__ loss_acc, int npos,
                             int nT) {
  __shared__ float w4[NCH * KT5];
  __shared__ double red[8];
  for (int i = threadIdx.x; i < NCH * KT5; i += blockDim.x) w4[i] = th[OFF_W4 + i];
  __syncthreads();
  double lsum = 0.0;
  for (int pos = blockIdx.x * blockDim.x + threadIdx.x; pos < npos; pos += gridDim.x * blockDim.x) {
    const int t = pos % nT;
    float v = th[OFF_B4];
#pragma unroll
    for (int j = 0; j < KT5; ++j) {
      const int tt = t + j - 2;
      if (tt < 0 || tt >= nT) continue;
      const uint4* hr = reinterpret_cast<const uint4*>(H3 + (size_t)(pos + j - 2) * NCH);
#pragma unroll
      for (int c = 0; c < NCH / 8; ++c) {
        const uint4 q = hr[c];
        const unsigned w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int i = c * 8 + e * 2;
          v = fmaf(w4[i * KT5 + j], bf2f((bf16_t)(w[e] & 0xffffu)), v);
          v = fmaf(w4[(i + 1) * KT5 + j], bf2f((bf16_t)(w[e] >> 16)), v);
        }
      }
    }
    y[pos] = v;
    if (target) {
      const float r = (v - target[pos]) * mask[pos];
      lsum += (double)r * (double)r;
      dy[pos] = 2.f * r * inv_nmask;
    }
  }
  if (target) {
    lsum = warp_sum(lsum);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = lsum;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
      atomicAdd(loss_acc, s);
    }
  }
}

// backward of the last layer: dz3[pos][i] = (sum_j W4[i][j] dy[pos - j + 2]) GELU'(z3),
// dW4[i][j] += sum_pos dy[pos] h3[pos + j - 2][i], db4 += sum dy
__global__ void k_layer4_bwd(const float* __restrict__ dy, const bf16_t* __restrict__ H3,
                             const float* __restrict__ Z3, const float* __restrict__ th,
                             bf16_t* __restrict__ DZ3, float* __restrict__ g, int npos, int nT) {
  __shared__ float gw[NCH * KT5];
  __shared__ float gb;
  for (int i = threadIdx.x; i < NCH * KT5; i += blockDim.x) gw[i] = 0.f;
  if (threadIdx.x == 0) gb = 0.f;
  __syncthreads();
  const int i = threadIdx.x & 63, pl = threadIdx.x >> 6, npl = blockDim.x >> 6;
  float accw[KT5] = {0.f, 0.f, 0.f, 0.f, 0.f};
  float accb = 0.f;
  for (int pos = blockIdx.x * npl + pl; pos < npos; pos += gridDim.x * npl) {
    const int t = pos % nT;
    float d = 0.f;
#pragma unroll
    for (int j = 0; j < KT5; ++j) {
      const int tt = t - j + 2;
      if (tt >= 0 && tt < nT) d = fmaf(th[OFF_W4 + i * KT5 + j], dy[pos - j + 2], d);
      const int ts = t + j - 2;
      if (ts >= 0 && ts < nT) accw[j] = fmaf(dy[pos], bf2f(H3[(size_t)(pos + j - 2) * NCH + i]), accw[j]);
    }
    const size_t idx = (size_t)pos * NCH + i;
    DZ3[idx] = f2bf(d * gelu_grad_f(Z3[idx]));
    if (i == 0) accb += dy[pos];
  }
#pragma unroll
  for (int j = 0; j < KT5; ++j) atomicAdd(&gw[i * KT5 + j], accw[j]);
  if (i == 0) atomicAdd(&gb, accb);
  __syncthreads();
  for (int k = threadIdx.x; k < NCH * KT5; k += blockDim.x) atomicAdd(g + OFF_W4 + k, gw[k]);
  if (threadIdx.x == 0) atomicAdd(g + OFF_B4, gb);
}

// first-layer weight gradient: dW1[o][j] += sum_pos dz1[pos][o] x[pos + j - 2]; db1[o]
__global__ void k_layer1_bwd(const bf16_t* __restrict__ DZ1, const float* __restrict__ x,
                             float* __restrict__ g, int npos, int nT) {
  const int o = threadIdx.x & 63, pl = threadIdx.x >> 6, npl = blockDim.x >> 6;
  float accw[KT5] = {0.f, 0.f, 0.f, 0.f, 0.f};
  float accb = 0.f;
  for (int pos = blockIdx.x * npl + pl; pos < npos; pos += gridDim.x * npl) {
    const int t = pos % nT;
    const float d = bf2f(DZ1[(size_t)pos * NCH + o]);
    accb += d;
#pragma unroll
    for (int j = 0; j < KT5; ++j) {
      const int tt = t + j - 2;
      if (tt >= 0 && tt < nT) accw[j] = fmaf(d, x[pos + j - 2], accw[j]);
    }
  }
#pragma unroll
  for (int j = 0; j < KT5; ++j) atomicAdd(g + OFF_W1 + o * KT5 + j, accw[j]);
  atomicAdd(g + OFF_B1 + o, accb);
}

// theta -> BF16 GEMM operands: Wg[o][j*64+i] = W[o][i][j],
// WgT[i][j*64+o] = W[o][i][4-j] (the transposed convolution as a forward one)
__global__ void k_pack(const float* __restrict__ th, bf16_t* __restrict__ Wg2,
                       bf16_t* __restrict__ Wt2, bf16_t* __restrict__ Wg3,
                       bf16_t* __restrict__ Wt3, bf16_t* __restrict__ Wg4,
                       bf16_t* __restrict__ Wc2, bf16_t* __restrict__ Wc3) {
  // tcgen05 operands: [tap j][chunk kc][row o][8 channels i]: W[o][kc*8 + e][j]
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < KT5 * NCH * NCH;
       idx += gridDim.x * blockDim.x) {
    const int e = idx & 7, o = (idx >> 3) & 63, jk = idx >> 9;
    const int j = jk >> 3, i = (jk & 7) * 8 + e;
    Wc2[idx] = f2bf(th[OFF_W2 + o * KDIM + i * KT5 + j]);
    Wc3[idx] = f2bf(th[OFF_W3 + o * KDIM + i * KT5 + j]);
  }
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < 16 * KDIM;
       idx += gridDim.x * blockDim.x) {
    // Wg4[0][j*64 + i] = hi(W4[i][j]), Wg4[1][...] = lo, other rows zero
    const int r = idx / KDIM, k = idx - r * KDIM;
    const int j = k / NCH, c = k - j * NCH;
    const float w = th[OFF_W4 + c * KT5 + j];
    const bf16_t hi = f2bf(w);
    Wg4[idx] = r == 0 ? hi : r == 1 ? f2bf(w - bf2f(hi)) : (bf16_t)0;
  }
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < NCH * KDIM;
       idx += gridDim.x * blockDim.x) {
    const int r = idx / KDIM, k = idx - r * KDIM;
    const int j = k / NCH, c = k - j * NCH;
    // Wg[r = o][k = j*64 + c = i]
    Wg2[idx] = f2bf(th[OFF_W2 + r * KDIM + c * KT5 + j]);
    Wg3[idx] = f2bf(th[OFF_W3 + r * KDIM + c * KT5 + j]);
    // Wt[r = i][k = j*64 + c = o] = W[o][i][4 - j]
    Wt2[idx] = f2bf(th[OFF_W2 + c * KDIM + r * KT5 + (KT5 - 1 - j)]);
    Wt3[idx] = f2bf(th[OFF_W3 + c * KDIM + r * KT5 + (KT5 - 1 - j)]);
  }
}

// Adam (FP32 master weights)
__global__ void k_adam(float* __restrict__ th, float* __restrict__ m, float* __restrict__ v,
                       const float* __restrict__ g, int n, float lr, float b1, float b2,
                       float c1, float c2, float eps) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    th[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// net object
// ---------------------------------------------------------------------------
struct asg_net {
  float *theta = nullptr, *adam_m = nullptr, *adam_v = nullptr, *grad = nullptr;
  bf16_t *wg2 = nullptr, *wt2 = nullptr, *wg3 = nullptr, *wt3 = nullptr, *wg4 = nullptr;
  bf16_t *wc2 = nullptr, *wc3 = nullptr;  // tcgen05 layouts of W2, W3
  int* tc_err = nullptr;                  // set by a tensor-core kernel whose wait timed out
  double* loss = nullptr;
  int adam_t = 0;
  float gamma = 1.f;  // output scale of the learned step (see GateParams)
  // activations of the largest batch seen
  size_t cap = 0;
  // inference of the learned step: input rows of every learned column, the
  // column list, and activations for one chunk of rows at a time
  size_t inf_cols = 0, inf_pos = 0;
  float *inf_x = nullptr, *inf_s = nullptr, *inf_y = nullptr;
  int* inf_col = nullptr;
  bf16_t *inf_a = nullptr, *inf_b = nullptr;
  float *z1 = nullptr, *z2 = nullptr, *z3 = nullptr, *dy = nullptr, *yb = nullptr;
  bf16_t *h1 = nullptr, *h2 = nullptr, *h3 = nullptr, *d1 = nullptr, *d2 = nullptr;
  int nsm = 152;
};

static int net_fail(int code, const char* msg) { return asg_fail_message(code, msg); }

static void net_free_acts(asg_net* n) {
  void* ps[] = {n->z1, n->z2, n->z3, n->dy, n->yb, n->h1, n->h2, n->h3, n->d1, n->d2};
  for (void* p : ps) cudaFree(p);
  n->z1 = n->z2 = n->z3 = n->dy = n->yb = nullptr;
  n->h1 = n->h2 = n->h3 = n->d1 = n->d2 = nullptr;
  n->cap = 0;
}

static void net_free_inf(asg_net* n) {
  void* ps[] = {n->inf_x, n->inf_s, n->inf_y, n->inf_col, n->inf_a, n->inf_b};
  for (void* p : ps) cudaFree(p);
  n->inf_x = n->inf_s = n->inf_y = nullptr;
  n->inf_col = nullptr;
  n->inf_a = n->inf_b = nullptr;
  n->inf_cols = n->inf_pos = 0;
}

// positions of one inference chunk: two BF16 activation buffers of 1 GiB
constexpr size_t INF_CHUNK_POS = (size_t)1 << 23;

static int net_ensure_inf(asg_net* n, size_t ncols, int nT) {
  const size_t npos = ncols * (size_t)nT;
  if (n->inf_cols >= ncols && n->inf_pos >= npos) return ASG_OK;
  net_free_inf(n);
  const size_t chunk = npos < INF_CHUNK_POS ? npos : INF_CHUNK_POS;
  bool ok = cudaMalloc(&n->inf_x, npos * 4) == cudaSuccess &&
            cudaMalloc(&n->inf_s, ncols * 4) == cudaSuccess &&
            cudaMalloc(&n->inf_col, (ncols + 4) * 4) == cudaSuccess &&
            cudaMalloc(&n->inf_y, chunk * 4) == cudaSuccess &&
            cudaMalloc(&n->inf_a, chunk * NCH * 2) == cudaSuccess &&
            cudaMalloc(&n->inf_b, chunk * NCH * 2) == cudaSuccess;
  if (!ok) {
    net_free_inf(n);
    return net_fail(ASG_ERR_NOMEM, "learned step scratch: cudaMalloc failed");
  }
  n->inf_cols = ncols;
  n->inf_pos = npos;
  return ASG_OK;
}

static int net_ensure(asg_net* n, size_t npos) {
  if (n->cap >= npos) return ASG_OK;
  net_free_acts(n);
  const size_t a = npos * NCH;
  bool ok = cudaMalloc(&n->z1, a * 4) == cudaSuccess && cudaMalloc(&n->z2, a * 4) == cudaSuccess &&
            cudaMalloc(&n->z3, a * 4) == cudaSuccess && cudaMalloc(&n->dy, npos * 4) == cudaSuccess &&
            cudaMalloc(&n->yb, npos * 4) == cudaSuccess &&
            cudaMalloc(&n->h1, a * 2) == cudaSuccess && cudaMalloc(&n->h2, a * 2) == cudaSuccess &&
            cudaMalloc(&n->h3, a * 2) == cudaSuccess && cudaMalloc(&n->d1, a * 2) == cudaSuccess &&
            cudaMalloc(&n->d2, a * 2) == cudaSuccess;
  if (!ok) {
    net_free_acts(n);
    return net_fail(ASG_ERR_NOMEM, "corrector activations: cudaMalloc failed");
  }
  n->cap = npos;
  return ASG_OK;
}

static int net_pack(asg_net* n, cudaStream_t st) {
  k_pack<<<80, 256, 0, st>>>(n->theta, n->wg2, n->wt2, n->wg3, n->wt3, n->wg4, n->wc2, n->wc3);
  return cudaPeekAtLastError() == cudaSuccess ? ASG_OK : net_fail(ASG_ERR_CUDA, "pack launch");
}

static int conv_smem_attr() {
  static bool done[ASG_MAX_DEVICES] = {};
  const int dev = asg_device_slot();
  if (done[dev]) return ASG_OK;
  if (cudaFuncSetAttribute(k_conv64_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM) != cudaSuccess ||
      cudaFuncSetAttribute(k_conv64_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM) != cudaSuccess ||
      cudaFuncSetAttribute(k_conv64<0, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CONV_SMEM) != cudaSuccess ||
      cudaFuncSetAttribute(k_conv_out, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)OUT_SMEM) != cudaSuccess ||
      cudaFuncSetAttribute(k_conv64<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CONV_SMEM) != cudaSuccess ||
      cudaFuncSetAttribute(k_conv64<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CONV_SMEM) != cudaSuccess ||
      cudaFuncSetAttribute(k_conv64_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)WGRAD_SMEM) != cudaSuccess)
    return net_fail(ASG_ERR_CUDA, "corrector kernels: shared-memory attribute");
  done[dev] = true;
  return ASG_OK;
}

// forward of the whole network: x [npos] -> y [npos] (z's kept when keep_z)
static int net_forward(asg_net* n, const float* x, float* y, const float* target,
                       const float* mask, float inv_nmask, int npos, int nT, bool keep_z,
                       cudaStream_t st) {
  CKS_NET(conv_smem_attr());
  const int tiles = npos / TPC;
  const int gconv = tiles < 2 * n->nsm ? tiles : 2 * n->nsm;
  k_layer1_fwd<<<4 * n->nsm, 256, 0, st>>>(x, n->theta, keep_z ? n->z1 : nullptr, n->h1, npos, nT);
  k_conv64<0><<<gconv, 128, CONV_SMEM, st>>>(n->h1, n->wg2, n->theta + OFF_B2, nullptr,
                                             keep_z ? n->z2 : nullptr, n->h2, npos, nT);
  k_conv64<0><<<gconv, 128, CONV_SMEM, st>>>(n->h2, n->wg3, n->theta + OFF_B3, nullptr,
                                             keep_z ? n->z3 : nullptr, n->h3, npos, nT);
  k_layer4_fwd<<<4 * n->nsm, 256, 0, st>>>(n->h3, n->theta, y, target, mask, inv_nmask, n->dy,
                                           n->loss, npos, nT);
  return cudaPeekAtLastError() == cudaSuccess ? ASG_OK : net_fail(ASG_ERR_CUDA, "forward launch");
}

static int net_backward(asg_net* n, const float* x, int npos, int nT, cudaStream_t st) {
  const int tiles = npos / TPC;
  const int gconv = tiles < 2 * n->nsm ? tiles : 2 * n->nsm;
  const int chunks = npos / TP;
  const int gw = chunks < n->nsm ? chunks : n->nsm;
  // last layer: dW4, db4, dz3 -> d2
  k_layer4_bwd<<<2 * n->nsm, 256, 0, st>>>(n->dy, n->h3, n->z3, n->theta, n->d2, n->grad, npos, nT);
  // layer 3: dW3 (dz3, h2), db3, dz2 = (W3^T * dz3) GELU'(z2) -> d1
  k_conv64_wgrad<<<dim3(gw, KDIM / WG_SLAB), 128, WGRAD_SMEM, st>>>(n->d2, n->h2, n->grad + OFF_W3, npos, nT);
  k_bias_grad<<<2 * n->nsm, 256, 0, st>>>(n->d2, n->grad + OFF_B3, npos);
  k_conv64<1><<<gconv, 128, CONV_SMEM, st>>>(n->d2, n->wt3, nullptr, n->z2, nullptr, n->d1, npos, nT);
  // layer 2: dW2 (dz2, h1), db2, dz1 = (W2^T * dz2) GELU'(z1) -> d2
  k_conv64_wgrad<<<dim3(gw, KDIM / WG_SLAB), 128, WGRAD_SMEM, st>>>(n->d1, n->h1, n->grad + OFF_W2, npos, nT);
  k_bias_grad<<<2 * n->nsm, 256, 0, st>>>(n->d1, n->grad + OFF_B2, npos);
  k_conv64<1><<<gconv, 128, CONV_SMEM, st>>>(n->d1, n->wt2, nullptr, n->z1, nullptr, n->d2, npos, nT);
  // layer 1
  k_layer1_bwd<<<2 * n->nsm, 256, 0, st>>>(n->d2, x, n->grad, npos, nT);
  return cudaPeekAtLastError() == cudaSuccess ? ASG_OK : net_fail(ASG_ERR_CUDA, "backward launch");
}

// a tensor-core kernel gave up waiting for its accumulator (reported once)
static int net_check_tc(asg_net* n) {
  int e = 0;
  if (cudaMemcpy(&e, n->tc_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
    return net_fail(ASG_ERR_CUDA, "status download");
  if (e == 0) return ASG_OK;
  cudaMemset(n->tc_err, 0, sizeof(int));
  return net_fail(ASG_ERR_TIMEOUT, "tensor-core accumulator wait timed out");
}

// inference: x [npos] -> y [npos] with two BF16 activation buffers
static int net_infer(asg_net* n, const float* x, float* y, int npos, int nT, bf16_t* a,
                     bf16_t* b, cudaStream_t st) {
  CKS_NET(conv_smem_attr());
  const int tiles = npos / TPC;
  const int gconv = tiles < 3 * n->nsm ? tiles : 3 * n->nsm;
  // layers 1 + 2 (x -> h2), layer 3 (h2 -> h3), layer 4 (h3 -> y)
  const int gtc = (tiles + 1) / 2 < 3 * n->nsm ? (tiles + 1) / 2 : 3 * n->nsm;
  k_conv64_tc<true><<<gtc, 256, TC_SMEM, st>>>(x, n->wc2, n->theta + OFF_B2, a, npos, nT,
                                               n->theta, n->tc_err);
  k_conv64_tc<false><<<gtc, 256, TC_SMEM, st>>>(a, n->wc3, n->theta + OFF_B3, b, npos, nT,
                                                n->theta, n->tc_err);
  const int gout = tiles < 6 * n->nsm ? tiles : 6 * n->nsm;
  k_conv_out<<<gout, 128, OUT_SMEM, st>>>(b, n->wg4, n->theta, y, npos, nT);
  return cudaPeekAtLastError() == cudaSuccess ? ASG_OK : net_fail(ASG_ERR_CUDA, "inference launch");
}

extern "C" int asg_net_param_count(void) { return NPARAM; }

extern "C" int asg_net_create(asg_net** out) {
  if (!out) return net_fail(ASG_ERR_ARG, "null argument");
  asg_net* n = new asg_net();
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n->nsm, cudaDevAttrMultiProcessorCount, dev);
  bool ok = cudaMalloc(&n->theta, NPARAM * 4) == cudaSuccess &&
            cudaMalloc(&n->adam_m, NPARAM * 4) == cudaSuccess &&
            cudaMalloc(&n->adam_v, NPARAM * 4) == cudaSuccess &&
            cudaMalloc(&n->grad, NPARAM * 4) == cudaSuccess &&
            cudaMalloc(&n->wg2, NCH * KDIM * 2) == cudaSuccess &&
            cudaMalloc(&n->wt2, NCH * KDIM * 2) == cudaSuccess &&
            cudaMalloc(&n->wg3, NCH * KDIM * 2) == cudaSuccess &&
            cudaMalloc(&n->wt3, NCH * KDIM * 2) == cudaSuccess &&
            cudaMalloc(&n->wg4, 16 * KDIM * 2) == cudaSuccess &&
            cudaMalloc(&n->wc2, NCH * KDIM * 2) == cudaSuccess &&
            cudaMalloc(&n->wc3, NCH * KDIM * 2) == cudaSuccess &&
            cudaMalloc(&n->tc_err, sizeof(int)) == cudaSuccess &&
            cudaMalloc(&n->loss, sizeof(double)) == cudaSuccess;
  if (!ok) {
    asg_net_destroy(n);
    return net_fail(ASG_ERR_NOMEM, "corrector parameters: cudaMalloc failed");
  }
  cudaMemset(n->theta, 0, NPARAM * 4);
  cudaMemset(n->tc_err, 0, sizeof(int));
  cudaMemset(n->adam_m, 0, NPARAM * 4);
  cudaMemset(n->adam_v, 0, NPARAM * 4);
  *out = n;
  return net_pack(n, 0) == ASG_OK && cudaDeviceSynchronize() == cudaSuccess
             ? ASG_OK : net_fail(ASG_ERR_CUDA, "corrector set-up");
}

extern "C" int asg_net_destroy(asg_net* n) {
  if (!n) return ASG_OK;
  net_free_acts(n);
  net_free_inf(n);
  void* ps[] = {n->theta, n->adam_m, n->adam_v, n->grad, n->wg2, n->wt2, n->wg3, n->wt3, n->wg4,
                n->wc2, n->wc3, n->tc_err, n->loss};
  for (void* p : ps) cudaFree(p);
  delete n;
  return ASG_OK;
}

extern "C" int asg_net_set_params(asg_net* n, const float* theta, int count) {
  if (!n || !theta || count != NPARAM) return net_fail(ASG_ERR_ARG, "bad parameter vector");
  if (cudaMemcpy(n->theta, theta, NPARAM * 4, cudaMemcpyHostToDevice) != cudaSuccess)
    return net_fail(ASG_ERR_CUDA, "parameter upload");
  cudaMemset(n->adam_m, 0, NPARAM * 4);
  cudaMemset(n->adam_v, 0, NPARAM * 4);
  n->adam_t = 0;
  CKS_NET(net_pack(n, 0));
  return cudaDeviceSynchronize() == cudaSuccess ? ASG_OK : net_fail(ASG_ERR_CUDA, "pack");
}

extern "C" int asg_net_get_params(asg_net* n, float* theta, int count) {
  if (!n || !theta || count != NPARAM) return net_fail(ASG_ERR_ARG, "bad parameter vector");
  return cudaMemcpy(theta, n->theta, NPARAM * 4, cudaMemcpyDeviceToHost) == cudaSuccess
             ? ASG_OK : net_fail(ASG_ERR_CUDA, "parameter download");
}

static int check_batch(int ncols, int nT) {
  if (ncols <= 0 || nT < TPC || nT % TPC != 0)
    return net_fail(ASG_ERR_SHAPE, "corrector batches need nT a multiple of 128");
  return ASG_OK;
}

extern "C" int asg_net_forward(asg_net* n, const float* d_x, float* d_y, int ncols, int nT,
                               void* stream) {
  if (!n || !d_x || !d_y) return net_fail(ASG_ERR_ARG, "null argument");
  CKS_NET(check_batch(ncols, nT));
  CKS_NET(net_ensure_inf(n, (size_t)ncols, nT));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int rows_per_chunk = (int)(INF_CHUNK_POS / (size_t)nT);
  for (int r0 = 0; r0 < ncols; r0 += rows_per_chunk) {
    const int rows = ncols - r0 < rows_per_chunk ? ncols - r0 : rows_per_chunk;
    CKS_NET(net_infer(n, d_x + (size_t)r0 * nT, d_y + (size_t)r0 * nT, rows * nT, nT, n->inf_a,
                      n->inf_b, st));
  }
  return ASG_OK;
}

// One training step on a device batch: loss (masked MSE) and gradients; with
// lr > 0 an Adam update follows.  h_grad (host, NPARAM floats) receives the
// gradients when not null.
extern "C" int asg_net_train_step(asg_net* n, const float* d_x, const float* d_target,
                                  const float* d_mask, int ncols, int nT, float lr,
                                  double* loss_out, float* h_grad) {
  if (!n || !d_x || !d_target || !d_mask) return net_fail(ASG_ERR_ARG, "null argument");
  CKS_NET(check_batch(ncols, nT));
  const size_t npos = (size_t)ncols * nT;
  CKS_NET(net_ensure(n, npos));
  cudaStream_t st = 0;
  // the loss is a mean over the masked samples: their count, on the host
  std::vector<float> hm(npos);
  if (cudaMemcpy(hm.data(), d_mask, npos * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
    return net_fail(ASG_ERR_CUDA, "mask download");
  double ms = 0.0;
  for (float v : hm) ms += v;
  const float nmask = (float)(ms > 0.0 ? ms : 1.0);
  cudaMemsetAsync(n->grad, 0, NPARAM * 4, st);
  cudaMemsetAsync(n->loss, 0, sizeof(double), st);
  CKS_NET(net_forward(n, d_x, n->yb, d_target, d_mask, 1.f / nmask, (int)npos, nT, true, st));
  CKS_NET(net_backward(n, d_x, (int)npos, nT, st));
  double l = 0.0;
  if (cudaMemcpy(&l, n->loss, sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
    return net_fail(ASG_ERR_CUDA, "loss download");
  if (loss_out) *loss_out = l / nmask;
  if (h_grad && cudaMemcpy(h_grad, n->grad, NPARAM * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
    return net_fail(ASG_ERR_CUDA, "gradient download");
  if (lr > 0.f) {
    n->adam_t++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f / (1.f - powf(b1, (float)n->adam_t));
    const float c2 = 1.f / (1.f - powf(b2, (float)n->adam_t));
    k_adam<<<(NPARAM + 255) / 256, 256, 0, st>>>(n->theta, n->adam_m, n->adam_v, n->grad, NPARAM,
                                                  lr, b1, b2, c1, c2, 1e-8f);
    CKS_NET(net_pack(n, st));
  }
  return cudaDeviceSynchronize() == cudaSuccess ? ASG_OK : net_fail(ASG_ERR_CUDA, "train step");
}

// ---------------------------------------------------------------------------
// Learned KT step on columns.
//
// Gate (one warp per column, the column in a skewed shared-memory copy):
//   s      = max|u|,  steep = max_t |u[t+1] - u[t]|
//   n_sub  = the per-column sub-cycle count of the plain KT step at cfl_target
//   learned when n_sub >= min_sub and steep <= shock_ratio * s: one coarse KT
//     step of the full dz, written to out and, in CFL units, to the network's
//     input rows (compacted, in the order the columns claim them);
//   otherwise the plain sub-cycled KT step (the fallback) is written to out.
// Apply: out[c][t] += s gamma cfl^3 y[k][t] for the learned columns,
// t = 1 .. nT-2 (the KT step never changes the end samples).
// ---------------------------------------------------------------------------
namespace {

struct GateParams {
  const float* in;
  float* out;
  int ncols, nT;
  float ndt, dz, cfl_target;
  int max_sub, min_sub, mc;
  float shock_ratio;
  // The network sees the coarse column in CFL units (w = u ndt dz, divided by
  // CFL_IN), so that the column's CFL number is visible to it, and predicts
  // the correction in units of s gamma cfl^3 (cfl = ndt s dz): the difference
  // between one SSP-RK2 KT step and the sub-cycled step is third order in the
  // column's CFL number, so these targets are of order one at every peak.
  float gamma;
  float in_scale;     // ndt dz / CFL_IN
  float* xrows;       // [ncols][nT] compacted network input
  int* list_col;      // [ncols]
  float* list_s;      // [ncols] output scale of each learned column
  int* counter;       // learned columns so far (starts at zero)
  unsigned* clamp;    // [2] fallback columns capped at max_sub, largest count needed
};

template <int CH>
__global__ void __launch_bounds__(256) k_flux_gate(GateParams p) {
  extern __shared__ float sk_raw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = blockIdx.x * 8 + warp;
  if (c >= p.ncols) return;
  const int nT = p.nT;
  const unsigned mask = 0xffffffffu;
  SkewColumn col{sk_raw + warp * skew_floats(32 * CH)};
  const float* src = p.in + (size_t)c * nT;
  float s = 0.f, steep = 0.f;
  for (int t = lane; t < nT; t += 32) {
    const float u = src[t];
    col.set(t, u);
    s = fmaxf(s, fabsf(u));
    if (t + 1 < nT) steep = fmaxf(steep, fabsf(src[t + 1] - u));
  }
  s = warp_max(s);
  steep = warp_max(steep);
  __syncwarp(mask);
  int nsub = 1;
  if (p.cfl_target > 0.f) {
    const float cfl = p.ndt * s * p.dz;
    if (!(cfl <= p.cfl_target || s < 1e-30f)) {
      const float q = ceilf(cfl / p.cfl_target);
      nsub = (q > (float)p.max_sub) ? p.max_sub : (int)q;
    }
  }
  // the coarse SSP-RK2 KT step is only a meaningful start below CFL 0.5 (its
  // stability bound); columns above take the plain sub-cycled step
  const bool learned = nsub >= p.min_sub && steep <= p.shock_ratio * s && s > 1e-30f &&
                       p.ndt * s * p.dz <= 0.5f;
  if (!learned && lane == 0 && p.cfl_target > 0.f) {
    // a fallback column capped at max_sub sub-cycles runs above its CFL target
    const float q = ceilf(p.ndt * s * p.dz / p.cfl_target);
    if (q > (float)p.max_sub) {
      atomicAdd(p.clamp, 1u);
      atomicMax(p.clamp + 1, q < 4.0e9f ? (unsigned)q : 0xffffffffu);
    }
  }
  const int steps = learned ? 1 : nsub;
  const float dzs = p.dz / (float)steps;
  for (int k = 0; k < steps; ++k) {
    if (p.mc) kt_column_step_chunk<CH, true>(col, nT, p.ndt, dzs, mask);
    else kt_column_step_chunk<CH, false>(col, nT, p.ndt, dzs, mask);
  }
  float* dst = p.out + (size_t)c * nT;
  for (int t = lane; t < nT; t += 32) dst[t] = col.get(t);
  if (learned) {
    int k = 0;
    if (lane == 0) {
      k = atomicAdd(p.counter, 1);
      const float cfl = p.ndt * s * p.dz;
      p.list_col[k] = c;
      p.list_s[k] = s * p.gamma * cfl * cfl * cfl;
    }
    k = __shfl_sync(mask, k, 0);
    float* xr = p.xrows + (size_t)k * nT;
    for (int t = lane; t < nT; t += 32) xr[t] = col.get(t) * p.in_scale;
  }
}

// rows row0 .. row0 + gridDim.x - 1 of the learned list; y holds their outputs
__global__ void k_apply_correction(const float* __restrict__ y, const int* __restrict__ list_col,
                                   const float* __restrict__ list_s, int row0,
                                   float* __restrict__ out, int nT) {
  const int k = row0 + blockIdx.x;
  const int c = list_col[k];
  const float s = list_s[k];
  const float* yr = y + (size_t)blockIdx.x * nT;
  for (int t = threadIdx.x; t < nT; t += blockDim.x)
    if (t >= 1 && t < nT - 1) out[(size_t)c * nT + t] += s * yr[t];
}

template <int CH>
int launch_gate(const GateParams& p, cudaStream_t st) {
  const size_t smem = (size_t)8 * skew_floats(32 * CH) * sizeof(float);
  k_flux_gate<CH><<<(p.ncols + 7) / 8, 256, smem, st>>>(p);
  return cudaPeekAtLastError() == cudaSuccess ? ASG_OK : ASG_ERR_CUDA;
}

}  // namespace

// Scale of the network's output in the learned step (see GateParams::gamma).
extern "C" int asg_net_set_output_scale(asg_net* n, float gamma) {
  if (!n || !(gamma > 0.f)) return net_fail(ASG_ERR_ARG, "bad output scale");
  n->gamma = gamma;
  return ASG_OK;
}

// Learned KT step on device columns (see the gate above).  n_coef = N (the
// nonlinearity coefficient); the network input rows, the column list and the
// activations of one chunk of rows are the net's own scratch (grown as
// needed, activations bounded by the chunk).  Synchronous:
// *n_learned receives the number of columns that took the learned path.
extern "C" int asg_flux_columns_learned(asg_net* n, const float* d_in, float* d_out, int ncols,
                                        int nT, int flux, double n_coef, double dz, double dt,
                                        double cfl_target, int max_subcycles, int min_subcycles,
                                        float shock_ratio, int* n_learned, void* stream) {
  if (!n || !d_in || !d_out || d_in == d_out) return net_fail(ASG_ERR_ARG, "bad argument");
  if (flux != ASG_FLUX_KT && flux != ASG_FLUX_KT_MINMOD)
    return net_fail(ASG_ERR_ARG, "the learned step corrects the KT schemes only");
  CKS_NET(check_batch(ncols, nT));
  if (nT > 1024) return net_fail(ASG_ERR_SHAPE, "learned step: columns up to 1024 samples");
  CKS_NET(net_ensure_inf(n, (size_t)ncols, nT));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  float* xrows = n->inf_x;
  int* list_col = n->inf_col;
  float* list_s = n->inf_s;
  int* counter = n->inf_col + ncols;  // then the two sub-cycle cap counters
  if (cudaMemsetAsync(counter, 0, 3 * sizeof(int), st) != cudaSuccess)
    return net_fail(ASG_ERR_CUDA, "counter reset");
  GateParams g;
  g.in = d_in;
  g.out = d_out;
  g.ncols = ncols;
  g.nT = nT;
  g.ndt = (float)(n_coef / dt);
  g.dz = (float)dz;
  g.cfl_target = (float)cfl_target;
  g.max_sub = max_subcycles > 0 ? max_subcycles : 1024;
  g.min_sub = min_subcycles;
  g.mc = flux == ASG_FLUX_KT;
  g.shock_ratio = shock_ratio;
  g.gamma = n->gamma;
  g.in_scale = (float)(n_coef / dt * dz / 0.3);  // CFL_IN = 0.3
  g.xrows = xrows;
  g.list_col = list_col;
  g.list_s = list_s;
  g.counter = counter;
  g.clamp = reinterpret_cast<unsigned*>(counter + 1);
  const int ch = (nT + 31) / 32;
  const int s = ch <= 2 ? launch_gate<2>(g, st) : ch <= 4 ? launch_gate<4>(g, st)
              : ch <= 8 ? launch_gate<8>(g, st) : ch <= 16 ? launch_gate<16>(g, st)
              : launch_gate<32>(g, st);
  if (s != ASG_OK) return net_fail(s, "gate launch");
  int cnt[3] = {0, 0, 0};
  if (cudaMemcpyAsync(cnt, counter, sizeof(cnt), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return net_fail(ASG_ERR_CUDA, "learned-column count");
  const int k = cnt[0];
  if (n_learned) *n_learned = k;
  const int rows_per_chunk = (int)(INF_CHUNK_POS / (size_t)nT);
  for (int r0 = 0; r0 < k; r0 += rows_per_chunk) {
    const int rows = k - r0 < rows_per_chunk ? k - r0 : rows_per_chunk;
    CKS_NET(net_infer(n, xrows + (size_t)r0 * nT, n->inf_y, rows * nT, nT, n->inf_a, n->inf_b, st));
    k_apply_correction<<<rows, 256, 0, st>>>(n->inf_y, list_col, list_s, r0, d_out, nT);
    if (cudaPeekAtLastError() != cudaSuccess) return net_fail(ASG_ERR_CUDA, "apply launch");
  }
  if (cudaStreamSynchronize(st) != cudaSuccess) return net_fail(ASG_ERR_CUDA, "learned step");
  CKS_NET(net_check_tc(n));
  if (cnt[1] != 0) {
    char msg[200];
    snprintf(msg, sizeof msg,
             "%u fallback columns needed more KT sub-cycles than the cap of %d (up to %u) and "
             "ran above the CFL target", (unsigned)cnt[1], g.max_sub, (unsigned)cnt[2]);
    return net_fail(ASG_ERR_SUBCYCLES, msg);
  }
  return ASG_OK;
}
