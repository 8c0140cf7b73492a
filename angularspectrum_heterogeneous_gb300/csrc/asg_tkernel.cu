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
// fast kernel: nT = 2M, M = N1*N2 (register-resident four-step FFT).
// A block of 8 warps handles C columns (C = 8 or 16): CY = C/2 consecutive y
// at row x and the same CY y at row x+X/2.  That pairing lets the kernel
// apply the first radix-2 stage of the x transform on the way out
// (split_out: planes hold a = (s(x) + s(x+X/2))/2 and
// b = (s(x) - s(x+X/2)) W_X^x/2 in rows x and x+X/2) and undo it on the way in
// (split_in: s = a +/- W_X^-x b), so the plane kernels work on X/2-row
// half-planes (their transforms are normalised by the half-plane size).
// Warp w owns columns w, w+8, ... (CPW = C/8 of them); with C = 16 the N1
// tasks of step B of two columns fill the 32 lanes of a warp, and each
// frequency plane is read and written in 64-byte runs.  MODE selects the
// column work at compile time.
// ---------------------------------------------------------------------------
enum TMode : int { TM_PLAIN = 0, TM_FLUX = 1, TM_STATS = 2 };

// Register budget: 3 blocks per SM with 16 columns or from 512 samples up
// (shared memory allows no more) and 4 otherwise, in every mode (the streamed
// KT step keeps about 25 values live).
template <class PL, int MODE, int C>
__global__ void __launch_bounds__(256, ((PL::N >= 512 || C == 16) ? 3 : 4))
    tk_fast(TParams p) {
  if (*p.status != 0) return;
  static_assert(C == 8 || C == 16, "8 or 16 columns per block");
  constexpr int CPW = C / 8;   // columns per warp
  constexpr int CY = C / 2;    // consecutive y per row
  constexpr int M = PL::N;
  constexpr int N1 = PL::N1;
  constexpr int N2 = PL::N2;
  constexpr int CH = (2 * M + 31) / 32;
  // column stride: padded line + 2, so the columns of a tile fall in
  // different shared-memory banks in the pair (k, M-k) phases
  constexpr int LS = PL::PADDED + 2;
  const int nT = 2 * M;
  // flux mode: the KT sub-steps stream along each column in place (every
  // fast length is a multiple of 32 samples), so no shared memory beyond the
  // lines is needed
  extern __shared__ float4 smraw[];
  float2* lines = reinterpret_cast<float2*>(smraw);
  float2* twM = lines + C * LS;
  const float2* __restrict__ twT = p.tw;                // W_2M^k, k <= M (L1-cached)
  __shared__ float red_max[8];

  const int tid = threadIdx.x, nthr = blockDim.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int Y = p.Y, X2 = p.X / 2;
  const int ncols = p.ncols;
  // tile -> (x, y0); column cc: row x + (cc >= CY)*X/2, y = y0 + cc % CY
  const int tile = blockIdx.x;
  const int xq = tile / (Y / CY), y0 = CY * (tile - xq * (Y / CY));
  if (p.prefetch_ahead > 0 && !p.in_real) {
    // blocks start in about index order: the tile of block b + (resident
    // blocks) starts about when this one ends, so its spectrum goes to L2 now
    const int nt = blockIdx.x + p.prefetch_ahead;
    if (nt < (int)gridDim.x) {
      const int xq2 = nt / (Y / CY), y02 = CY * (nt - xq2 * (Y / CY));
      const size_t cA = (size_t)xq2 * Y + y02, cB = cA + (size_t)X2 * Y;
      // M + 1 planes, rows x and x + X/2: runs of CY complex (32 or 64 bytes)
      for (int i = tid; i < 2 * (M + 1); i += nthr) {
        const float2* a = p.spec + (size_t)(i >> 1) * ncols + ((i & 1) ? cB : cA);
        asm volatile("prefetch.global.L2 [%0];" ::"l"(a));
        if (CY == 8) asm volatile("prefetch.global.L2 [%0];" ::"l"(a + 4));
      }
    }
  }
  for (int i = tid; i < M; i += nthr) twM[i] = p.twM[i];
  const float2 wx = p.twX[xq];  // W_X^x of this tile's column pair
  auto col_of = [&](int cc) {
    return (xq + (cc >= CY ? X2 : 0)) * Y + y0 + (cc & (CY - 1));
  };

  // ---------------- phase 1: input ----------------
  if (p.in_real) {
    __syncthreads();
#pragma unroll
    for (int j = 0; j < CPW; ++j) {
      const int cc = warp + 8 * j;
      float2* line = lines + cc * LS;
      const float2* src = reinterpret_cast<const float2*>(p.real_in + (size_t)col_of(cc) * nT);
      for (int i = lane; i < M; i += 32) line[PL::pos(i)] = src[i];
    }
    __syncwarp();
  } else {
    __syncthreads();
    const float inv2M = 0.5f / (float)M;
    const int npairs = M / 2 + 1;
    const size_t colA = (size_t)xq * Y + y0;        // row x
    const size_t colB = colA + (size_t)X2 * Y;       // row x + X/2
    // two neighbouring columns per thread: 16-byte loads of (y, y+1)
#pragma unroll 2
    for (int it = tid; it < npairs * (CY / 2); it += nthr) {
      const int u0 = 2 * (it & (CY / 2 - 1)), k = it / (CY / 2);
      const int k2 = M - k;
      const int sk = (k == 0) ? 0 : PL::slot_of_freq(k);
      const int sk2 = (k == 0) ? M : PL::slot_of_freq(k2);
      const float2* pk = p.spec + (size_t)sk * ncols + u0;
      const float2* pm = p.spec + (size_t)sk2 * ncols + u0;
      const float4 xa2 = *reinterpret_cast<const float4*>(pk + colA);
      const float4 xb2 = *reinterpret_cast<const float4*>(pk + colB);
      const float4 ma2 = *reinterpret_cast<const float4*>(pm + colA);
      const float4 mb2 = *reinterpret_cast<const float4*>(pm + colB);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
      const int u = u0 + h;
      float2 xa = h ? make_float2(xa2.z, xa2.w) : make_float2(xa2.x, xa2.y);
      float2 xb = h ? make_float2(xb2.z, xb2.w) : make_float2(xb2.x, xb2.y);
      float2 ma = h ? make_float2(ma2.z, ma2.w) : make_float2(ma2.x, ma2.y);
      float2 mb = h ? make_float2(mb2.z, mb2.w) : make_float2(mb2.x, mb2.y);
      if (p.split_in) {
        const float2 tb = cmulc(xb, wx), tm = cmulc(mb, wx);
        const float2 a0 = xa, m0 = ma;
        xa = cadd(a0, tb);
        xb = csub(a0, tb);
        ma = cadd(m0, tm);
        mb = csub(m0, tm);
      }
      float2* la = lines + u * LS;
      float2* lb = lines + (u + CY) * LS;
      if (k == 0) {
        // bins 0 and M: imaginary parts dropped (irfft)
        la[PL::pos(0)] = make_float2((xa.x + ma.x) * inv2M, (xa.x - ma.x) * inv2M);
        lb[PL::pos(0)] = make_float2((xb.x + mb.x) * inv2M, (xb.x - mb.x) * inv2M);
      } else {
        const float2 wk = __ldg(twT + k);
#pragma unroll
        for (int side = 0; side < 2; ++side) {
          const float2 xk = side ? xb : xa;
          const float2 xm = side ? mb : ma;
          float2* line = side ? lb : la;
          // E and D here are twice the even/odd parts: the halving folds into the
          // final 1/M scaling (power-of-two scalings are exact)
          const float2 E = make_float2(xk.x + xm.x, xk.y - xm.y);
          const float2 D = make_float2(xk.x - xm.x, xk.y + xm.y);
          const float2 O = cmulc(D, wk);
          // Z[k] = E + iO ; Z[M-k] = conj(E) + i conj(O)
          line[PL::pos(sk)] = make_float2((E.x - O.y) * inv2M, (E.y + O.x) * inv2M);
          line[PL::pos(sk2)] = make_float2((E.x + O.y) * inv2M, (-E.y + O.x) * inv2M);
        }
      }
      }
    }
    __syncthreads();
    // inverse four-step on my columns: B^-1 then A^-1
    for (int i = lane; i < CPW * N1; i += 32) {
      const int j = i / N1, ka = i - j * N1;
      stepB_smem<PL, true>(lines + (warp + 8 * j) * LS, ka);
    }
    __syncwarp();
    for (int i = lane; i < CPW * N2; i += 32) {
      const int j = i / N2, b = i - j * N2;
      stepA_inv_smem<PL>(lines + (warp + 8 * j) * LS, b, twM);
    }
    __syncwarp();
    if (MODE != TM_STATS && p.op.abl_xy != nullptr) {
      // boundary taper on sample pairs (slot s holds samples 2s, 2s+1)
      const float2* __restrict__ abl2 = reinterpret_cast<const float2*>(p.op.abl_t);
#pragma unroll 1
      for (int j = 0; j < CPW; ++j) {
        float2* line = lines + (warp + 8 * j) * LS;
        const float axy = __ldg(p.op.abl_xy + col_of(warp + 8 * j));
#pragma unroll 4
        for (int s = lane; s < M; s += 32) {
          const float2 v = line[PL::pos(s)], w = __ldg(abl2 + s);
          line[PL::pos(s)] = make_float2(v.x * (axy * w.x), v.y * (axy * w.y));
        }
      }
      __syncwarp();
    }
  }

  // ---------------- phase 2: column work ----------------
  float am = 0.f;
#pragma unroll 1
  for (int j = 0; j < CPW; ++j) {
    const int cc = warp + 8 * j;
    float2* line = lines + cc * LS;
    const int mycol = col_of(cc);
    PaddedColumn<N2> col{reinterpret_cast<float*>(line)};
    ColumnOps op = p.op;
    if (MODE != TM_FLUX) op.flux = FLUX_NONE;
    op.abl_xy = nullptr;  // tapered at the end of phase 1
    const float a =
        column_phase<CH, MODE == TM_FLUX>(col, col, mycol, nT, op, MODE == TM_STATS);
    am = (a != a || am != am) ? __uint_as_float(0x7fc00000u) : fmaxf(am, a);
    if (p.write_real) {
      float2* dst = reinterpret_cast<float2*>(p.real_out + (size_t)mycol * nT);
      for (int i = lane; i < M; i += 32) dst[i] = line[PL::pos(i)];
    }
  }
  if (MODE == TM_STATS) {
    if (lane == 0) red_max[warp] = am;
    __syncthreads();
    if (tid == 0) {
      float m = 0.f;
      bool bad = false;
      for (int w = 0; w < 8; ++w) {
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
  for (int i = lane; i < CPW * N2; i += 32) {
    const int j = i / N2, b = i - j * N2;
    stepA_fwd_smem<PL, false>(lines + (warp + 8 * j) * LS, b, twM);
  }
  __syncwarp();
  for (int i = lane; i < CPW * N1; i += 32) {
    const int j = i / N1, ka = i - j * N1;
    stepB_smem<PL, false>(lines + (warp + 8 * j) * LS, ka);
  }
  __syncthreads();
  {
    const int npairs = M / 2 + 1;
    const size_t colA = (size_t)xq * Y + y0;
    const size_t colB = colA + (size_t)X2 * Y;
    // two neighbouring columns per thread: 16-byte stores of (y, y+1)
#pragma unroll 2
    for (int it = tid; it < npairs * (CY / 2); it += nthr) {
      const int u0 = 2 * (it & (CY / 2 - 1)), k = it / (CY / 2);
      const int k2 = M - k;
      const int sk = (k == 0) ? 0 : PL::slot_of_freq(k);
      const int sk2 = (k == 0) ? M : PL::slot_of_freq(k2);
      const float2 wk = (k == 0) ? make_float2(1.f, 0.f) : __ldg(twT + k);
      float2 oa[2][2], ob[2][2];  // [h][bin k, bin M-k] of columns u0 + h
#pragma unroll
      for (int h = 0; h < 2; ++h) {
      const int u = u0 + h;
      float2 ra[2], rb[2];  // [0]: bin k, [1]: bin M-k, for rows x and x+X/2
#pragma unroll
      for (int side = 0; side < 2; ++side) {
        const float2* line = lines + (u + CY * side) * LS;
        // r0, r1: twice the bins k and M-k (the halvings of the even/odd parts
        // fold into the output scaling below; power-of-two scalings are exact)
        float2 r0, r1;
        if (k == 0) {
          const float2 z = line[PL::pos(0)];
          r0 = make_float2(2.f * (z.x + z.y), 0.f);
          r1 = make_float2(2.f * (z.x - z.y), 0.f);
        } else {
          const float2 zk = line[PL::pos(sk)];
          const float2 zm = line[PL::pos(sk2)];
          const float2 E = make_float2(zk.x + zm.x, zk.y - zm.y);
          const float2 D = make_float2(zk.x - zm.x, zk.y + zm.y);
          const float2 O = make_float2(D.y, -D.x);  // -i (zk - conj zm)
          const float2 WO = cmul(O, wk);
          r0 = make_float2(E.x + WO.x, E.y + WO.y);
          r1 = make_float2(E.x - WO.x, -(E.y - WO.y));
        }
        if (side == 0) { ra[0] = r0; ra[1] = r1; }
        else { rb[0] = r0; rb[1] = r1; }
      }
      if (p.split_out) {
        // a = (s(x) + s(x+X/2))/2, b = (s(x) - s(x+X/2)) W_X^x / 2: the input
        // side s = a +/- W_X^-x b then inverts it exactly
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          const float2 a = cscale(cadd(ra[j], rb[j]), 0.25f);
          const float2 b = cmul(csub(ra[j], rb[j]), make_float2(0.25f * wx.x, 0.25f * wx.y));
          ra[j] = a;
          rb[j] = b;
        }
      } else {
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          ra[j] = cscale(ra[j], 0.5f);
          rb[j] = cscale(rb[j], 0.5f);
        }
      }
      oa[h][0] = ra[0];
      oa[h][1] = ra[1];
      ob[h][0] = rb[0];
      ob[h][1] = rb[1];
      }
      float2* so = p.spec_out ? p.spec_out : p.spec;
      float2* pk = so + (size_t)sk * ncols + u0;
      float2* pm = so + (size_t)sk2 * ncols + u0;
      *reinterpret_cast<float4*>(pk + colA) = make_float4(oa[0][0].x, oa[0][0].y, oa[1][0].x, oa[1][0].y);
      *reinterpret_cast<float4*>(pk + colB) = make_float4(ob[0][0].x, ob[0][0].y, ob[1][0].x, ob[1][0].y);
      *reinterpret_cast<float4*>(pm + colA) = make_float4(oa[0][1].x, oa[0][1].y, oa[1][1].x, oa[1][1].y);
      *reinterpret_cast<float4*>(pm + colB) = make_float4(ob[0][1].x, ob[0][1].y, ob[1][1].x, ob[1][1].y);
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
  float* stg_base = reinterpret_cast<float*>(tw + nT);  // KT stage-1 values [C][nT]
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
    PlainColumn stg{stg_base + warp * nT};
    am = column_phase<CH>(col, stg, mycol, nT, p.op, p.stats != 0);
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
    if (c < ncols) (p.spec_out ? p.spec_out : p.spec)[(size_t)f * ncols + c] = res[cc * nT + f];
  }
}

// ---------------------------------------------------------------------------
// host-side launchers
// ---------------------------------------------------------------------------
template <int M, int MODE, int C>
static int launch_fast_t_mode(const TParams& p, cudaStream_t st) {
  using PL = FastPlan<M>;
  constexpr int LS = PL::PADDED + 2;
  const size_t smem = (size_t)(C * LS + M) * sizeof(float2);
  static bool attr_done[ASG_MAX_DEVICES] = {};
  static int resident[ASG_MAX_DEVICES] = {};
  const int dev = asg_device_slot();
  if (!attr_done[dev]) {
    if (cudaFuncSetAttribute(tk_fast<PL, MODE, C>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess)
      return ASG_ERR_CUDA;
    int per_sm = 0, nsm = 0, d = 0;
    if (cudaGetDevice(&d) == cudaSuccess &&
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, d) == cudaSuccess &&
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tk_fast<PL, MODE, C>, 256,
                                                      smem) == cudaSuccess)
      resident[dev] = per_sm * nsm;
    attr_done[dev] = true;
  }
  const int grid = (p.X / 2) * (p.Y / (C / 2));
  TParams q = p;
  q.prefetch_ahead = p.prefetch ? resident[dev] : 0;
  tk_fast<PL, MODE, C><<<grid, 256, smem, st>>>(q);
  return cudaPeekAtLastError() == cudaSuccess ? ASG_OK : ASG_ERR_CUDA;
}

// 16 columns per block exist up to 1024-sample columns (three blocks of 256
// threads still fit an SM in the transform-only and statistics modes, two in
// the flux mode).
bool asg_t_cols_supported(int nT, int Y, int flux, int cols) {
  (void)flux;
  if (cols == 8) return Y % 4 == 0;
  if (cols == 16) return nT <= 1024 && Y % 8 == 0;
  return false;
}

int asg_t_default_cols(int nT, int Y, int flux) {
  return asg_t_cols_supported(nT, Y, flux, 16) ? 16 : 8;
}

template <int M>
static int launch_fast_t(const TParams& p, cudaStream_t st) {
  const bool flux = p.op.flux != FLUX_NONE && !p.stats;
  int c = p.cols_per_block ? p.cols_per_block : asg_t_default_cols(2 * M, p.Y, flux);
  if (!asg_t_cols_supported(2 * M, p.Y, flux, c)) return ASG_ERR_SHAPE;
  if (p.stats)
    return c == 16 ? launch_fast_t_mode<M, TM_STATS, (M <= 512 ? 16 : 8)>(p, st)
                   : launch_fast_t_mode<M, TM_STATS, 8>(p, st);
  if (flux)
    return c == 16 ? launch_fast_t_mode<M, TM_FLUX, (M <= 512 ? 16 : 8)>(p, st)
                   : launch_fast_t_mode<M, TM_FLUX, 8>(p, st);
  return c == 16 ? launch_fast_t_mode<M, TM_PLAIN, (M <= 512 ? 16 : 8)>(p, st)
                 : launch_fast_t_mode<M, TM_PLAIN, 8>(p, st);
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
size_t asg_t_generic_smem(int nT) {
  return (size_t)(2 * 4 * nT + nT) * sizeof(float2) + (size_t)4 * nT * sizeof(float);
}

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
