// xy-plane kernels: per rfft bin (one "plane" of X*Y complex values), the
// forward 2-D FFT over (x, y), the per-mode multiplier of the step
// (diffraction x attenuation/Kramers-Kronig, diffraction alone or attenuation
// alone; FP64-built, stored as complex64 class tables), the inverse 2-D FFT
// and, for the stage that closes a step, the (x, y, omega) epilogue:
// frequency-weighted boundary, super-absorbing boundary and phase/amplitude
// screens.
//
// Fast kernel: the plane is held by a thread-block cluster of G = X/32 CTAs,
// 32 rows each, in shared memory; the x transform is split into a G-point DFT
// across the cluster (distributed shared memory, in place) and a 32-point DFT
// inside each CTA.  One HBM read and one HBM write per plane.
//
// Reference semantics (angular_spectrum_solver.py):
//   diffraction  _angular_spectrum_step :649-655 with HH from :396-462.  The
//     full complex 3-D FFT times the analytic-signal propagator (negative t
//     frequencies and DC zeroed, positive doubled) followed by the real part
//     equals: rfft along t, 2-D FFT, times HH on bins 1..ceil(nT/2)-1, zero
//     on bins 0 and nT/2, 2-D inverse FFT, irfft along t.
//   attenuation  _attenuation_step :667-685
//   freq-weighted  :658-664, super-absorbing :185-272, phase screen :352-390
//   beam obliquity power sums :630-643
#include <cooperative_groups.h>

#include "asg_generic.cuh"
#include "asg_internal.h"

namespace cg = cooperative_groups;

ASG_DEFINE_ROOT_UPLOADER(asg_roots_upload_xy)

// ---------------------------------------------------------------------------
// stability test and plane skip (uniform across a cluster)
// ---------------------------------------------------------------------------
ASG_DEV bool xy_should_skip(const XYParams& p) {
  if (*((volatile const unsigned*)p.status) != 0u) return true;
  if (p.check_stability) {
    const float m = __uint_as_float(*p.max_cur);
    const bool nan = (m != m) || isinf(m);
    const bool bad = nan || (p.stab_coef * (double)m > p.stab_thr);
    if (bad) {
      if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) {
        if (atomicCAS(p.status, 0u, (unsigned)(nan ? -ASG_ERR_NAN : -ASG_ERR_STABILITY)) == 0u)
          *p.status_step = *p.step;
      }
      return true;
    }
  }
  return false;
}

ASG_DEV bool is_dc_or_nyq(int f, int nT) { return f == 0 || 2 * f == nT; }

// ---------------------------------------------------------------------------
// (x, y, omega) epilogue on rows [0, R) of a plane held in shared memory.
// Row r is global x = x0 + r; element (r, y) at base[r*RS + POS(y)].
// halo_lo / halo_hi: rows x0-1 and x0+R (null at the global edges).
// ---------------------------------------------------------------------------
struct PosIdentity {
  ASG_DEV static int pos(int s) { return s; }
};

template <class POS>
ASG_DEV void epilogue(const XYParams& p, int plane, int f, float2* base, int RS, int R, int x0,
                      const float2* halo_lo, const float2* halo_hi) {
  const int X = p.X, Y = p.Y;
  const int tid = threadIdx.x, nthr = blockDim.x;
  const bool realify = is_dc_or_nyq(f, p.nT);
  // Re() after the attenuation inverse (irfft between reference steps)
  if (realify) {
    for (int i = tid; i < R * Y; i += nthr) {
      const int r = i / Y, y = i - (i / Y) * Y;
      base[r * RS + POS::pos(y)].y = 0.f;
    }
    __syncthreads();
  }
  if (p.epi & EPI_FREQW) {
    const float e = p.fw_exp[plane];
    for (int i = tid; i < R * Y; i += nthr) {
      const int r = i / Y, y = i - (i / Y) * Y;
      const float g = exp2f(e * (p.fw_lx[x0 + r] + p.fw_ly[y]));
      float2& v = base[r * RS + POS::pos(y)];
      v = cscale(v, g);
    }
    __syncthreads();
  }
  if (p.epi & EPI_SUPERABS) {
    const float c = p.sa_coef[plane];  // coeff = -i c
    const float s = p.sa_strength;
    // ---- x edges: one thread per y walks the rows, keeping the originals ----
    for (int y = tid; y < Y; y += nthr) {
      const int py = POS::pos(y);
      float2 prev = halo_lo ? halo_lo[py] : make_float2(0.f, 0.f);
      float2 cur = base[py];
      for (int r = 0; r < R; ++r) {
        const int x = x0 + r;
        float2 next = (r + 1 < R) ? base[(r + 1) * RS + py]
                                  : (halo_hi ? halo_hi[py] : make_float2(0.f, 0.f));
        const float w = p.sa_wx[x];
        if (w != 0.f) {
          float2 d;
          if (x == 0) d = cscale(csub(next, cur), p.sa_invdx);
          else if (x == X - 1) d = cscale(csub(cur, prev), p.sa_invdx);
          else d = cscale(csub(next, prev), p.sa_inv2dx);
          // coeff * d = -i c d = (c d.y, -c d.x)
          const float2 cd = make_float2(c * d.y, -c * d.x);
          const bool lo = x < X / 2;
          const float2 P = lo ? make_float2(0.5f * (cur.x + cd.x), 0.5f * (cur.y + cd.y))
                              : make_float2(0.5f * (cur.x - cd.x), 0.5f * (cur.y - cd.y));
          base[r * RS + py] = make_float2(cur.x - s * w * P.x, cur.y - s * w * P.y);
        }
        prev = cur;
        cur = next;
      }
    }
    __syncthreads();
    // ---- y edges on the x-corrected values: one warp per row ----
    const int lane = tid & 31, warp = tid >> 5, nw = nthr >> 5;
    for (int r = warp; r < R; r += nw) {
      float2* row = base + r * RS;
      float2 res[32];
#pragma unroll
      for (int k = 0; k < 32; ++k) {
        const int y = lane + 32 * k;
        if (y < Y) {
          const float2 cur = row[POS::pos(y)];
          res[k] = cur;
          const float w = p.sa_wy[y];
          if (w != 0.f) {
            float2 d;
            if (y == 0) d = cscale(csub(row[POS::pos(1)], cur), p.sa_invdy);
            else if (y == Y - 1) d = cscale(csub(cur, row[POS::pos(Y - 2)]), p.sa_invdy);
            else d = cscale(csub(row[POS::pos(y + 1)], row[POS::pos(y - 1)]), p.sa_inv2dy);
            const float2 cd = make_float2(c * d.y, -c * d.x);
            const bool lo = y < Y / 2;
            const float2 P = lo ? make_float2(0.5f * (cur.x + cd.x), 0.5f * (cur.y + cd.y))
                                : make_float2(0.5f * (cur.x - cd.x), 0.5f * (cur.y - cd.y));
            res[k] = make_float2(cur.x - s * w * P.x, cur.y - s * w * P.y);
          }
        }
      }
      __syncwarp();
#pragma unroll
      for (int k = 0; k < 32; ++k) {
        const int y = lane + 32 * k;
        if (y < Y) {
          float2 v = res[k];
          if (realify) v.y = 0.f;
          row[POS::pos(y)] = v;
        }
      }
      __syncwarp();
    }
    __syncthreads();
  }
  for (int k = 0; k < p.nscreens; ++k) {
    const float fs = p.screen_fscale[plane];
    const ScreenDev sc = p.screens[k];
    for (int i = tid; i < R * Y; i += nthr) {
      const int r = i / Y, y = i - (i / Y) * Y;
      const size_t g = (size_t)(x0 + r) * Y + y;
      float sn, cs;
      sincosf(sc.phase[g] * fs, &sn, &cs);
      float2 v = cmul(base[r * RS + POS::pos(y)], make_float2(cs, -sn));
      if (sc.amp != nullptr) {
        const float a = fminf(fmaxf(sc.amp[g], 1e-6f), 1.0f);
        v = cscale(v, exp2f(fs * log2f(a)));
      }
      if (realify) v.y = 0.f;
      base[r * RS + POS::pos(y)] = v;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// cross-CTA G-point DFT along x (in place over the cluster)
// ---------------------------------------------------------------------------
template <int G, bool INV, class PY>
ASG_DEV void cross_dft(cg::cluster_group& cl, float2* rows, int RS, int R, int Y, int X,
                       const float2* twX, int rank, int nthr) {
  float2* rem[G];
#pragma unroll
  for (int h = 0; h < G; ++h) rem[h] = cl.map_shared_rank(rows, h);
  for (int i = rank * nthr + (int)threadIdx.x; i < R * Y; i += G * nthr) {
    const int r = i / Y, s = i - (i / Y) * Y;
    const int off = r * RS + PY::pos(s);
    float2 v[G];
#pragma unroll
    for (int h = 0; h < G; ++h) v[h] = rem[h][off];
    dft<G, INV>(v);
    if (!INV) {
#pragma unroll
      for (int k1 = 1; k1 < G; ++k1) v[k1] = cmul(v[k1], twX[(r * k1) % X]);
    }
#pragma unroll
    for (int h = 0; h < G; ++h) rem[h][off] = v[h];
  }
}

template <bool INV, class PY>
ASG_DEV void cross_dft_rt(cg::cluster_group& cl, int G, float2* rows, int RS, int R, int Y, int X,
                          const float2* twX, int rank, int nthr) {
  switch (G) {
    case 2: cross_dft<2, INV, PY>(cl, rows, RS, R, Y, X, twX, rank, nthr); break;
    case 3: cross_dft<3, INV, PY>(cl, rows, RS, R, Y, X, twX, rank, nthr); break;
    case 4: cross_dft<4, INV, PY>(cl, rows, RS, R, Y, X, twX, rank, nthr); break;
    case 6: cross_dft<6, INV, PY>(cl, rows, RS, R, Y, X, twX, rank, nthr); break;
    case 8: cross_dft<8, INV, PY>(cl, rows, RS, R, Y, X, twX, rank, nthr); break;
    case 12: cross_dft<12, INV, PY>(cl, rows, RS, R, Y, X, twX, rank, nthr); break;
    case 16: cross_dft<16, INV, PY>(cl, rows, RS, R, Y, X, twX, rank, nthr); break;
    default: break;
  }
}

// ---------------------------------------------------------------------------
// fast kernel
// ---------------------------------------------------------------------------
constexpr int XY_R = 32;

template <class PY, int NT>
__global__ void __launch_bounds__(NT) xy_fast(XYParams p) {
  constexpr int Y = PY::N, N1 = PY::N1, N2 = PY::N2, RS = PY::PADDED, R = XY_R;
  constexpr int NW = NT / 32;
  extern __shared__ float4 smraw[];
  float2* rows = reinterpret_cast<float2*>(smraw);
  float2* halo = rows + R * RS;       // 2 rows (epilogue)
  float2* twY = halo + 2 * RS;
  float2* twX = twY + Y;              // X <= 512
  int* clsy = reinterpret_cast<int*>(twX + 512);
  int* clsx = clsy + Y;
  __shared__ float red[2][NW];

  const int G = p.G, X = p.X;
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (G > 1) ? (int)cl.block_rank() : 0;
  const int plane = blockIdx.y;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (xy_should_skip(p)) return;
  const int f = p.f_of_plane[plane];
  float2* gplane = p.spec + (size_t)plane * X * Y;
  if (p.zero_dc_nyq && is_dc_or_nyq(f, p.nT)) {
    float4* g4 = reinterpret_cast<float4*>(gplane + (size_t)rank * R * Y);
    for (int i = tid; i < R * Y / 2; i += NT) g4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    return;
  }
  for (int i = tid; i < Y; i += NT) {
    twY[i] = p.twY[i];
    clsy[i] = p.cls_y[i];
  }
  for (int i = tid; i < X; i += NT) twX[i] = p.twX[i];
  for (int i = tid; i < R; i += NT) clsx[i] = p.cls_x[rank * R + i];
  __syncthreads();

  // ---- forward FFT along y, fused with the HBM load ----
  for (int r = warp; r < R; r += NW) {
    float2* row = rows + r * RS;
    const float2* grow = gplane + (size_t)(rank * R + r) * Y;
    for (int b = lane; b < N2; b += 32) {
      float2 v[N1];
#pragma unroll
      for (int a = 0; a < N1; ++a) v[a] = grow[b + N2 * a];
      dft<N1, false>(v);
      row[PY::pos(b)] = v[0];
#pragma unroll
      for (int ka = 1; ka < N1; ++ka) row[PY::pos(b + N2 * ka)] = cmul(v[ka], twY[(b * ka) % Y]);
    }
    __syncwarp();
    for (int ka = lane; ka < N1; ka += 32) stepB_smem<PY, false>(row, ka);
    __syncwarp();
  }

  // ---- x: G-point DFT across the cluster ----
  if (G > 1) {
    cl.sync();
    cross_dft_rt<false, PY>(cl, G, rows, RS, R, Y, X, twX, rank, NT);
    cl.sync();
  } else {
    __syncthreads();
  }

  // ---- x: 32-point DFT per column, multiplier, inverse ----
  float psum = 0.f, pden = 0.f;
  for (int s = tid; s < Y; s += NT) {
    const int ps = PY::pos(s);
    float2 v[R];
#pragma unroll
    for (int j = 0; j < R; ++j) v[j] = rows[j * RS + ps];
    dft<R, false>(v);
    if (p.power_only) {
      const float* ot = p.obl_table + (size_t)plane * p.ncx * p.ncy + clsy[s];
#pragma unroll
      for (int j = 0; j < R; ++j) {
        const float o = ot[(size_t)clsx[j] * p.ncy];
        const float P = v[j].x * v[j].x + v[j].y * v[j].y;
        psum = fmaf(P, o, psum);
        pden += (o > 0.f) ? P : 0.f;
      }
      continue;
    }
    if (p.table != nullptr) {
      const float2* tt = p.table + (size_t)plane * p.ncx * p.ncy + clsy[s];
#pragma unroll
      for (int j = 0; j < R; ++j) v[j] = cmul(v[j], tt[(size_t)clsx[j] * p.ncy]);
    } else {
      const float nrm = 1.0f / ((float)X * (float)Y);
#pragma unroll
      for (int j = 0; j < R; ++j) v[j] = cscale(v[j], nrm);
    }
    dft<R, true>(v);
    if (G > 1) {
#pragma unroll
      for (int j = 1; j < R; ++j) v[j] = cmulc(v[j], twX[(j * rank) % X]);
    }
#pragma unroll
    for (int j = 0; j < R; ++j) rows[j * RS + ps] = v[j];
  }
  if (p.power_only) {
    psum = warp_sum(psum);
    pden = warp_sum(pden);
    if (lane == 0) {
      red[0][warp] = psum;
      red[1][warp] = pden;
    }
    __syncthreads();
    if (tid == 0) {
      double a = 0.0, b = 0.0;
      for (int w = 0; w < NW; ++w) {
        a += (double)red[0][w];
        b += (double)red[1][w];
      }
      atomicAdd(p.power_acc, a);
      atomicAdd(p.power_acc + 1, b);
    }
    if (G > 1) cl.sync();  // no CTA leaves while others may read its rows
    return;
  }

  // ---- x: inverse G-point DFT across the cluster ----
  if (G > 1) {
    cl.sync();
    cross_dft_rt<true, PY>(cl, G, rows, RS, R, Y, X, twX, rank, NT);
    cl.sync();
  } else {
    __syncthreads();
  }

  // ---- inverse FFT along y (and store, unless an epilogue follows) ----
  const bool epi = p.epi != 0 || p.nscreens > 0;
  for (int r = warp; r < R; r += NW) {
    float2* row = rows + r * RS;
    float2* grow = gplane + (size_t)(rank * R + r) * Y;
    for (int ka = lane; ka < N1; ka += 32) stepB_smem<PY, true>(row, ka);
    __syncwarp();
    for (int b = lane; b < N2; b += 32) {
      float2 v[N1];
      v[0] = row[PY::pos(b)];
#pragma unroll
      for (int ka = 1; ka < N1; ++ka) v[ka] = cmulc(row[PY::pos(b + N2 * ka)], twY[(b * ka) % Y]);
      dft<N1, true>(v);
      if (!epi) {
#pragma unroll
        for (int a = 0; a < N1; ++a) grow[b + N2 * a] = v[a];
      } else {
        // lane b reads and writes only the slots of its own subline
#pragma unroll
        for (int a = 0; a < N1; ++a) row[PY::pos(b + N2 * a)] = v[a];
      }
    }
    __syncwarp();
  }
  if (!epi) return;

  // ---- (x, y, omega) epilogue ----
  __syncthreads();
  const float2* hlo = nullptr;
  const float2* hhi = nullptr;
  if ((p.epi & EPI_SUPERABS) && G > 1) {
    // rows x0-1 and x0+R from the neighbours, taken before anyone updates
    cl.sync();
    if (rank > 0) {
      const float2* nb = cl.map_shared_rank(rows, rank - 1) + (R - 1) * RS;
      for (int i = tid; i < RS; i += NT) halo[i] = nb[i];
      hlo = halo;
    }
    if (rank < G - 1) {
      const float2* nb = cl.map_shared_rank(rows, rank + 1);
      for (int i = tid; i < RS; i += NT) halo[RS + i] = nb[i];
      hhi = halo + RS;
    }
    cl.sync();
  }
  epilogue<PY>(p, plane, f, rows, RS, R, rank * R, hlo, hhi);
  for (int i = tid; i < R * Y; i += NT) {
    const int r = i / Y, y = i - (i / Y) * Y;
    gplane[(size_t)(rank * R + r) * Y + y] = rows[r * RS + PY::pos(y)];
  }
}

// ---------------------------------------------------------------------------
// generic kernel: one CTA per plane, whole plane in shared memory (ping-pong)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) xy_generic(XYParams p, GenPlan plx, GenPlan ply) {
  const int X = p.X, Y = p.Y;
  extern __shared__ float4 smraw[];
  float2* A = reinterpret_cast<float2*>(smraw);
  float2* B = A + X * Y;
  float2* twX = B + X * Y;
  float2* twY = twX + X;
  int* clsx = reinterpret_cast<int*>(twY + Y);
  int* clsy = clsx + X;
  __shared__ float red[2][8];
  const int plane = blockIdx.y;
  const int tid = threadIdx.x, nthr = blockDim.x;
  if (xy_should_skip(p)) return;
  const int f = p.f_of_plane[plane];
  float2* gplane = p.spec + (size_t)plane * X * Y;
  if (p.zero_dc_nyq && is_dc_or_nyq(f, p.nT)) {
    for (int i = tid; i < X * Y; i += nthr) gplane[i] = make_float2(0.f, 0.f);
    return;
  }
  for (int i = tid; i < X; i += nthr) {
    twX[i] = p.twX[i];
    clsx[i] = p.cls_x[i];
  }
  for (int i = tid; i < Y; i += nthr) {
    twY[i] = p.twY[i];
    clsy[i] = p.cls_y[i];
  }
  for (int i = tid; i < X * Y; i += nthr) A[i] = gplane[i];
  __syncthreads();
  float2* r1 = gen_fft<false>(A, B, X, Y, 1, ply, twY);
  float2* o1 = (r1 == A) ? B : A;
  float2* r2 = gen_fft<false>(r1, o1, Y, 1, Y, plx, twX);
  float psum = 0.f, pden = 0.f;
  const float nrm = 1.0f / ((float)X * (float)Y);
  for (int i = tid; i < X * Y; i += nthr) {
    const int x = i / Y, y = i - (i / Y) * Y;
    const size_t ti = ((size_t)plane * p.ncx + clsx[x]) * p.ncy + clsy[y];
    if (p.power_only) {
      const float o = p.obl_table[ti];
      const float P = r2[i].x * r2[i].x + r2[i].y * r2[i].y;
      psum = fmaf(P, o, psum);
      pden += (o > 0.f) ? P : 0.f;
    } else if (p.table != nullptr) {
      r2[i] = cmul(r2[i], p.table[ti]);
    } else {
      r2[i] = cscale(r2[i], nrm);
    }
  }
  if (p.power_only) {
    psum = warp_sum(psum);
    pden = warp_sum(pden);
    if ((tid & 31) == 0) {
      red[0][tid >> 5] = psum;
      red[1][tid >> 5] = pden;
    }
    __syncthreads();
    if (tid == 0) {
      double a = 0.0, b = 0.0;
      for (int w = 0; w < nthr / 32; ++w) {
        a += (double)red[0][w];
        b += (double)red[1][w];
      }
      atomicAdd(p.power_acc, a);
      atomicAdd(p.power_acc + 1, b);
    }
    return;
  }
  __syncthreads();
  float2* o2 = (r2 == A) ? B : A;
  float2* r3 = gen_fft<true>(r2, o2, Y, 1, Y, plx, twX);
  float2* o3 = (r3 == A) ? B : A;
  float2* r4 = gen_fft<true>(r3, o3, X, Y, 1, ply, twY);
  if (p.epi != 0 || p.nscreens > 0) epilogue<PosIdentity>(p, plane, f, r4, Y, X, 0, nullptr, nullptr);
  for (int i = tid; i < X * Y; i += nthr) gplane[i] = r4[i];
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
bool asg_xy_fast_supported(int X, int Y, int* G_out) {
  if (X % XY_R != 0) return false;
  const int G = X / XY_R;
  if (!(G == 1 || G == 2 || G == 3 || G == 4 || G == 6 || G == 8 || G == 12 || G == 16))
    return false;
  switch (Y) {
    case 64: case 96: case 128: case 192: case 256: case 384: case 512: break;
    default: return false;
  }
  if (G_out) *G_out = G;
  return true;
}

size_t asg_xy_generic_smem(int X, int Y) {
  return (size_t)(2 * X * Y + X + Y) * sizeof(float2) + (size_t)(X + Y) * sizeof(int);
}

template <int Yn>
static int launch_fast_xy(const XYParams& p, cudaStream_t st) {
  using PY = FastPlan<Yn>;
  constexpr int NT = (Yn >= 256) ? 512 : 256;
  const size_t smem = (size_t)(XY_R * PY::PADDED + 2 * PY::PADDED + Yn + 512) * sizeof(float2) +
                      (size_t)(Yn + XY_R) * sizeof(int);
  static bool attr_done = false;
  if (!attr_done) {
    if (cudaFuncSetAttribute(xy_fast<PY, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess)
      return ASG_ERR_CUDA;
    cudaFuncSetAttribute(xy_fast<PY, NT>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    attr_done = true;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(p.G, p.nplanes, 1);
  cfg.blockDim = dim3(NT, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = p.G;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaError_t e = cudaLaunchKernelEx(&cfg, xy_fast<PY, NT>, p);
  return e == cudaSuccess ? ASG_OK : ASG_ERR_CUDA;
}

int asg_launch_xy(const XYParams& p, bool fast, const GenPlan& plx, const GenPlan& ply,
                  cudaStream_t st) {
  if (fast) {
    switch (p.Y) {
      case 64: return launch_fast_xy<64>(p, st);
      case 96: return launch_fast_xy<96>(p, st);
      case 128: return launch_fast_xy<128>(p, st);
      case 192: return launch_fast_xy<192>(p, st);
      case 256: return launch_fast_xy<256>(p, st);
      case 384: return launch_fast_xy<384>(p, st);
      case 512: return launch_fast_xy<512>(p, st);
      default: return ASG_ERR_SHAPE;
    }
  }
  const size_t smem = asg_xy_generic_smem(p.X, p.Y);
  if (cudaFuncSetAttribute(xy_generic, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return ASG_ERR_CUDA;
  xy_generic<<<dim3(1, p.nplanes, 1), 256, smem, st>>>(p, plx, ply);
  return cudaPeekAtLastError() == cudaSuccess ? ASG_OK : ASG_ERR_CUDA;
}
