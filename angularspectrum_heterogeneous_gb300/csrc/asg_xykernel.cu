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
    // ---- y edges on the x-corrected values: one warp per row, 32 y at a
    //      time; neighbours come from shuffles, the chunk borders from the
    //      original values kept before they are overwritten ----
    const int lane = tid & 31, warp = tid >> 5, nw = nthr >> 5;
    for (int r = warp; r < R; r += nw) {
      float2* row = base + r * RS;
      float2 prev_last = make_float2(0.f, 0.f);  // original value at y0-1
      for (int y0 = 0; y0 < Y; y0 += 32) {
        const int y = y0 + lane;
        const float2 cur = (y < Y) ? row[POS::pos(y)] : make_float2(0.f, 0.f);
        float2 left, right;
        left.x = __shfl_up_sync(0xffffffffu, cur.x, 1);
        left.y = __shfl_up_sync(0xffffffffu, cur.y, 1);
        right.x = __shfl_down_sync(0xffffffffu, cur.x, 1);
        right.y = __shfl_down_sync(0xffffffffu, cur.y, 1);
        if (lane == 0) left = prev_last;
        if (lane == 31 && y + 1 < Y) right = row[POS::pos(y + 1)];
        float2 res = cur;
        if (y < Y) {
          const float w = p.sa_wy[y];
          if (w != 0.f) {
            float2 d;
            if (y == 0) d = cscale(csub(right, cur), p.sa_invdy);
            else if (y == Y - 1) d = cscale(csub(cur, left), p.sa_invdy);
            else d = cscale(csub(right, left), p.sa_inv2dy);
            const float2 cd = make_float2(c * d.y, -c * d.x);
            const bool lo = y < Y / 2;
            const float2 P = lo ? make_float2(0.5f * (cur.x + cd.x), 0.5f * (cur.y + cd.y))
                                : make_float2(0.5f * (cur.x - cd.x), 0.5f * (cur.y - cd.y));
            res = make_float2(cur.x - s * w * P.x, cur.y - s * w * P.y);
          }
          if (realify) res.y = 0.f;
        }
        prev_last.x = __shfl_sync(0xffffffffu, cur.x, 31);
        prev_last.y = __shfl_sync(0xffffffffu, cur.y, 31);
        __syncwarp();
        if (y < Y) row[POS::pos(y)] = res;
        __syncwarp();
      }
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
// asynchronous global -> shared copies (16 bytes per thread and copy)
// ---------------------------------------------------------------------------
ASG_DEV void cp_async16(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
ASG_DEV void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
ASG_DEV void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// ---------------------------------------------------------------------------
// cross-CTA G-point DFT along x, in place over the cluster, two slots
// (16 bytes) per access
// ---------------------------------------------------------------------------
ASG_DEV unsigned cluster_addr(const void* local_smem, int rank) {
  const unsigned la = (unsigned)__cvta_generic_to_shared(local_smem);
  unsigned ra;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;\n" : "=r"(ra) : "r"(la), "r"(rank));
  return ra;
}
ASG_DEV float4 ld_cluster4(unsigned a) {
  float4 v;
  asm volatile("ld.shared::cluster.v4.f32 {%0,%1,%2,%3}, [%4];\n"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "r"(a)
               : "memory");
  return v;
}
ASG_DEV void st_cluster4(unsigned a, float4 v) {
  asm volatile("st.shared::cluster.v4.f32 [%0], {%1,%2,%3,%4};\n" ::"r"(a), "f"(v.x), "f"(v.y),
               "f"(v.z), "f"(v.w)
               : "memory");
}

ASG_DEV float2 ld_cluster2(unsigned a) {
  float2 v;
  asm volatile("ld.shared::cluster.v2.f32 {%0,%1}, [%2];\n" : "=f"(v.x), "=f"(v.y) : "r"(a) : "memory");
  return v;
}
ASG_DEV void st_cluster2(unsigned a, float2 v) {
  asm volatile("st.shared::cluster.v2.f32 [%0], {%1,%2};\n" ::"r"(a), "f"(v.x), "f"(v.y) : "memory");
}

// pairs of slots (16-byte accesses) for G <= 8, single slots above (registers)
template <int G, bool INV, class PY, int R, int NT>
ASG_DEV void cross_dft(float2* rows, const float2* twX, int rank) {
  constexpr int Y = PY::N, RS = PY::PADDED;
  unsigned base[G];
#pragma unroll
  for (int h = 0; h < G; ++h) base[h] = cluster_addr(rows, h);
  if constexpr (G <= 8) {
    constexpr int NPAIR = R * Y / 2;
    for (int i = rank * NT + (int)threadIdx.x; i < NPAIR; i += G * NT) {
      const int r = i / (Y / 2), s = 2 * (i - r * (Y / 2));
      const unsigned off = (unsigned)(r * RS + PY::pos(s)) * 8u;
      float2 a[G], b[G];
#pragma unroll
      for (int h = 0; h < G; ++h) {
        const float4 q = ld_cluster4(base[h] + off);
        a[h] = make_float2(q.x, q.y);
        b[h] = make_float2(q.z, q.w);
      }
      dft<G, INV>(a);
      dft<G, INV>(b);
      if (!INV) {
#pragma unroll
        for (int k1 = 1; k1 < G; ++k1) {
          const float2 w = twX[r * k1];  // r*k1 < R*G = rows of the (sub-)plane
          a[k1] = cmul(a[k1], w);
          b[k1] = cmul(b[k1], w);
        }
      }
#pragma unroll
      for (int h = 0; h < G; ++h)
        st_cluster4(base[h] + off, make_float4(a[h].x, a[h].y, b[h].x, b[h].y));
    }
  } else {
    constexpr int NS = R * Y;
    for (int i = rank * NT + (int)threadIdx.x; i < NS; i += G * NT) {
      const int r = i / Y, s = i - r * Y;
      const unsigned off = (unsigned)(r * RS + PY::pos(s)) * 8u;
      float2 a[G];
#pragma unroll
      for (int h = 0; h < G; ++h) a[h] = ld_cluster2(base[h] + off);
      dft<G, INV>(a);
      if (!INV) {
#pragma unroll
        for (int k1 = 1; k1 < G; ++k1) a[k1] = cmul(a[k1], twX[r * k1]);
      }
#pragma unroll
      for (int h = 0; h < G; ++h) st_cluster2(base[h] + off, a[h]);
    }
  }
}

template <bool INV, class PY, int R, int NT>
ASG_DEV void cross_dft_rt(int G, float2* rows, const float2* twX, int rank) {
  switch (G) {
    case 2: cross_dft<2, INV, PY, R, NT>(rows, twX, rank); break;
    case 3: cross_dft<3, INV, PY, R, NT>(rows, twX, rank); break;
    case 4: cross_dft<4, INV, PY, R, NT>(rows, twX, rank); break;
    case 6: cross_dft<6, INV, PY, R, NT>(rows, twX, rank); break;
    case 8: cross_dft<8, INV, PY, R, NT>(rows, twX, rank); break;
    case 12: cross_dft<12, INV, PY, R, NT>(rows, twX, rank); break;
    case 16: cross_dft<16, INV, PY, R, NT>(rows, twX, rank); break;
    default: break;
  }
}

// ---------------------------------------------------------------------------
// fast kernel: persistent thread-block clusters, one (sub-)plane at a time.
// A cluster of G CTAs holds an Xs x Y (sub-)plane, R rows per CTA, in shared
// memory; rows of the next plane are prefetched with cp.async as soon as the
// current plane's rows are stored.
// ---------------------------------------------------------------------------
template <class PY, int R, int NT>
__global__ void __launch_bounds__(NT, (NT == 256 ? 2 : 1)) xy_fast(XYParams p) {
  constexpr int Y = PY::N, N1 = PY::N1, N2 = PY::N2, RS = PY::PADDED;
  constexpr int NW = NT / 32;
  extern __shared__ float4 smraw[];
  float2* rows = reinterpret_cast<float2*>(smraw);
  float2* halo = rows + R * RS;       // 2 rows (epilogue)
  float2* twY = halo + 2 * RS;
  float2* twX = twY + Y;              // Xs <= 512
  int* clsy = reinterpret_cast<int*>(twX + 512);
  int* clsx = clsy + Y;               // [nsub][R]
  __shared__ float red[2][NW];

  const int G = p.G;
  const int nsub = p.nsub;
  const int Xs = p.X / nsub;          // rows of one (sub-)plane
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (G > 1) ? (int)cl.block_rank() : 0;
  const int cid = blockIdx.x / G, ncl = gridDim.x / G;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nq = p.nplanes * nsub;

  if (xy_should_skip(p)) return;
  for (int i = tid; i < Y; i += NT) {
    twY[i] = p.twY[i];
    clsy[i] = p.cls_y[i];
  }
  // roots of the (sub-)plane length Xs: W_Xs^i = W_X^(nsub i)
  for (int i = tid; i < Xs; i += NT) twX[i] = p.twX[i * nsub];
  for (int i = tid; i < nsub * R; i += NT) {
    const int h = i / R, j = i - (i / R) * R;
    clsx[i] = p.cls_x[h * Xs + rank * R + j];
  }
  auto zero_plane = [&](int q) {
    return p.zero_dc_nyq && is_dc_or_nyq(p.f_of_plane[q / nsub], p.nT);
  };
  auto sub_base = [&](int q) {  // first element of this CTA's rows of sub-plane q
    const int plane = q / nsub, h = q - (q / nsub) * nsub;
    return p.spec + ((size_t)plane * p.X + (size_t)h * Xs + (size_t)rank * R) * Y;
  };
  auto prefetch_row = [&](int q, int r) {  // one warp
    const float2* g = sub_base(q) + (size_t)r * Y;
    float2* d = rows + r * RS;
    for (int s2 = lane; s2 < Y / 2; s2 += 32) cp_async16(d + PY::pos(2 * s2), g + 2 * s2);
  };
  const bool epi = p.epi != 0 || p.nscreens > 0;
  int issued = -1;

  for (int q = cid; q < nq; q += ncl) {
    const int plane = q / nsub, h = q - (q / nsub) * nsub;
    const int f = p.f_of_plane[plane];
    if (zero_plane(q)) {
      float4* g4 = reinterpret_cast<float4*>(sub_base(q));
      for (int i = tid; i < R * Y / 2; i += NT) g4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
      continue;
    }
    if (issued != q) {
      for (int r = warp; r < R; r += NW) prefetch_row(q, r);
      cp_async_commit();
    }
    cp_async_wait_all();
    __syncthreads();

    // ---- forward FFT along y ----
    for (int r = warp; r < R; r += NW) {
      float2* row = rows + r * RS;
      for (int b = lane; b < N2; b += 32) stepA_fwd_smem<PY, false>(row, b, twY);
      __syncwarp();
      for (int ka = lane; ka < N1; ka += 32) stepB_smem<PY, false>(row, ka);
      __syncwarp();
    }

    // ---- x: G-point DFT across the cluster ----
    if (G > 1) {
      cl.sync();
      cross_dft_rt<false, PY, R, NT>(G, rows, twX, rank);
      cl.sync();
    } else {
      __syncthreads();
    }

    // ---- x: R-point DFT per column, multiplier, inverse ----
    float psum = 0.f, pden = 0.f;
    const int* cx = clsx + h * R;
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
          const float o = ot[(size_t)cx[j] * p.ncy];
          const float P = v[j].x * v[j].x + v[j].y * v[j].y;
          psum = fmaf(P, o, psum);
          pden += (o > 0.f) ? P : 0.f;
        }
        continue;
      }
      if (p.table != nullptr) {
        const float2* tt = p.table + (size_t)plane * p.ncx * p.ncy + clsy[s];
#pragma unroll
        for (int j = 0; j < R; ++j) v[j] = cmul(v[j], tt[(size_t)cx[j] * p.ncy]);
      } else {
        const float nrm = 1.0f / ((float)Xs * (float)Y);
#pragma unroll
        for (int j = 0; j < R; ++j) v[j] = cscale(v[j], nrm);
      }
      dft<R, true>(v);
      if (G > 1) {
#pragma unroll
        for (int j = 1; j < R; ++j) v[j] = cmulc(v[j], twX[j * rank]);  // j*rank < Xs
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
      // every CTA finished reading the cluster's rows before they are reused
      if (G > 1) cl.sync();
      else __syncthreads();
      continue;
    }

    // ---- x: inverse G-point DFT across the cluster ----
    if (G > 1) {
      cl.sync();
      cross_dft_rt<true, PY, R, NT>(G, rows, twX, rank);
      cl.sync();
    } else {
      __syncthreads();
    }

    // next (sub-)plane of this cluster, prefetched while this one finishes
    int qn = q + ncl;
    while (qn < nq && zero_plane(qn)) qn += ncl;
    const bool pref = qn < nq;

    // ---- inverse FFT along y; store (or keep for the epilogue) ----
    float2* gbase = sub_base(q);
    for (int r = warp; r < R; r += NW) {
      float2* row = rows + r * RS;
      float2* grow = gbase + (size_t)r * Y;
      for (int ka = lane; ka < N1; ka += 32) stepB_smem<PY, true>(row, ka);
      __syncwarp();
      for (int b = lane; b < N2; b += 32) {
        float2 v[N1];
        v[0] = row[PY::pos(b)];
#pragma unroll
        for (int ka = 1; ka < N1; ++ka) v[ka] = cmulc(row[PY::pos(b + N2 * ka)], twY[b * ka]);
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
      if (!epi && pref) prefetch_row(qn, r);
    }
    if (!epi) {
      if (pref) {
        cp_async_commit();
        issued = qn;
      }
      continue;
    }

    // ---- (x, y, omega) epilogue (whole plane in the cluster: nsub == 1) ----
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
    for (int i = tid; i < R * Y / 2; i += NT) {
      const int r = i / (Y / 2), s = 2 * (i - r * (Y / 2));
      reinterpret_cast<float4*>(gbase + (size_t)r * Y + s)[0] =
          reinterpret_cast<const float4*>(rows + r * RS + PY::pos(s))[0];
    }
    __syncthreads();
    if (pref) {
      for (int r = warp; r < R; r += NW) prefetch_row(qn, r);
      cp_async_commit();
      issued = qn;
    }
  }
  cp_async_wait_all();
  // no CTA leaves while a neighbour may still read its shared memory
  if (G > 1) cl.sync();
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
// Generic kernels for planes too large for one CTA's shared memory (the odd
// sizes of the reference's validation scripts: 257 x 257, 365 x 365, ...):
// the plane transform runs as three passes over HBM, rows (y transform) of
// RB rows per CTA, then columns (x transform, multiplier, inverse x
// transform) of CB columns per CTA, then rows again (inverse y transform),
// each line a mixed-radix Stockham FFT in shared memory.  The boundary and
// screen epilogue, when the stage has one, follows as the tiled epilogue pass.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) xy_big_rows(XYParams p, GenPlan ply, const float2* src,
                                                   float2* dst, int inverse, int rb) {
  const int X = p.X, Y = p.Y;
  extern __shared__ float4 smraw[];
  float2* A = reinterpret_cast<float2*>(smraw);
  float2* B = A + rb * Y;
  float2* twY = B + rb * Y;
  const int plane = blockIdx.y, x0 = blockIdx.x * rb;
  const int tid = threadIdx.x, nthr = blockDim.x;
  if (xy_should_skip(p)) return;
  // (planes of bins 0 and nT/2 of the analytic-signal propagator are zeroed
  // by the column pass; the inverse row pass carries the zeros to dst)
  const int nr = min(rb, X - x0);
  for (int i = tid; i < Y; i += nthr) twY[i] = p.twY[i];
  const float2* s = src + ((size_t)plane * X + x0) * Y;
  for (int i = tid; i < nr * Y; i += nthr) A[i] = s[i];
  __syncthreads();
  float2* r = inverse ? gen_fft<true>(A, B, nr, Y, 1, ply, twY) : gen_fft<false>(A, B, nr, Y, 1, ply, twY);
  float2* d = dst + ((size_t)plane * X + x0) * Y;
  for (int i = tid; i < nr * Y; i += nthr) d[i] = r[i];
}

__global__ void __launch_bounds__(256) xy_big_cols(XYParams p, GenPlan plx, float2* buf, int cb) {
  const int X = p.X, Y = p.Y;
  extern __shared__ float4 smraw[];
  float2* A = reinterpret_cast<float2*>(smraw);  // [c][x]: one line per column
  float2* B = A + cb * X;
  float2* twX = B + cb * X;
  __shared__ float red[2][8];
  const int plane = blockIdx.y, y0 = blockIdx.x * cb;
  const int tid = threadIdx.x, nthr = blockDim.x;
  if (xy_should_skip(p)) return;
  const int nc = min(cb, Y - y0);
  float2* g = buf + (size_t)plane * X * Y + y0;
  if (p.zero_dc_nyq && is_dc_or_nyq(p.f_of_plane[plane], p.nT)) {
    for (int i = tid; i < X * nc; i += nthr) {
      const int x = i / nc, c = i - x * nc;
      g[(size_t)x * Y + c] = make_float2(0.f, 0.f);
    }
    return;
  }
  for (int i = tid; i < X; i += nthr) twX[i] = p.twX[i];
  for (int i = tid; i < X * nc; i += nthr) {
    const int x = i / nc, c = i - x * nc;
    A[c * X + x] = g[(size_t)x * Y + c];
  }
  __syncthreads();
  float2* r = gen_fft<false>(A, B, nc, X, 1, plx, twX);
  float psum = 0.f, pden = 0.f;
  const float nrm = 1.0f / ((float)X * (float)Y);
  for (int i = tid; i < X * nc; i += nthr) {
    const int c = i / X, x = i - c * X;
    const size_t ti = ((size_t)plane * p.ncx + p.cls_x[x]) * p.ncy + p.cls_y[y0 + c];
    if (p.power_only) {
      const float o = p.obl_table[ti];
      const float P = r[i].x * r[i].x + r[i].y * r[i].y;
      psum = fmaf(P, o, psum);
      pden += (o > 0.f) ? P : 0.f;
    } else if (p.table != nullptr) {
      r[i] = cmul(r[i], p.table[ti]);
    } else {
      r[i] = cscale(r[i], nrm);
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
  float2* o = (r == A) ? B : A;
  float2* r2 = gen_fft<true>(r, o, nc, X, 1, plx, twX);
  for (int i = tid; i < X * nc; i += nthr) {
    const int x = i / nc, c = i - x * nc;
    g[(size_t)x * Y + c] = r2[c * X + x];
  }
}

// lines per CTA of the row and column passes: about 4096 complex (two 32 KB
// ping-pong buffers)
static int big_lines_per_cta(int n) { return 4096 / n > 0 ? 4096 / n : 1; }

// rows forward (spec -> tmp), columns (tmp), rows inverse (tmp -> spec, or
// tmp -> tmp and the epilogue pass tmp -> spec); the power reduction stops
// after the columns and leaves spec untouched
static int launch_xy_big(const XYParams& p, const GenPlan& plx, const GenPlan& ply,
                         cudaStream_t st) {
  if (p.spec_tmp == nullptr) return ASG_ERR_STATE;
  const int rb = big_lines_per_cta(p.Y), cb = big_lines_per_cta(p.X);
  const size_t smr = (size_t)(2 * rb * p.Y + p.Y) * sizeof(float2);
  const size_t smc = (size_t)(2 * cb * p.X + p.X) * sizeof(float2);
  if (cudaFuncSetAttribute(xy_big_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smr) !=
          cudaSuccess ||
      cudaFuncSetAttribute(xy_big_cols, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smc) !=
          cudaSuccess)
    return ASG_ERR_CUDA;
  const dim3 gr((p.X + rb - 1) / rb, p.nplanes), gc((p.Y + cb - 1) / cb, p.nplanes);
  xy_big_rows<<<gr, 256, smr, st>>>(p, ply, p.spec, p.spec_tmp, 0, rb);
  xy_big_cols<<<gc, 256, smc, st>>>(p, plx, p.spec_tmp, cb);
  if (p.power_only) return cudaPeekAtLastError() == cudaSuccess ? ASG_OK : ASG_ERR_CUDA;
  const bool epi = p.epi != 0 || p.nscreens > 0;
  xy_big_rows<<<gr, 256, smr, st>>>(p, ply, p.spec_tmp, epi ? p.spec_tmp : p.spec, 1, rb);
  if (cudaPeekAtLastError() != cudaSuccess) return ASG_ERR_CUDA;
  if (epi) return asg_launch_epilogue_pass(p, p.spec_tmp, p.spec, 0, st);
  return ASG_OK;
}

// ---------------------------------------------------------------------------
// (x, y, omega) epilogue as its own pass over 32 x 32 tiles with a one-cell
// halo.  Input: the closing stage's output, either whole planes or the
// half-plane form (rows x < X/2 hold a, rows x >= X/2 hold b, and
// s(x) = a(x) + W_X^-x b(x), s(x + X/2) = a(x) - W_X^-x b(x)).  Output: whole
// planes s(x, y) with, in order, Re() on bins 0 and nT/2, frequency-weighted
// damping, the Engquist-Majda corrections (x edges, then y edges on the
// x-corrected values) and the phase/amplitude screens
// (angular_spectrum_solver.py:658-664, :185-272, :352-390, :1494-1518).
// ---------------------------------------------------------------------------
constexpr int EPT = 32;  // tile edge

__global__ void __launch_bounds__(256) xy_epilogue_pass(XYParams p, const float2* __restrict__ src,
                                                        float2* __restrict__ dst, int split) {
  __shared__ float2 S[EPT + 2][EPT + 3];
  __shared__ float2 XS[EPT][EPT + 3];
  if (*((volatile const unsigned*)p.status) != 0u) return;
  const int X = p.X, Y = p.Y, X2 = p.X / 2;
  const int ty = (Y + EPT - 1) / EPT;
  const int plane = blockIdx.y;
  const int x0 = (blockIdx.x / ty) * EPT, y0 = (blockIdx.x % ty) * EPT;
  const int f = p.f_of_plane[plane];
  const bool realify = is_dc_or_nyq(f, p.nT);
  const float2* sp = src + (size_t)plane * X * Y;
  float2* dp = dst + (size_t)plane * X * Y;
  const int tid = threadIdx.x;
  const bool fw = (p.epi & EPI_FREQW) != 0;
  const float fe = fw ? p.fw_exp[plane] : 0.f;
  // 1) s on the haloed tile
  for (int i = tid; i < (EPT + 2) * (EPT + 2); i += blockDim.x) {
    const int r = i / (EPT + 2), c = i - r * (EPT + 2);
    const int x = x0 - 1 + r, y = y0 - 1 + c;
    float2 v = make_float2(0.f, 0.f);
    if (x >= 0 && x < X && y >= 0 && y < Y) {
      if (split) {
        const int xh = x < X2 ? x : x - X2;
        const float2 a = sp[(size_t)xh * Y + y];
        const float2 b = cmulc(sp[(size_t)(xh + X2) * Y + y], p.twX[xh]);
        v = x < X2 ? cadd(a, b) : csub(a, b);
      } else {
        v = sp[(size_t)x * Y + y];
      }
      if (realify) v.y = 0.f;
      if (fw) v = cscale(v, exp2f(fe * (p.fw_lx[x] + p.fw_ly[y])));
    }
    S[r][c] = v;
  }
  __syncthreads();
  const bool sa = (p.epi & EPI_SUPERABS) != 0;
  const float cf = sa ? p.sa_coef[plane] : 0.f;  // coeff = -i cf
  const float st = p.sa_strength;
  // 2) x edges on rows of the tile, columns y0-1 .. y0+EPT
  if (sa) {
    for (int i = tid; i < EPT * (EPT + 2); i += blockDim.x) {
      const int r = i / (EPT + 2), c = i - r * (EPT + 2);
      const int x = x0 + r;
      float2 cur = S[r + 1][c];
      float2 res = cur;
      if (x < X) {
        const float w = p.sa_wx[x];
        if (w != 0.f) {
          float2 d;
          if (x == 0) d = cscale(csub(S[r + 2][c], cur), p.sa_invdx);
          else if (x == X - 1) d = cscale(csub(cur, S[r][c]), p.sa_invdx);
          else d = cscale(csub(S[r + 2][c], S[r][c]), p.sa_inv2dx);
          const float2 cd = make_float2(cf * d.y, -cf * d.x);
          const float2 P = (x < X / 2) ? make_float2(0.5f * (cur.x + cd.x), 0.5f * (cur.y + cd.y))
                                       : make_float2(0.5f * (cur.x - cd.x), 0.5f * (cur.y - cd.y));
          res = make_float2(cur.x - st * w * P.x, cur.y - st * w * P.y);
        }
      }
      XS[r][c] = res;
    }
    __syncthreads();
  }
  // 3) y edges, screens, store
  for (int i = tid; i < EPT * EPT; i += blockDim.x) {
    const int r = i / EPT, c = i - r * EPT;
    const int x = x0 + r, y = y0 + c;
    if (x >= X || y >= Y) continue;
    float2 v;
    if (sa) {
      const float2 cur = XS[r][c + 1];
      v = cur;
      const float w = p.sa_wy[y];
      if (w != 0.f) {
        float2 d;
        if (y == 0) d = cscale(csub(XS[r][c + 2], cur), p.sa_invdy);
        else if (y == Y - 1) d = cscale(csub(cur, XS[r][c]), p.sa_invdy);
        else d = cscale(csub(XS[r][c + 2], XS[r][c]), p.sa_inv2dy);
        const float2 cd = make_float2(cf * d.y, -cf * d.x);
        const float2 P = (y < Y / 2) ? make_float2(0.5f * (cur.x + cd.x), 0.5f * (cur.y + cd.y))
                                     : make_float2(0.5f * (cur.x - cd.x), 0.5f * (cur.y - cd.y));
        v = make_float2(cur.x - st * w * P.x, cur.y - st * w * P.y);
      }
      if (realify) v.y = 0.f;
    } else {
      v = S[r + 1][c + 1];
    }
    for (int k = 0; k < p.nscreens; ++k) {
      const float fs = p.screen_fscale[plane];
      const ScreenDev sc = p.screens[k];
      const size_t g = (size_t)x * Y + y;
      float sn, cs;
      sincosf(sc.phase[g] * fs, &sn, &cs);
      v = cmul(v, make_float2(cs, -sn));
      if (sc.amp != nullptr) {
        const float a = fminf(fmaxf(sc.amp[g], 1e-6f), 1.0f);
        v = cscale(v, exp2f(fs * log2f(a)));
      }
      if (realify) v.y = 0.f;
    }
    dp[(size_t)x * Y + y] = v;
  }
}

int asg_launch_epilogue_pass(const XYParams& p, const float2* src, float2* dst, int split,
                             cudaStream_t st) {
  const int tiles = ((p.X + EPT - 1) / EPT) * ((p.Y + EPT - 1) / EPT);
  xy_epilogue_pass<<<dim3(tiles, p.nplanes, 1), 256, 0, st>>>(p, src, dst, split);
  return cudaPeekAtLastError() == cudaSuccess ? ASG_OK : ASG_ERR_CUDA;
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
bool asg_xy_fast_supported(int X, int Y, int* G_out) {
  if (X % 32 != 0) return false;
  const int G = X / 32;
  if (!(G == 1 || G == 2 || G == 3 || G == 4 || G == 6 || G == 8 || G == 12 || G == 16))
    return false;
  switch (Y) {
    case 64: case 96: case 128: case 192: case 256: case 384: case 512: break;
    default: return false;
  }
  if (G_out) *G_out = G;
  return true;
}

bool asg_xy_split_supported(int X, int Y, int* G_out) {
  if (X % 32 != 0) return false;
  const int G = X / 32;  // half-plane of X/2 rows, 16 rows per CTA
  if (!(G == 1 || G == 2 || G == 3 || G == 4 || G == 6 || G == 8 || G == 12 || G == 16))
    return false;
  switch (Y) {
    case 128: case 192: case 256: case 384: case 512: break;
    default: return false;
  }
  if (G_out) *G_out = G;
  return true;
}

size_t asg_xy_generic_smem(int X, int Y) {
  return (size_t)(2 * X * Y + X + Y) * sizeof(float2) + (size_t)(X + Y) * sizeof(int);
}

template <int Yn, int R>
static int launch_fast_xy(const XYParams& p, cudaStream_t st) {
  using PY = FastPlan<Yn>;
  constexpr int NT = (R == 32 && Yn >= 256) ? 512 : 256;
  const size_t smem = (size_t)(R * PY::PADDED + 2 * PY::PADDED + Yn + 512) * sizeof(float2) +
                      (size_t)(Yn + 2 * R) * sizeof(int);
  static int max_clusters_dev[ASG_MAX_DEVICES], cached_G_dev[ASG_MAX_DEVICES];
  static bool init_dev[ASG_MAX_DEVICES] = {};
  const int dev = asg_device_slot();
  int& max_clusters = max_clusters_dev[dev];
  int& cached_G = cached_G_dev[dev];
  if (!init_dev[dev]) {
    max_clusters = -1;
    cached_G = -1;
    init_dev[dev] = true;
  }
  auto kern = xy_fast<PY, R, NT>;
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = p.G;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.blockDim = dim3(NT, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (max_clusters < 0 || cached_G != p.G) {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
      return ASG_ERR_CUDA;
    cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    cfg.gridDim = dim3(p.G * 1024, 1, 1);
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, kern, &cfg) != cudaSuccess || n <= 0) n = 1;
    max_clusters = n;
    cached_G = p.G;
  }
  const int nq = p.nplanes * p.nsub;
  const int ncl = max_clusters < nq ? max_clusters : nq;
  cfg.gridDim = dim3(p.G * ncl, 1, 1);
  cudaError_t e = cudaLaunchKernelEx(&cfg, kern, p);
  return e == cudaSuccess ? ASG_OK : ASG_ERR_CUDA;
}

int asg_launch_xy(const XYParams& p, bool fast, const GenPlan& plx, const GenPlan& ply,
                  cudaStream_t st) {
  if (fast) {
    const int R = p.X / p.nsub / p.G;
    if (R == 32) {
      switch (p.Y) {
        case 64: return launch_fast_xy<64, 32>(p, st);
        case 96: return launch_fast_xy<96, 32>(p, st);
        case 128: return launch_fast_xy<128, 32>(p, st);
        case 192: return launch_fast_xy<192, 32>(p, st);
        case 256: return launch_fast_xy<256, 32>(p, st);
        case 384: return launch_fast_xy<384, 32>(p, st);
        case 512: return launch_fast_xy<512, 32>(p, st);
        default: return ASG_ERR_SHAPE;
      }
    }
    if (R == 16) {
      switch (p.Y) {
        case 128: return launch_fast_xy<128, 16>(p, st);
        case 192: return launch_fast_xy<192, 16>(p, st);
        case 256: return launch_fast_xy<256, 16>(p, st);
        case 384: return launch_fast_xy<384, 16>(p, st);
        case 512: return launch_fast_xy<512, 16>(p, st);
        default: return ASG_ERR_SHAPE;
      }
    }
    return ASG_ERR_SHAPE;
  }
  const size_t smem = asg_xy_generic_smem(p.X, p.Y);
  if (smem > ASG_XY_GENERIC_MAX_SMEM) return launch_xy_big(p, plx, ply, st);
  if (cudaFuncSetAttribute(xy_generic, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return ASG_ERR_CUDA;
  xy_generic<<<dim3(1, p.nplanes, 1), 256, smem, st>>>(p, plx, ply);
  return cudaPeekAtLastError() == cudaSuccess ? ASG_OK : ASG_ERR_CUDA;
}
