// Per-(x,y)-column work along t, executed by one warp per column on a
// column held in shared memory: boundary taper, Burgers step (Rusanov,
// TVD-Rusanov, KT-MC, KT-minmod; SSP-RK2; optional per-column CFL
// sub-cycling), source-plane injection and the per-step accumulators.
//
// Reference semantics (angular_spectrum_solver.py):
//   taper                 :125-129, :655   (u * abl, separable x*y*t)
//   _rusanov_flux_standard :688-696
//   _rusanov_flux_tvd      :699-724
//   _kt_rhs/_kt_rhs_minmod :758-830,  _kt_flux/_kt_flux_minmod :833-868
//   _kt_flux_adaptive      :842-859  (here per column, see below)
//   source injection      :1521-1527
//   accumulators          :1445, :1529-1535
#pragma once
#include "asg_common.cuh"

enum FluxKind : int {
  FLUX_NONE = 0,
  FLUX_RUSANOV = 1,      // _rusanov_flux_standard
  FLUX_RUSANOV_TVD = 2,  // _rusanov_flux_tvd
  FLUX_KT_MC = 3,        // _kt_flux
  FLUX_KT_MINMOD = 4,    // _kt_flux_minmod
};

struct SourceEvent {
  const int* map;     // [ncols] -> row in val, or -1
  const float* val;   // [nactive][nT]
};

// Everything the column phase needs (plain POD, passed by value inside the
// kernel parameter block).
struct ColumnOps {
  // taper: u *= abl_xy[c] * abl_t[t]   (null abl_xy -> no taper)
  const float* abl_xy;
  const float* abl_t;
  // Burgers
  int flux;
  // coefficients rounded once from FP64 on the host, as the reference's
  // float32 arrays see its float64 scalars: coef_rus = N dZ/dT, coef_kt = N/dT
  float coef_rus, coef_kt;
  const double* n_scale; // optional device pair (sum P k/kz, sum P) for <k/kz>, or null
  double n_rus64, n_kt64;  // the same coefficients in FP64 (used with n_scale)
  float dz, beta_tvd;
  float cfl_target;      // > 0: per-column sub-cycling for the KT schemes
  int max_subcycles;     // bound on the per-column sub-cycle count
  // sources (step end)
  int nsrc;
  const SourceEvent* src;
  // accumulators (step end); step index read from *step
  int accumulate;
  const int* step;
  float *pnp, *ppp, *pI, *pIloss;  // [step][ncols]
  float* pax;                       // [step][nT]
  int pax_col;
  int ncols;
  double* iprev;                    // [ncols]
  unsigned* max_next;               // stability max of the field entering the next step
  unsigned* subcycle_hist;          // optional [64] histogram of per-column sub-cycles
  unsigned* subcycle_clamp;         // optional [2]: columns whose sub-cycle count was capped at
                                    // max_subcycles, and the largest count one of them needed
  int init_stats;                   // first upload: only iprev / max_next
};

// Column accessor over shared memory: real samples t = 0..nT-1.
// Fast layout: complex slots with one pad every N2 slots (LinePlan::pos).
template <int N2>
struct PaddedColumn {
  float* base;
  ASG_DEV int idx(int t) const { int j = t >> 1; return 2 * (j + 2 * (j / N2)) + (t & 1); }
  ASG_DEV float get(int t) const { return base[idx(t)]; }
  ASG_DEV void set(int t, float v) const { base[idx(t)] = v; }
  // Runs of CH samples starting at multiples of CH lie inside one padded row
  // (2 N2 samples) and start on a 16-byte boundary (the rows and their pads
  // are multiples of four floats): such a run is a contiguous float4 array.
  template <int CH>
  static constexpr bool kVecRun = (2 * N2) % CH == 0 && CH % 4 == 0;
  ASG_DEV float4* run4(int t0) const { return reinterpret_cast<float4*>(base + idx(t0)); }
};
struct PlainColumn {
  float* base;
  ASG_DEV float get(int t) const { return base[t]; }
  ASG_DEV void set(int t, float v) const { base[t] = v; }
  template <int CH>
  static constexpr bool kVecRun = false;
  ASG_DEV float4* run4(int t0) const { return reinterpret_cast<float4*>(base + t0); }
};
// Skewed copy of a column for the chunked KT step (lane l owns samples
// 32l .. 32l+31): one pad word per 32 samples puts the 32 lanes' i-th samples
// in 32 different shared-memory banks.  Holds nT + nT/32 floats.
struct SkewColumn {
  float* base;
  ASG_DEV int idx(int t) const { return t + (t >> 5); }
  ASG_DEV float get(int t) const { return base[idx(t)]; }
  ASG_DEV void set(int t, float v) const { base[idx(t)] = v; }
};
__host__ __device__ constexpr int skew_floats(int nT) { return nT + nT / 32 + 4; }

// ---------------------------------------------------------------------------
// flux primitives (float32, same formulas and order as the reference)
// ---------------------------------------------------------------------------
ASG_DEV float sgnf(float x) { return x > 0.f ? 1.f : (x < 0.f ? -1.f : 0.f); }

// interface flux of _rusanov_flux_standard (:691-694)
ASG_DEV float rus_std_fh(float uL, float uR) {
  float a = fmaxf(fabsf(uL), fabsf(uR));
  return -(uL * uL + uR * uR) / 2.f - a * (uR - uL);
}
// interface flux of _rusanov_flux_tvd (:702-705)
ASG_DEV float rus_tvd_fh(float uL, float uR) {
  float a = fmaxf(fabsf(uL), fabsf(uR));
  return 0.5f * (-0.5f * (uL * uL + uR * uR)) - 0.5f * a * (uR - uL);
}
ASG_DEV float tvd_phi(float r, float b) {
  return fmaxf(0.f, fminf(fminf(b * r, 1.f), fminf(r, b)));
}
ASG_DEV float minmod2(float a, float b) {
  return (a * b > 0.f) ? sgnf(a) * fminf(fabsf(a), fabsf(b)) : 0.f;
}
ASG_DEV float minmod3(float a, float b, float c) {
  bool ok = (a * b > 0.f) && (b * c > 0.f);
  return ok ? sgnf(a) * fminf(fminf(fabsf(a), fabsf(b)), fabsf(c)) : 0.f;
}
// limited slope at a cell given its left/right neighbours (MC or minmod).
// MC: minmod3(2 dm, (dm + dp)/2, 2 dp) = sign(dm) 2 min(|dm|, |dm + dp|/4, |dp|)
// when dm dp > 0 (then all three arguments share the sign), else 0; the
// power-of-two scalings are exact, so this is the same number with fewer
// operations.
template <bool MC>
ASG_DEV float kt_slope(float um1, float u0, float up1) {
  const float dm = u0 - um1, dp = up1 - u0;
  const float m = MC ? 2.f * fminf(fminf(fabsf(dm), fabsf(dp)), 0.25f * fabsf(dm + dp))
                     : fminf(fabsf(dm), fabsf(dp));
  return (dm * dp > 0.f) ? copysignf(m, dm) : 0.f;
}
// KT interface flux from the reconstructed states (:772-793), for Burgers'
// flux f(u) = -u^2/2, whose speeds are a = -u.  With aL = -um, aR = -up the
// reference forms ap = max(aL, aR, 0), am = min(aL, aR, 0) and divides
// (ap fm - am fp - ap am (up - um)) / (ap - am); for this flux the quotient is
// a polynomial in each sign case (exact algebra, no division):
//   um, up <= 0 (both speeds >= 0):            fm = -um^2/2
//   um, up >= 0 (both speeds <= 0):            fp = -up^2/2
//   um < 0 < up (aL > 0 > aR):  (-um^3/2 + ... )/(aL - aR) = -(um^2 + 3 um up + up^2)/2
//   um > 0 > up (aL < 0 < aR):                            =  3/2 um up
// The reference's Lax-Friedrichs branch (ap - am < 1e-14) differs from these
// only where |um| and |up| are below 1e-14, where both fluxes are below 1e-28.
ASG_DEV float kt_fh(float um, float up) {
  const float q = um * up;
  const float m2 = um * um, p2 = up * up;
  const float same = -0.5f * ((um + up <= 0.f) ? m2 : p2);
  const float q15 = 1.5f * q;  // -1.5f * q is -(1.5f * q) exactly
  const float mixed = (um < 0.f) ? fmaf(-0.5f, m2 + p2, -q15) : q15;
  return (q >= 0.f) ? same : mixed;
}
// Half the limited slope: every KT reconstruction uses u +/- slope/2.  The
// MC slope is 2 min(...) and the halving undoes the doubling exactly (power
// of two scalings are exact), so u + kt_half_slope() equals u + 0.5f * kt_slope()
// bit for bit, with one multiplication less.
template <bool MC>
ASG_DEV float kt_half_slope(float um1, float u0, float up1) {
  const float dm = u0 - um1, dp = up1 - u0;
  const float m = MC ? fminf(fminf(fabsf(dm), fabsf(dp)), 0.25f * fabsf(dm + dp))
                     : 0.5f * fminf(fabsf(dm), fabsf(dp));
  return (dm * dp > 0.f) ? copysignf(m, dm) : 0.f;
}

// ---------------------------------------------------------------------------
// Burgers step on one column by one warp, 32 samples t = t0 + lane at a time.
// Stencil neighbours come from warp shuffles; across the 32-sample blocks the
// original values / interface fluxes are carried in registers, so the update
// runs in place in shared memory with a handful of registers.  The column
// end points t=0 and t=nT-1 are never updated (zero boundary rhs).
// ---------------------------------------------------------------------------
template <class Col>
ASG_DEV void rusanov_column(const Col& col, int nT, float coef, bool tvd, float beta_tvd,
                            unsigned mask) {
  const int lane = threadIdx.x & 31;
  float carry = 0.f;  // original u[t0-1]
  for (int t0 = 0; t0 < nT; t0 += 32) {
    const int t = t0 + lane;
    const float u = (t < nT) ? col.get(t) : 0.f;
    float um = __shfl_up_sync(mask, u, 1);
    float up = __shfl_down_sync(mask, u, 1);
    if (lane == 0) um = carry;
    if (lane == 31) up = (t + 1 < nT) ? col.get(t + 1) : 0.f;
    float out = u;
    if (t >= 1 && t < nT - 1) {
      if (!tvd) {
        const float fd = rus_std_fh(u, up) - rus_std_fh(um, u);
        out = u + (-coef * fd);
      } else {
        const float fd = rus_tvd_fh(u, up) - rus_tvd_fh(um, u);
        const float dm = u - um, dp = up - u;
        const float eps = 1e-30f;
        const float r = dp / (dm + eps * sgnf(dm + eps));
        const float ri = dm / (dp + eps * sgnf(dp + eps));
        out = u + (-coef * (0.5f * (tvd_phi(r, beta_tvd) + tvd_phi(ri, beta_tvd)) * fd));
      }
    }
    carry = __shfl_sync(mask, u, 31);
    __syncwarp(mask);
    if (t < nT) col.set(t, out);
  }
  __syncwarp(mask);
}

// rhs of the KT scheme (MUSCL slopes, KT interface fluxes) at t = t0+lane,
// reading src; fh_carry holds the flux at t0-1/2 from the previous block.
template <bool MC, class Col>
ASG_DEV float kt_rhs_lane(const Col& src, int t, int nT, float ndt, float& fh_carry,
                          float& u_out, unsigned mask) {
  const int lane = threadIdx.x & 31;
  const float u0 = (t < nT) ? src.get(t) : 0.f;
  float um1 = __shfl_up_sync(mask, u0, 1);
  float up1 = __shfl_down_sync(mask, u0, 1);
  if (lane == 0) um1 = (t >= 1) ? src.get(t - 1) : 0.f;
  if (lane == 31) up1 = (t + 1 < nT) ? src.get(t + 1) : 0.f;
  const float sg = (t >= 1 && t < nT - 1) ? kt_slope<MC>(um1, u0, up1) : 0.f;
  float sn = __shfl_down_sync(mask, sg, 1);
  if (lane == 31) {
    const float up2 = (t + 2 < nT) ? src.get(t + 2) : 0.f;
    sn = (t + 1 >= 1 && t + 1 < nT - 1) ? kt_slope<MC>(u0, up1, up2) : 0.f;
  }
  // interface t+1/2
  const float fh = kt_fh(u0 + 0.5f * sg, up1 - 0.5f * sn);
  float fp = __shfl_up_sync(mask, fh, 1);
  if (lane == 0) fp = fh_carry;
  fh_carry = __shfl_sync(mask, fh, 31);
  u_out = u0;
  return (t >= 1 && t < nT - 1) ? (-ndt * (fh - fp)) : 0.f;
}

// one SSP-RK2 KT step of size dz; stage-1 values go to `stg`
template <bool MC, class Col>
ASG_DEV void kt_column_step(const Col& col, const Col& stg, int nT, float ndt, float dz,
                            unsigned mask) {
  const int lane = threadIdx.x & 31;
  float carry = 0.f;
  for (int t0 = 0; t0 < nT; t0 += 32) {
    const int t = t0 + lane;
    float u;
    const float r = kt_rhs_lane<MC>(col, t, nT, ndt, carry, u, mask);
    if (t < nT) stg.set(t, u + dz * r);
  }
  __syncwarp(mask);
  carry = 0.f;
  for (int t0 = 0; t0 < nT; t0 += 32) {
    const int t = t0 + lane;
    float s1;
    const float r = kt_rhs_lane<MC>(stg, t, nT, ndt, carry, s1, mask);
    if (t < nT) col.set(t, 0.5f * col.get(t) + 0.5f * (s1 + dz * r));
  }
  __syncwarp(mask);
}

// Chunked variant of the KT step: lane l owns samples [l*CH, (l+1)*CH) and keeps
// its window, stage-1 values and right-hand sides in registers (faster when
// CH <= 32; the shuffle variant above is used for longer columns).
// rhs of the KT scheme at the lane's CH points from a window of CH+4 values
template <int CH, bool MC>
ASG_DEV void kt_rhs_window(const float (&w)[CH + 4], int t0, int nT, float ndt, float (&rhs)[CH]) {
  // slopes at window positions 1..CH+2  (t0-1 .. t0+CH); zero at the column ends
  float s[CH + 2];
#pragma unroll
  for (int i = 0; i < CH + 2; ++i) {
    int t = t0 - 1 + i;
    s[i] = (t >= 1 && t < nT - 1) ? kt_slope<MC>(w[i], w[i + 1], w[i + 2]) : 0.f;
  }
  // interface fluxes at t+1/2 for t = t0-1 .. t0+CH-1
  float fh[CH + 1];
#pragma unroll
  for (int i = 0; i < CH + 1; ++i) {
    float um = w[i + 1] + 0.5f * s[i];
    float up = w[i + 2] - 0.5f * s[i + 1];
    fh[i] = kt_fh(um, up);
  }
#pragma unroll
  for (int i = 0; i < CH; ++i) {
    int t = t0 + i;
    rhs[i] = (t >= 1 && t < nT - 1) ? (-ndt * (fh[i + 1] - fh[i])) : 0.f;
  }
}

template <int CH, bool MC, class Col>
ASG_DEV void load_window4(const Col& col, int t0, int nT, float (&w)[CH + 4]) {
#pragma unroll
  for (int i = 0; i < CH + 4; ++i) {
    int t = t0 - 2 + i;
    w[i] = (t >= 0 && t < nT) ? col.get(t) : 0.f;
  }
}

// Column length exactly 32 CH: only the first lane's two leading and the last
// lane's two trailing window values lie outside the column, and only their
// slopes and end-sample rhs need zeroing, so the per-point range tests go.
template <int CH, class Col>
ASG_DEV void load_window4_exact(const Col& col, int t0, int lane, float (&w)[CH + 4]) {
  const bool first = lane != 0, last = lane != 31;
  w[0] = first ? col.get(t0 > 2 ? t0 - 2 : 0) : 0.f;
  w[1] = first ? col.get(t0 > 1 ? t0 - 1 : 0) : 0.f;
#pragma unroll
  for (int i = 2; i < CH + 2; ++i) w[i] = col.get(t0 - 2 + i);
  w[CH + 2] = last ? col.get(last ? t0 + CH : t0) : 0.f;
  w[CH + 3] = last ? col.get(last ? t0 + CH + 1 : t0) : 0.f;
}

// One stage of the exact-length KT step, streamed along the lane's window:
// slopes, interface fluxes and the update are formed point by point (only
// the previous slope and flux stay live), and each updated value is written
// as soon as it is known (every lane has its window in registers by then):
//   stage 1: col[t] = u[t] + dz rhs(w)
//   stage 2: col[t] = u[t]/2 + (w[t] + dz rhs(w))/2
template <int CH, bool MC, bool STAGE2, class Col>
ASG_DEV void kt_stage_exact(const Col& col, const float (&w)[CH + 4], const float (&u)[CH],
                            int t0, int lane, float ndt, float dz) {
  const bool first = lane != 0, last = lane != 31;
  // slope at window position i+1 (t = t0 - 1 + i); zero at the column ends
  auto slope = [&](int i) {
    const float v = kt_slope<MC>(w[i], w[i + 1], w[i + 2]);
    if (i <= 1) return first ? v : 0.f;
    if (i >= CH) return last ? v : 0.f;
    return v;
  };
  float sl = slope(0), sr = slope(1);
  float fprev = kt_fh(w[1] + 0.5f * sl, w[2] - 0.5f * sr);  // interface t0 - 1/2
#pragma unroll
  for (int i = 0; i < CH; ++i) {
    sl = sr;
    sr = slope(i + 2);
    const float f = kt_fh(w[i + 2] + 0.5f * sl, w[i + 3] - 0.5f * sr);  // t0 + i + 1/2
    float rhs = -ndt * (f - fprev);
    if (i == 0) rhs = first ? rhs : 0.f;
    if (i == CH - 1) rhs = last ? rhs : 0.f;
    fprev = f;
    if (STAGE2) col.set(t0 + i, 0.5f * u[i] + 0.5f * (w[i + 2] + dz * rhs));
    else col.set(t0 + i, u[i] + dz * rhs);
  }
}

// one SSP-RK2 KT step of size dz on the column
template <int CH, bool MC, class Col>
ASG_DEV void kt_column_step_chunk(const Col& col, int nT, float ndt, float dz, unsigned mask) {
  const int lane = threadIdx.x & 31;
  const int t0 = lane * CH;
  if (nT == 32 * CH && CH >= 2) {  // uniform across the warp
    float w[CH + 4], u[CH];
    load_window4_exact<CH>(col, t0, lane, w);
#pragma unroll
    for (int i = 0; i < CH; ++i) u[i] = w[i + 2];
    __syncwarp(mask);  // every window is read before any lane writes
    kt_stage_exact<CH, MC, false>(col, w, u, t0, lane, ndt, dz);
    __syncwarp(mask);
    load_window4_exact<CH>(col, t0, lane, w);
    __syncwarp(mask);
    kt_stage_exact<CH, MC, true>(col, w, u, t0, lane, ndt, dz);
    __syncwarp(mask);
    return;
  }
  float w[CH + 4];
  load_window4<CH, MC>(col, t0, nT, w);
  float u[CH], rhs[CH];
#pragma unroll
  for (int i = 0; i < CH; ++i) u[i] = w[i + 2];
  kt_rhs_window<CH, MC>(w, t0, nT, ndt, rhs);
  __syncwarp(mask);
#pragma unroll
  for (int i = 0; i < CH; ++i) {
    int t = t0 + i;
    if (t < nT) col.set(t, u[i] + dz * rhs[i]);  // stage1
  }
  __syncwarp(mask);
  load_window4<CH, MC>(col, t0, nT, w);
  kt_rhs_window<CH, MC>(w, t0, nT, ndt, rhs);
  __syncwarp(mask);
#pragma unroll
  for (int i = 0; i < CH; ++i) {
    int t = t0 + i;
    float s1 = w[i + 2];
    if (t < nT) col.set(t, 0.5f * u[i] + 0.5f * (s1 + dz * rhs[i]));
  }
  __syncwarp(mask);
}

// One SSP-RK2 KT step of size dz in a single streaming pass, in place, for a
// column of exactly nT = 32 CH samples (CH >= 4); lane l owns samples
// [l CH, (l+1) CH).  Stage 2 at t needs stage-1 values s1 at t-2..t+2, which
// need u at t-4..t+4, so each lane walks its run once with sliding windows:
// iteration t loads u[t+4], forms the slope at t+3, the flux at t+5/2 and
// s1[t+2], then the slope of s1 at t+1, its flux at t+1/2 and the new u[t].
// About 25 values stay live instead of the whole run.  The four samples on
// either side of a run come from the neighbouring lanes by shuffles before
// any write (every later read is of the lane's own, not yet written,
// samples); the lane recomputes s1 at t0-2, t0-1 (a short prologue).  The
// column ends t = 0 and nT-1 keep zero slope and zero rhs, as in the reference
// (:758-839).
//
// When the lane's run is a contiguous, 16-byte aligned float4 array
// (Col::kVecRun), it is read and written four samples at a time: the 32
// lanes' runs start in only 8 distinct shared-memory banks, so scalar accesses
// cost four wavefronts each, while a warp's float4 access is 4 wavefronts for
// four samples.  The arithmetic is the same.
template <int CH, bool MC, class Col>
ASG_DEV void kt_step_stream(const Col& col, float ndt, float dz, unsigned mask) {
  static_assert(CH >= 4, "four halo samples per side");
  constexpr bool VEC = Col::template kVecRun<CH>;
  const int lane = threadIdx.x & 31;
  const int t0 = lane * CH;
  const bool nf = lane != 0, nl = lane != 31;  // run not at the column start / end
  const float c = -ndt * dz;
  // sl gives half slopes (kt_half_slope): the reconstructions are u +/- sl(...)
  auto sl = [](float a, float b, float d) { return kt_half_slope<MC>(a, b, d); };
  float4* run = VEC ? col.run4(t0) : nullptr;
  float a0, a1, a2, a3, z0, z1, z2, z3;
  if constexpr (VEC) {
    const float4 h = run[0], e = run[CH / 4 - 1];
    a0 = h.x; a1 = h.y; a2 = h.z; a3 = h.w;
    z0 = e.x; z1 = e.y; z2 = e.z; z3 = e.w;
  } else {
    a0 = col.get(t0); a1 = col.get(t0 + 1); a2 = col.get(t0 + 2); a3 = col.get(t0 + 3);
    z0 = col.get(t0 + CH - 4); z1 = col.get(t0 + CH - 3); z2 = col.get(t0 + CH - 2);
    z3 = col.get(t0 + CH - 1);
  }
  float hm4 = __shfl_up_sync(mask, z0, 1), hm3 = __shfl_up_sync(mask, z1, 1);
  float hm2 = __shfl_up_sync(mask, z2, 1), hm1 = __shfl_up_sync(mask, z3, 1);
  float hp[4] = {__shfl_down_sync(mask, a0, 1), __shfl_down_sync(mask, a1, 1),
                 __shfl_down_sync(mask, a2, 1), __shfl_down_sync(mask, a3, 1)};
  if (!nf) hm4 = hm3 = hm2 = hm1 = 0.f;
  if (!nl) hp[0] = hp[1] = hp[2] = hp[3] = 0.f;
  // prologue: slopes at t0-3 .. t0+2, fluxes at t0-5/2 .. t0+3/2, s1 at t0-2 .. t0+1
  const float sm3 = nf ? sl(hm4, hm3, hm2) : 0.f, sm2 = nf ? sl(hm3, hm2, hm1) : 0.f;
  const float sm1 = nf ? sl(hm2, hm1, a0) : 0.f, s0 = nf ? sl(hm1, a0, a1) : 0.f;
  float sA = sl(a0, a1, a2), sB = sl(a1, a2, a3);  // slopes at t+1, t+2
  const float fm25 = kt_fh(hm3 + sm3, hm2 - sm2);
  const float fm15 = kt_fh(hm2 + sm2, hm1 - sm1);
  const float fm05 = kt_fh(hm1 + sm1, a0 - s0);
  const float fp05 = kt_fh(a0 + s0, a1 - sA);
  float F = kt_fh(a1 + sA, a2 - sB);  // flux at t+3/2
  const float r_m2 = hm2 + c * (fm15 - fm25);
  const float r_m1 = hm1 + c * (fm05 - fm15);
  float r0 = nf ? a0 + c * (fp05 - fm05) : a0;  // s1[t]
  float r1 = a1 + c * (F - fp05);               // s1[t+1]
  const float qm1 = nf ? sl(r_m2, r_m1, r0) : 0.f;
  float q0 = nf ? sl(r_m1, r0, r1) : 0.f;        // slope of s1 at t
  float G = kt_fh(r_m1 + qm1, r0 - q0);  // flux of s1 at t-1/2
  float w0 = a0, w1 = a1, w2 = a2, w3 = a3;      // u[t .. t+3]
  // VEC: one float4 holds the chunk of samples 4q+4 .. 4q+7 (read at i = 4q)
  // and, component by component as each is used, the new samples 4q .. 4q+3
  // (written back at i = 4q+3)
  float4 ahead = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int i = 0; i < CH; ++i) {
    const int t = t0 + i;
    float u4;
    if constexpr (VEC) {
      // the chunk i+4 .. i+7 is read before any of it is written (writes reach
      // sample i at most)
      if ((i & 3) == 0 && i + 4 < CH) ahead = run[i / 4 + 1];
      const int k = i & 3;
      u4 = (i + 4 < CH) ? (k == 0 ? ahead.x : k == 1 ? ahead.y : k == 2 ? ahead.z : ahead.w)
                        : hp[(i + 4 - CH) & 3];
    } else {
      u4 = (i + 4 < CH) ? col.get(t + 4) : hp[(i + 4 - CH) & 3];
    }
    float sC = sl(w2, w3, u4);                    // slope at t+3
    if (i >= CH - 4 && !nl) sC = 0.f;             // t+3 >= nT-1
    const float F2 = kt_fh(w2 + sB, w3 - sC);  // flux at t+5/2
    float r2 = w2 + c * (F2 - F);                 // s1[t+2]
    if (i >= CH - 3 && !nl) r2 = w2;              // t+2 >= nT-1 (zero outside)
    float q1 = sl(r0, r1, r2);                    // slope of s1 at t+1
    if (i >= CH - 2 && !nl) q1 = 0.f;
    const float G1 = kt_fh(r0 + q0, r1 - q1);  // flux of s1 at t+1/2
    float out = 0.5f * (w0 + (r0 + c * (G1 - G)));  // = w0/2 + (...)/2: the halvings are exact
    if ((i == 0 && !nf) || (i == CH - 1 && !nl)) out = w0;    // column ends
    if constexpr (VEC) {
      const int k = i & 3;
      if (k == 0) ahead.x = out;
      else if (k == 1) ahead.y = out;
      else if (k == 2) ahead.z = out;
      else ahead.w = out;
      if (k == 3) run[i / 4] = ahead;
    } else {
      col.set(t, out);
    }
    w0 = w1; w1 = w2; w2 = w3; w3 = u4;
    sA = sB; sB = sC; F = F2;
    r0 = r1; r1 = r2; q0 = q1; G = G1;
  }
  __syncwarp(mask);
}

template <class Col>
ASG_DEV float column_absmax(const Col& col, int nT) {
  const int lane = threadIdx.x & 31;
  float m = 0.f;
  for (int t = lane; t < nT; t += 32) m = fmaxf(m, fabsf(col.get(t)));
  return warp_max(m);
}

// ---------------------------------------------------------------------------
// The whole column phase.  CH = ceil(nT/32) samples per lane.
// ---------------------------------------------------------------------------
// STREAM: the column holds exactly nT = 32 CH samples (CH >= 4) and the KT
// sub-steps stream along it in place (kt_step_stream).
template <int CH, bool STREAM = false, class Col>
ASG_DEV float column_phase(const Col& col, const Col& stg, int c, int nT, const ColumnOps& op,
                           bool write_stats) {
  const int lane = threadIdx.x & 31;
  const unsigned mask = 0xffffffffu;
  // 1) taper
  if (op.abl_xy != nullptr) {
    const float axy = op.abl_xy[c];
#pragma unroll
    for (int i = 0; i < CH; ++i) {
      int t = lane + 32 * i;
      if (t < nT) col.set(t, col.get(t) * (axy * op.abl_t[t]));
    }
    __syncwarp(mask);
  }
  // 2) Burgers
  if (op.flux != FLUX_NONE) {
    float coef_rus = op.coef_rus, ndt = op.coef_kt;
    if (op.n_scale != nullptr) {
      // n_scale = {sum P k/kz, sum P over propagating modes}: <k/kz> (:641-643)
      const double sc = op.n_scale[0] / (op.n_scale[1] + 1e-30);
      coef_rus = (float)(op.n_rus64 * sc);
      ndt = (float)(op.n_kt64 * sc);
    }
    if (op.flux == FLUX_RUSANOV || op.flux == FLUX_RUSANOV_TVD) {
      rusanov_column(col, nT, coef_rus, op.flux == FLUX_RUSANOV_TVD, op.beta_tvd, mask);
    } else {
      int nsub = 1;
      if (op.cfl_target > 0.f) {
        const float um = column_absmax(col, nT);
        float cfl = ndt * um * op.dz;
        if (!(cfl <= op.cfl_target || um < 1e-30f)) {
          float q = ceilf(cfl / op.cfl_target);
          nsub = (q > (float)op.max_subcycles) ? op.max_subcycles : (int)q;
          // a capped column runs above its CFL target: counted for the host
          if (q > (float)op.max_subcycles && op.subcycle_clamp != nullptr && lane == 0) {
            atomicAdd(op.subcycle_clamp, 1u);
            atomicMax(op.subcycle_clamp + 1, q < 4.0e9f ? (unsigned)q : 0xffffffffu);
          }
        }
        if (op.subcycle_hist != nullptr && lane == 0)
          atomicAdd(op.subcycle_hist + min(nsub, 63), 1u);
      }
      const float dzs = op.dz / (float)nsub;
      for (int k = 0; k < nsub; ++k) {
        if constexpr (STREAM) {
          static_assert(CH >= 4 && CH <= 64, "streamed KT: 128 to 2048 samples");
          if (op.flux == FLUX_KT_MC) kt_step_stream<CH, true>(col, ndt, dzs, mask);
          else kt_step_stream<CH, false>(col, ndt, dzs, mask);
        } else if constexpr (CH <= 32) {
          if (op.flux == FLUX_KT_MC) kt_column_step_chunk<CH, true>(col, nT, ndt, dzs, mask);
          else kt_column_step_chunk<CH, false>(col, nT, ndt, dzs, mask);
        } else {
          if (op.flux == FLUX_KT_MC) kt_column_step<true>(col, stg, nT, ndt, dzs, mask);
          else kt_column_step<false>(col, stg, nT, ndt, dzs, mask);
        }
      }
    }
  }
  // 3) sources, in list order
  for (int e = 0; e < op.nsrc; ++e) {
    int row = op.src[e].map[c];
    if (row >= 0) {
      const float* v = op.src[e].val + (size_t)row * nT;
#pragma unroll
      for (int i = 0; i < CH; ++i) {
        int t = lane + 32 * i;
        if (t < nT) col.set(t, col.get(t) + v[t]);
      }
    }
    __syncwarp(mask);
  }
  // 4) accumulators (pI/pIloss sums in FP64 across lanes); returns max|u|
  //    (NaN/inf if the column holds a non-finite value) for the stability test
  float am = 0.f;
  if (write_stats) {
    float s = 0.f, mn = INFINITY, mx = -INFINITY;
    double sd = 0.0;
    bool bad = false;
#pragma unroll
    for (int i = 0; i < CH; ++i) {
      int t = lane + 32 * i;
      if (t < nT) {
        float u = col.get(t);
        s = fmaf(u, u, s);
        mn = fminf(mn, u);
        mx = fmaxf(mx, u);
        am = fmaxf(am, fabsf(u));
        bad |= !(fabsf(u) <= 3.402823466e38f);
        if ((i & 7) == 7) { sd += (double)s; s = 0.f; }
      }
    }
    sd += (double)s;
    sd = warp_sum(sd);
    mn = warp_min(mn);
    mx = warp_max(mx);
    am = warp_max(am);
    bad = __any_sync(mask, bad);
    if (bad) am = __uint_as_float(0x7fc00000u);
    if (lane == 0) {
      if (!op.init_stats) {
        const size_t o = (size_t)(*op.step) * (size_t)op.ncols + (size_t)c;
        const double ib = op.iprev[c];
        op.pIloss[o] = (float)fmax(0.0, ib - sd);
        op.pI[o] = (float)sd;
        op.pnp[o] = mn;
        op.ppp[o] = mx;
      }
      op.iprev[c] = sd;
    }
    if (c == op.pax_col && !op.init_stats) {
      float* pa = op.pax + (size_t)(*op.step) * (size_t)nT;
#pragma unroll
      for (int i = 0; i < CH; ++i) {
        int t = lane + 32 * i;
        if (t < nT) pa[t] = col.get(t);
      }
    }
  }
  return am;
}
