// Set-up kernels: FP64 construction of the per-mode multiplier tables, and
// the small bookkeeping kernels of the march.
//
// Multiplier of one mode (kx, ky, bin f), its phases and exponents in FP64:
//   propagator (precalculate_mas, angular_spectrum_solver.py:396-462)
//     kk < k^2 : mask(kk) * exp(i dz kk / (k + sqrt(k^2 - kk)))
//                (the cancellation-free form of exp(i dz (k - kz)), :441)
//     else     : mask(kk) * exp(-dz sqrt(kk - k^2)) * exp(i dz k)   (:440)
//     zero for bins 0 and nT/2 (:455), k = centred temporal grid value of the
//     bin (:403-404), mask = cosine k-filter sized from the full step (:410-433)
//   attenuation/KK (_build_oblique_atten_filter, :468-520)
//     kz^2 = km^2 - kk > 0 : exp(-(alpha + i alphaStar) dz s km / max(kz, km 1e-6))
//     otherwise 1; bin 0 -> 1; water model clips Re < 0 to 0 (:518-519)
// The tables are indexed by (plane, x-class, y-class): modes whose |kx|, |ky|
// coincide on the reference's symmetric centred grid share one entry.
#include <math.h>

#include "asg_internal.h"

// sin and cos of an FP64 angle: reduced to [-pi, pi] in FP64 by Cody and
// Waite's method (2 pi split into its nearest double and the remainder), then
// evaluated in FP32.  The angles here are below a few hundred radians, so the
// reduction error stays near 1e-14 rad; the FP32 evaluation adds about one
// FP32 ulp, the precision of the stored table entry.
__device__ __forceinline__ void sincos_reduced(double ph, float* s, float* c) {
  const double two_pi_hi = 6.283185307179586;      // nearest double to 2 pi
  const double two_pi_lo = 2.4492935982947064e-16;  // 2 pi - two_pi_hi
  const double n = rint(ph * 0.15915494309189535);  // ph / (2 pi), rounded
  double r = fma(-n, two_pi_hi, ph);
  r = fma(-n, two_pi_lo, r);
  sincosf((float)r, s, c);
}

// All multiplier tables of one step size in one pass: per mode the propagator
// factor P and the attenuation/KK factor A are formed once and written as
// out_pa = P A, out_p = P, out_a = A (any output may be null).  The phases,
// the wavenumbers and the exponents' arguments are FP64 (the propagator
// phase in the cancellation-free form); exp and sin/cos of them are taken in
// FP32 after an FP64 argument reduction; each entry is rounded to FP32 once
// from the FP64 product.
__global__ void k_build_table(TableParams p) {
  const size_t n = (size_t)p.nplanes * p.ncx * p.ncy;
  const double kstart2 = p.kstart * p.kstart, kmax2 = p.kmax_t * p.kmax_t;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int cy = (int)(i % p.ncy);
    const int cx = (int)((i / p.ncy) % p.ncx);
    const int pl = (int)(i / ((size_t)p.ncy * p.ncx));
    const int f = p.f_of_plane[pl];
    const double kk = p.kx2[cx] + p.ky2[cy];
    double pr = 1.0, pi = 0.0;
    if (p.use_prop) {
      if (f == 0 || 2 * f == p.nT) {
        pr = 0.0;
        pi = 0.0;
      } else {
        const double k = p.kt_prop[pl];
        double mask = 1.0;
        if (kk > kmax2) {
          mask = 0.0;
        } else if (kk > kstart2) {
          const double kr = sqrt(kk);
          if (kr > p.kmax_t) mask = 0.0;
          else if (kr > p.kstart)
            mask = 0.5 * (1.0 + (double)cosf((float)(M_PI * (kr - p.kstart) /
                                                      (p.kmax_t - p.kstart))));
        }
        if (mask != 0.0) {
          double amp, ph;
          if (kk < k * k) {
            amp = 1.0;
            ph = p.dz_prop * kk / (k + sqrt(k * k - kk));
          } else {
            amp = (double)expf((float)(-p.dz_prop * sqrt(kk - k * k)));
            ph = p.dz_prop * k;
          }
          float sn, cs;
          sincos_reduced(ph, &sn, &cs);
          // the reference's factor 2 on the kept bins is cancelled by the real
          // part it takes afterwards (Re(ifftn) = ifftn of (W(k)+conj W(-k))/2)
          pr = mask * amp * (double)cs;
          pi = mask * amp * (double)sn;
        } else {
          pr = 0.0;
          pi = 0.0;
        }
      }
    }
    double ar = 1.0, ai = 0.0;
    if (p.use_att) {
      const double km = p.km_att[pl];
      if (km != 0.0) {
        const double br = -p.alpha[pl] * p.dz_att;
        const double bi = -p.astar[pl] * p.dz_att;
        bool prop = true;
        double obl = 1.0;
        if (p.obliquity) {
          const double kzsq = km * km - kk;
          prop = kzsq > 0.0;
          if (prop) {
            const double kz = fmax(sqrt(fmax(kzsq, 0.0)), fabs(km) * 1e-6);
            obl = fabs(km) / kz;
          }
        }
        if (prop) {
          const double mag = (double)expf((float)(br * obl));
          float sn, cs;
          sincos_reduced(bi * obl, &sn, &cs);
          ar = mag * (double)cs;
          ai = mag * (double)sn;
        }
      }
      if (p.clip_negative && ar < 0.0) {
        ar = 0.0;
        ai = 0.0;
      }
    }
    const double nrm = p.norm;
    if (p.out_pa != nullptr)
      p.out_pa[i] = make_float2((float)((pr * ar - pi * ai) * nrm), (float)((pr * ai + pi * ar) * nrm));
    if (p.out_p != nullptr) p.out_p[i] = make_float2((float)(pr * nrm), (float)(pi * nrm));
    if (p.out_a != nullptr) p.out_a[i] = make_float2((float)(ar * nrm), (float)(ai * nrm));
  }
}

// k/kz on the rfft bins (precalculate_obliquity_map, :598-627), float32
__global__ void k_build_obl(TableParams p, float* out) {
  const size_t n = (size_t)p.nplanes * p.ncx * p.ncy;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int cy = (int)(i % p.ncy);
    const int cx = (int)((i / p.ncy) % p.ncx);
    const int pl = (int)(i / ((size_t)p.ncy * p.ncx));
    const double km = p.km_att[pl];
    const double kk = p.kx2[cx] + p.ky2[cy];
    float v = 0.f;
    if (km != 0.0) {
      const double kzsq = km * km - kk;
      if (kzsq > 0.0) {
        const double kz = fmax(sqrt(fmax(kzsq, 0.0)), fabs(km) * 1e-6);
        v = (float)(fabs(km) / kz);
      }
    }
    out[i] = v;
  }
}

int asg_launch_table(const TableParams& p, cudaStream_t st) {
  k_build_table<<<4 * 152, 256, 0, st>>>(p);
  return cudaPeekAtLastError() == cudaSuccess ? ASG_OK : ASG_ERR_CUDA;
}

int asg_launch_obl_table(const TableParams& p, float* out, cudaStream_t st) {
  k_build_obl<<<4 * 152, 256, 0, st>>>(p, out);
  return cudaPeekAtLastError() == cudaSuccess ? ASG_OK : ASG_ERR_CUDA;
}

// one thread: advance the step counter and rotate the stability maxima
__global__ void k_advance(int* step, unsigned* max_cur, unsigned* max_next) {
  *step += 1;
  *max_cur = *max_next;
  *max_next = 0u;
}

int asg_launch_advance(int* step, unsigned* max_cur, unsigned* max_next, cudaStream_t st) {
  k_advance<<<1, 1, 0, st>>>(step, max_cur, max_next);
  return cudaPeekAtLastError() == cudaSuccess ? ASG_OK : ASG_ERR_CUDA;
}

// out[c*nz + z] = in[z*ncols + c]
__global__ void k_transpose(const float* __restrict__ in, float* __restrict__ out, int nz,
                            int ncols) {
  __shared__ float tile[32][33];
  const int c0 = blockIdx.x * 32, z0 = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int z = z0 + j, c = c0 + threadIdx.x;
    if (z < nz && c < ncols) tile[j][threadIdx.x] = in[(size_t)z * ncols + c];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int c = c0 + j, z = z0 + threadIdx.x;
    if (z < nz && c < ncols) out[(size_t)c * nz + z] = tile[threadIdx.x][j];
  }
}

int asg_launch_transpose(const float* in, float* out, int nz, int ncols, cudaStream_t st) {
  dim3 grid((ncols + 31) / 32, (nz + 31) / 32);
  k_transpose<<<grid, dim3(32, 8), 0, st>>>(in, out, nz, ncols);
  return cudaPeekAtLastError() == cudaSuccess ? ASG_OK : ASG_ERR_CUDA;
}
