// Set-up kernels: FP64 construction of the per-mode multiplier tables, and
// the small bookkeeping kernels of the march.
//
// Multiplier of one mode (kx, ky, bin f), built in FP64 and rounded once:
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

__global__ void k_build_table(TableParams p) {
  const size_t n = (size_t)p.nplanes * p.ncx * p.ncy;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int cy = (int)(i % p.ncy);
    const int cx = (int)((i / p.ncy) % p.ncx);
    const int pl = (int)(i / ((size_t)p.ncy * p.ncx));
    const int f = p.f_of_plane[pl];
    const double kk = p.kx2[cx] + p.ky2[cy];
    double re = 1.0, im = 0.0;
    if (p.use_prop) {
      if (f == 0 || 2 * f == p.nT) {
        re = 0.0;
        im = 0.0;
      } else {
        const double k = p.kt_prop[pl];
        const double kr = sqrt(kk);
        double mask = 1.0;
        if (kr > p.kmax_t) mask = 0.0;
        else if (kr > p.kstart)
          mask = 0.5 * (1.0 + cos(M_PI * (kr - p.kstart) / (p.kmax_t - p.kstart)));
        double amp, ph;
        if (kk < k * k) {
          amp = 1.0;
          ph = p.dz_prop * kk / (k + sqrt(k * k - kk));
        } else {
          amp = exp(-p.dz_prop * sqrt(kk - k * k));
          ph = p.dz_prop * k;
        }
        double s, c;
        sincos(ph, &s, &c);
        // the reference's factor 2 on the kept bins is cancelled by the real
        // part it takes afterwards (Re(ifftn) = ifftn of (W(k)+conj W(-k))/2)
        re = mask * amp * c;
        im = mask * amp * s;
      }
    }
    if (p.use_att) {
      const double km = p.km_att[pl];
      double ar = 1.0, ai = 0.0;
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
          const double mag = exp(br * obl);
          double s, c;
          sincos(bi * obl, &s, &c);
          ar = mag * c;
          ai = mag * s;
        }
      }
      if (p.clip_negative && ar < 0.0) {
        ar = 0.0;
        ai = 0.0;
      }
      const double nr = re * ar - im * ai;
      const double ni = re * ai + im * ar;
      re = nr;
      im = ni;
    }
    p.out[i] = make_float2((float)(re * p.norm), (float)(im * p.norm));
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
