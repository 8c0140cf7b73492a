// Generic mixed-radix Stockham FFT over lines held in shared memory.
//
// Used for grid sizes that the fast register-resident kernels do not cover
// (odd or prime lengths such as 51, 101, 801, 1001 that the reference's own
// validation scripts use).  Out-of-place (ping-pong between two buffers),
// natural order in and out, any length; radices 2,3,4,8 run in registers,
// any other prime factor as a direct DFT.
#pragma once
#include "asg_common.cuh"

struct GenPlan {
  int n;
  int nrad;
  int rad[24];
};

template <int R, bool INV>
ASG_DEV void gen_butterfly_reg(const float2* s, float2* d, int es, int j, int nb, int Ns,
                               int twstep, int n, const float2* twn) {
  float2 v[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    float2 x = s[(j + r * nb) * es];
    if (r > 0 && twstep != 0) {
      float2 w = twn[(r * twstep) % n];
      x = INV ? cmulc(x, w) : cmul(x, w);
    }
    v[r] = x;
  }
  dft<R, INV>(v);
  const int jm = j % Ns;
  const int db = (j / Ns) * Ns * R + jm;
#pragma unroll
  for (int r = 0; r < R; ++r) d[(db + r * Ns) * es] = v[r];
}

// Output k of a direct radix-R butterfly (any prime factor).  The twiddle of
// input r is W_n^e with e = (r twstep + ((r k) mod R) nb) mod n
// = r (twstep + k nb) mod n (since R nb = n), stepped incrementally.
template <bool INV>
ASG_DEV void gen_butterfly_direct(const float2* s, float2* d, int es, int j, int nb, int Ns,
                                  int twstep, int R, int n, const float2* twn, int k) {
  const int jm = j % Ns;
  const int db = (j / Ns) * Ns * R + jm;
  const int inc = (int)(((long long)twstep + (long long)k * nb) % n);
  float accx = 0.f, accy = 0.f;
  int e = 0;
  for (int r = 0; r < R; ++r) {
    float2 x = s[(j + r * nb) * es];
    float2 w = twn[e];
    float2 y = INV ? cmulc(x, w) : cmul(x, w);
    accx += y.x;
    accy += y.y;
    e += inc;
    if (e >= n) e -= n;
  }
  d[(db + k * Ns) * es] = make_float2(accx, accy);
}

// FFT of `nlines` lines: element e of line l at buf[l*ls + e*es].  Runs over
// all threads of the block; returns the buffer holding the result.
template <bool INV>
ASG_DEV float2* gen_fft(float2* buf0, float2* buf1, int nlines, int ls, int es, const GenPlan& pl,
                        const float2* twn) {
  float2* src = buf0;
  float2* dst = buf1;
  int Ns = 1;
  const int n = pl.n;
  for (int p = 0; p < pl.nrad; ++p) {
    const int R = pl.rad[p];
    const int nb = n / R;
    // direct butterflies spread their R outputs over threads
    const int per = (R == 2 || R == 3 || R == 4 || R == 8) ? 1 : R;
    const int total = nlines * nb * per;
    for (int it = threadIdx.x; it < total; it += blockDim.x) {
      const int q = it / per, k = it - q * per;
      const int l = q / nb, j = q - l * nb;
      const float2* s = src + (size_t)l * ls;
      float2* d = dst + (size_t)l * ls;
      const int twstep = (j % Ns) * (n / (Ns * R));
      switch (R) {
        case 2: gen_butterfly_reg<2, INV>(s, d, es, j, nb, Ns, twstep, n, twn); break;
        case 3: gen_butterfly_reg<3, INV>(s, d, es, j, nb, Ns, twstep, n, twn); break;
        case 4: gen_butterfly_reg<4, INV>(s, d, es, j, nb, Ns, twstep, n, twn); break;
        case 8: gen_butterfly_reg<8, INV>(s, d, es, j, nb, Ns, twstep, n, twn); break;
        default: gen_butterfly_direct<INV>(s, d, es, j, nb, Ns, twstep, R, n, twn, k); break;
      }
    }
    __syncthreads();
    float2* t = src;
    src = dst;
    dst = t;
    Ns *= R;
  }
  return src;
}
