// Internal declarations shared by the kernel translation units and the
// C-ABI layer.  Not part of the public interface (see include/asg_gb300.h).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "asg_gb300.h"

struct SourceEvent;
struct GenPlan;

// ---- t-column pass ---------------------------------------------------------
#include "asg_column.cuh"

struct TParams {
  float2* spec;          // [planes][ncols] input spectrum (output too unless spec_out)
  float2* spec_out;      // output spectrum, or null for in place
  int ncols, nT;
  int X, Y;              // grid (fast kernels tile pairs of columns x, x+X/2)
  int split_in, split_out;  // first radix-2 x stage undone on input / applied on output
  const float2* twX;     // W_X^k, k < X
  int in_real;           // read real columns from real_in instead of the spectrum
  const float* real_in;  // [ncols][nT]
  int write_real;        // write the real column to real_out after the column phase
  float* real_out;
  int do_r2c;            // write the spectrum back
  int stats;             // accumulators / stability max in the column phase
  ColumnOps op;
  const float2* tw;      // W_nT^k, k < nT
  const float2* twM;     // W_M^k,  k < M (fast kernels)
  const unsigned* status;
  int cols_per_block;    // fast kernels: 8 or 16 columns per block, 0 = default
  int prefetch;          // fast kernels: 1 = each block prefetches into L2 the spectrum of the
                         // tile that starts about one block lifetime later (set by the launcher)
  int prefetch_ahead;    // that distance in blocks (the launcher: resident blocks of the GPU)
};

int asg_t_default_cols(int nT, int Y, int flux);
bool asg_t_cols_supported(int nT, int Y, int flux, int cols);

bool asg_t_fast_supported(int nT);
size_t asg_t_generic_smem(int nT);
int asg_launch_t(const TParams& p, bool fast, const GenPlan& pl, cudaStream_t st);

// ---- xy-plane pass ---------------------------------------------------------
struct ScreenDev {
  const float* phase;    // [X][Y]
  const float* amp;      // [X][Y] or null
};

enum EpiFlags : int {
  EPI_FREQW = 1,         // frequency-weighted boundary
  EPI_SUPERABS = 2,      // Engquist-Majda super-absorbing boundary
};

struct XYParams {
  float2* spec;          // [planes][X][Y]
  int X, Y, G;           // G CTAs per (sub-)plane (thread-block cluster)
  int nsub;              // sub-planes per plane along x (1, or 2 when the column pass
                         // applies the first radix-2 stage of the x transform)
  int nplanes;
  int nT;
  const int* f_of_plane; // rfft bin held by each plane
  const float2* table;   // [plane][ncx][ncy] multiplier (normalisation folded in) or null
  int ncx, ncy;
  const int* cls_x;      // [X] multiplier class of each x slot
  const int* cls_y;      // [Y] multiplier class of each y slot
  int zero_dc_nyq;       // planes of bin 0 and nT/2 are zeroed (analytic-signal propagator)
  const float2* twX;     // W_X^k
  const float2* twY;     // W_Y^k
  // power-spectrum reduction (nonlinear obliquity); forward transform only
  int power_only;
  const float* obl_table;  // [plane][ncx][ncy] k/kz (0 = excluded)
  double* power_acc;       // [2] sum P*obl, sum P*mask
  // stability test at the start of a step
  int check_stability;
  const unsigned* max_cur;
  double stab_coef;        // N dZ_step / dT
  double stab_thr;
  // epilogue in (x, y, omega): stage closing a step
  int epi;
  const float* fw_lx;      // log2 taper along x [X]   (freq-weighted)
  const float* fw_ly;      // log2 taper along y [Y]
  const float* fw_exp;     // exponent per plane
  const float* sa_wx;      // boundary weights [X]       (super-absorbing)
  const float* sa_wy;      // [Y]
  const float* sa_coef;    // per plane: c0/omega (0 where excluded); coeff = -i*sa_coef
  float sa_strength;
  float sa_inv2dx, sa_invdx, sa_inv2dy, sa_invdy;
  int nscreens;
  const ScreenDev* screens;
  const float* screen_fscale;  // per plane: f / max(f0_bin, 1)
  unsigned* status;
  int* status_step;
  const int* step;
  // L2-exchange plane kernel
  float2* l2_scratch;      // [clusters][2][Xs][Y]
  const int* l2_cls_x;     // [nsub][Xs] x class of each slot of the Xs-point FFT times ncy
                           //    (its row offset in the multiplier tables)
  int l2_buf_elems;        // set by the launcher
  int l2_max_clusters;     // clusters the scratch was sized for
  int coop;                // 1: CTA groups of a cooperative launch synchronised by
                           //    counters in grp_cnt instead of thread-block clusters
  unsigned* grp_cnt;       // [2][l2_max_clusters] arrival counters (zeroed by the launcher;
                           //    the second set is used by the pipelined flow)
  int pipe;                // 1 (with coop): split-phase barriers over two scratch halves
  unsigned grp_skew;       // added to every barrier target (test hook: 0 in normal runs)
  float2* spec_tmp;        // [planes][X][Y] work spectrum of the large generic planes
  int skip_plane;          // closing-stage kernel: plane left without epilogue (-1: none)
  int bulk_rows;           // L2-exchange kernels' HBM row loads: 0 cp.async, 1 bulk copies in
                           // the diffraction kernel, 2 bulk copies in both kernels
  int rows8;               // 1: a cooperative launch of the diffraction kernel uses 8-row CTAs
                           //    of 4 warps (planes from 256 wide), 0: 16-row CTAs of 8 warps
};

bool asg_xy_fast_supported(int X, int Y, int* G_out);
// L2-exchange plane kernel (asg_xyl2.cu)
bool asg_xy_l2_supported(int X, int Y, int nsub, int* G_out);
int asg_launch_xy_l2(const XYParams& p, cudaStream_t st);
// closing stage with the epilogue fused, whole planes out (same support as above, nsub = 2)
int asg_launch_xy_l2_closing(const XYParams& p, cudaStream_t st);
// half-plane kernels (rows x < X/2 and x >= X/2 transformed separately)
bool asg_xy_split_supported(int X, int Y, int* G_out);
int asg_launch_epilogue_pass(const XYParams& p, const float2* src, float2* dst, int split,
                             cudaStream_t st);
size_t asg_xy_generic_smem(int X, int Y);
// planes whose generic transform needs more shared memory than this run as
// row and column passes over HBM through XYParams::spec_tmp (nX <= 1024)
constexpr size_t ASG_XY_GENERIC_MAX_SMEM = 200 * 1024;
int asg_launch_xy(const XYParams& p, bool fast, const GenPlan& plx, const GenPlan& ply,
                  cudaStream_t st);

// ---- set-up kernels (FP64) -------------------------------------------------
struct TableParams {
  int nplanes, ncx, ncy;
  const double* kx2;       // [ncx] kx^2 of each class
  const double* ky2;       // [ncy]
  const double* kt_prop;   // [plane] propagator temporal wavenumber (shifted centred grid)
  const double* km_att;    // [plane] 2 pi f / (nT dT c0)
  const double* alpha;     // [plane] alpha(f)
  const double* astar;     // [plane] alphaStar(f)
  const int* f_of_plane;
  int nT;
  double dz_prop;          // dZ or dZ/2
  double dz_att;           // dZ * scale
  double kstart, kmax_t;   // cosine k-filter band
  int use_prop, use_att, obliquity, clip_negative;
  double norm;             // 1/(X*Y) folded in
  float2* out_pa;          // propagator x attenuation (or null)
  float2* out_p;           // propagator alone (or null)
  float2* out_a;           // attenuation alone (or null)
};
int asg_launch_table(const TableParams& p, cudaStream_t st);
int asg_launch_obl_table(const TableParams& p, float* out, cudaStream_t st);

// device-side bookkeeping between steps
int asg_launch_advance(int* step, unsigned* max_cur, unsigned* max_next, cudaStream_t st);
// (x,y,nZ) <- [nZ][x*y] transposes for the outputs
int asg_launch_transpose(const float* in, float* out, int nz, int ncols, cudaStream_t st);

int asg_roots_upload_t(const float2* w192, const float2* w64);
int asg_roots_upload_xy(const float2* w192, const float2* w64);
int asg_roots_upload_l2(const float2* w192, const float2* w64);

// One-time launcher set-up (shared-memory attributes, occupancy queries,
// constant tables) is per device: what is set with one device current does not
// carry over to another.  Launchers keep their flags per device ordinal.
constexpr int ASG_MAX_DEVICES = 64;
inline int asg_device_slot() {
  int d = 0;
  if (cudaGetDevice(&d) != cudaSuccess || d < 0 || d >= ASG_MAX_DEVICES) d = 0;
  return d;
}

// error reporting shared by the translation units (message for asg_last_error)
int asg_fail_message(int code, const char* msg);
#define CKS_NET(expr)            \
  do {                           \
    int s_ = (expr);             \
    if (s_ != ASG_OK) return s_; \
  } while (0)
