/*
 * asg_gb300.h -- C ABI of the GB300 angular-spectrum march.
 *
 * One plan = one grid (nX, nY, nT) and one option set.  The plan owns all
 * device memory; the caller owns every host buffer it passes.  A plan is not
 * thread-safe: use one plan per host thread.  Every entry point returns an
 * asg_status (0 = OK, negative = error); asg_last_error() gives the message of
 * the last failure on the calling thread.
 *
 * The entry points replace the reference's Python call stack of the march
 * (angular_spectrum_solver.py of pinton-lab/angularspectrum_heterogeneous):
 *   asg_plan_create      <- angular_spectrum_solve set-up, :1283-1296, and
 *                           SolverParams, :35-76
 *   asg_set_step_operators <- _build_operators / _to_jax, :1301-1371
 *                           (precalculate_mas :396-462, precalculate_abl :116-138,
 *                            precalculate_ad(_pow2) :468-592, precalculate_abl_freq
 *                            :144-179, _make_boundary_weights :275-284,
 *                            precalculate_obliquity_map :598-627)
 *   asg_add_screen       <- SolverParams.phaseScreens and :1505-1518
 *   asg_add_source       <- SolverParams.sourcePlanes and :1521-1527
 *   asg_run              <- the march loop, :1408-1550
 *   asg_get_outputs      <- the trimmed return tuple, :1556-1567
 *   asg_apply_operator   <- one step operator on a field: _angular_spectrum_step
 *                           :649-655, _attenuation_step :667-685,
 *                           _freq_weighted_boundary_step :658-664,
 *                           _super_absorbing_step :185-272, _apply_phase_screen
 *                           :352-390
 *   asg_flux_columns     <- _rusanov_flux_standard :688-696, _rusanov_flux_tvd
 *                           :699-724, _kt_flux :833-839, _kt_flux_minmod
 *                           :862-868, _kt_flux_adaptive :842-859
 */
#ifndef ASG_GB300_H
#define ASG_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  ASG_OK = 0,
  ASG_ERR_ARG = -1,        /* bad argument (null pointer, unknown option) */
  ASG_ERR_SHAPE = -2,      /* grid shape not supported */
  ASG_ERR_NAN = -3,        /* non-finite value in the field */
  ASG_ERR_STABILITY = -4,  /* N dZ/dT max|p| > stabilityThreshold (the reference restarts forever) */
  ASG_ERR_TIMEOUT = -5,    /* a bounded device wait gave up */
  ASG_ERR_CUDA = -6,       /* CUDA runtime error */
  ASG_ERR_STATE = -7,      /* call out of order (e.g. run before operators) */
  ASG_ERR_NOMEM = -8,      /* device allocation failed */
  ASG_ERR_SUBCYCLES = -9   /* per-column KT sub-cycling: a column needed more sub-cycles
                            * than the cap and ran above the CFL target (the outputs are
                            * complete; the run is reported, not silently accepted) */
} asg_status;

typedef struct asg_plan asg_plan;

/* Flux schemes (SolverParams.fluxScheme/useTVD/useSplitStep select among these). */
enum {
  ASG_FLUX_RUSANOV = 1,      /* _rusanov_flux_standard */
  ASG_FLUX_RUSANOV_TVD = 2,  /* _rusanov_flux_tvd */
  ASG_FLUX_KT = 3,           /* _kt_flux (MUSCL-MC) */
  ASG_FLUX_KT_MINMOD = 4     /* _kt_flux_minmod */
};

/* Options of one solve.  Doubles are SI units as in SolverParams. */
typedef struct {
  int nX, nY, nT;
  double dX, dY, dT, c0, rho0, beta, f0;
  int split_step;            /* useSplitStep */
  int flux;                  /* ASG_FLUX_* for the nonlinear step */
  int boundary_layer;        /* useBoundaryLayer */
  int freq_weighted;         /* useFreqWeightedBoundary */
  int super_absorbing;       /* useSuperAbsorbing */
  double super_absorbing_strength;
  int nonlinear_obliquity;   /* useNonlinearityObliquity */
  double stability_threshold;
  double adaptive_filter_strength; /* enters the per-step TVD parameter beta_tvd */
  double kt_cfl_target;      /* > 0: per-column KT sub-cycling at this CFL (extension) */
  int kt_max_subcycles;      /* cap on a column's sub-cycle count (0: 1024); a column that
                              * needs more makes asg_run return ASG_ERR_SUBCYCLES */
  int pax_x, pax_y;          /* column recorded in pax (reference: nX//2, nY//2) */
} asg_config;

/* 1-D operator description for one step size, all FP64, built on the host
 * (the device expands them into its multiplier tables). */
typedef struct {
  double dz;                 /* step size these operators are for */
  const double* kx;          /* [nX] centred grid of precalculate_mas, :405-406 */
  const double* ky;          /* [nY] */
  const double* kt;          /* [nT] centred temporal grid (/c0), :403-404 */
  double kfilt_start;        /* cosine k-filter start (k_trans_start) */
  double kfilt_max;          /* k_trans_max */
  const double* alpha;       /* [nT] alpha(f_m), f_m = m/(nT dT) */
  const double* alpha_star;  /* [nT] alphaStar(f_m) */
  int atten_obliquity;       /* useObliquityCorrection */
  int atten_clip_negative;   /* water model clips Re<0 to 0 */
  const double* abl_x;       /* [nX] 1-D taper (all ones without a boundary layer) */
  const double* abl_y;       /* [nY] */
  const double* abl_t;       /* [nT] */
  const double* fw_exponent; /* [nT/2+1] freq-weighted exponent per bin (or NULL) */
  const double* fw_taper_x;  /* [nX] taper of the freq-weighted mask */
  const double* fw_taper_y;  /* [nY] */
  const double* sa_wx;       /* [nX] super-absorbing weights (or NULL) */
  const double* sa_wy;       /* [nY] */
  double beta_tvd;           /* unused: the driver forms beta_tvd per step */
} asg_step_operators;

/* Plan lifecycle */
int asg_plan_create(const asg_config* cfg, asg_plan** out);
int asg_plan_destroy(asg_plan* plan);

/* Operators for the regular step (slot 0) and for a partial last step (slot 1). */
int asg_set_step_operators(asg_plan* plan, int slot, const asg_step_operators* ops);

/* Phase/amplitude screen at depth z: phase[nX*nY], amp[nX*nY] or NULL. */
int asg_add_screen(asg_plan* plan, double z, const float* phase, const float* amp);

/* Dense source plane at depth z_mid: plane[nX*nY*nT]; stored compressed to
 * its non-zero columns. */
int asg_add_source(asg_plan* plan, double z, const float* plane);

/* The same source given compact: ncols_active column indices x*nY + y and
 * their samples values[ncols_active][nT].  An extension: no dense plane is
 * ever formed (a 14.5 mm deep bowl on a 384x384x512 grid sliced every 0.308 mm
 * is 40 dense planes, 12 GB; its active columns are 114 MB). Rejects a column
 * outside the grid or given twice (ASG_ERR_ARG). */
int asg_add_source_compact(asg_plan* plan, double z, const int* cols, int ncols_active,
                           const float* values);

/* Per-step callback: step index, z after the step, device pointer to the real
 * field (nX*nY*nT float32, valid during the call). */
typedef void (*asg_step_cb)(void* user, int step, double z, const float* dev_field);

/* March from the given initial field (host, nX*nY*nT float32) over propDist
 * with step dZ (last step partial if needed).  n_steps_out receives the step
 * count; the outputs stay on the device until asg_get_outputs. */
int asg_run(asg_plan* plan, const float* initial_field, double prop_dist, double dz,
            asg_step_cb cb, void* user, int* n_steps_out);

/* Copy the outputs of the last run into host buffers laid out as the
 * reference returns them: field (nX,nY,nT), pnp/ppp/pI/pIloss (nX,nY,nZ),
 * zaxis (nZ), pax (nT,nZ).  Any pointer may be NULL to skip it. */
int asg_get_outputs(asg_plan* plan, float* field, float* pnp, float* ppp, float* pI,
                    float* pIloss, double* zaxis, float* pax);

/* Device time of the last run's march in milliseconds (CUDA events). */
int asg_last_run_ms(asg_plan* plan, double* ms);

/* Kernel kinds of one march step, for asg_kernel_stats. */
enum {
  ASG_K_XY_A = 0,      /* plane pass opening the step (+ stability test) */
  ASG_K_T_NONLIN = 1,  /* column pass with the Burgers step */
  ASG_K_XY_B = 2,      /* second half-step diffraction plane pass (Strang) */
  ASG_K_T_MID = 3,     /* column pass with the taper only (Strang) */
  ASG_K_XY_C = 4,      /* attenuation plane pass + boundary/screen epilogue */
  ASG_K_T_END = 5,     /* column pass closing the step (sources, accumulators) */
  ASG_K_OTHER = 6,     /* bookkeeping and beam-obliquity passes */
  ASG_NKINDS = 7
};

/* Record CUDA events around every kernel launch of subsequent runs. */
int asg_set_profiling(asg_plan* plan, int enable);

/* Per kind: summed device milliseconds (profiling on) and launch counts of
 * the last run (counts are kept whether or not profiling is on). */
int asg_kernel_stats(asg_plan* plan, double* ms, long* launches, int nkinds);

/* Regular march steps (full step, no screen or source crossing, no callback,
 * profiling off, not the last) replay one captured CUDA graph of the step's
 * launches; enable = 0 launches every step eagerly.  On by default.  No
 * counterpart in the reference. */
int asg_set_graphs(asg_plan* plan, int enable);

/* Batched march of independent plans (no counterpart in the reference, which
 * solves one instance per call).  Plans may have different grids and options;
 * each keeps its own operators, screens, sources and outputs (asg_get_outputs
 * per plan after the run).  Step k of all plans is issued together: the
 * plans' regular steps as one CUDA-graph launch forking to every plan's
 * stream, the others eagerly.  A plan belongs to at most one batch at a time
 * and must not run on its own while the batch runs. */
typedef struct asg_batch asg_batch;
int asg_batch_create(asg_plan* const* plans, int n, asg_batch** out);
int asg_batch_destroy(asg_batch* batch);
int asg_batch_set_graphs(asg_batch* batch, int enable);
/* fields[i]: host nX*nY*nT float32 of plan i; prop_dist[i], dz[i] as asg_run;
 * n_steps_out[i] receives each plan's step count.  Returns the first error of
 * any plan (its index in the message). */
int asg_batch_run(asg_batch* batch, const float* const* fields, const double* prop_dist,
                  const double* dz, int* n_steps_out);
/* Device time of the last batched march (all plans' steps), milliseconds. */
int asg_batch_last_run_ms(asg_batch* batch, double* ms);

/* Launch shapes of a plan (no counterpart in the reference: its XLA program
 * has no tunable launch shapes). 0 in a field selects the built-in default. */
typedef struct {
  int t_cols_flux;   /* columns per block of the column pass with the Burgers step: 8, 16 */
  int t_cols_plain;  /* columns per block of the taper-only column pass: 8, 16 */
  int t_cols_stats;  /* columns per block of the column pass closing a step: 8, 16 */
  int xy_clusters;   /* cap on resident CTA groups (clusters) of the L2-exchange plane kernel: 0..64 */
  int xy_clusters_closing; /* the same for the closing-stage kernel (fused epilogue): 0..64 */
  int xy_sync;       /* group barrier of those kernels: 1 thread-block cluster, 2 counter
                      * barrier in a cooperative launch, 3 the same with split-phase
                      * barriers over two scratch halves in the diffraction kernel (the
                      * block runs the next plane's first stage, or this plane's last,
                      * between arriving at a barrier and waiting on it); the launch is sized to fill the GPU
                      * (plans in a batch use 1; so should a plan whose stream runs
                      * beside other heavy work on the same GPU); 0 = default (3 from
                      * 256-wide planes and for groups of 12 or more CTAs, else 1) */
  int t_prefetch;    /* column passes: 1 none, 2 each block prefetches into L2 the spectrum of
                      * the tile that starts about one block lifetime later; 0 = default (1) */
  int xy_bulk;       /* HBM row loads of those kernels: 1 16-byte cp.async per lane, 2 bulk
                      * async copies (cp.async.bulk, one per row segment, mbarrier
                      * completion) in the diffraction kernel, 3 bulk copies in the
                      * closing-stage kernel too; 0 = default (1 from 256-wide planes,
                      * where cooperative launches run 8-row CTAs, else 2) */
  int xy_rows;       /* rows per CTA of the diffraction kernel in a cooperative launch
                      * (planes from 256 wide): 1 sixteen (8 warps), 2 eight (4 warps,
                      * twice the CTAs per SM); 0 = default (2).  Clusters use 16. */
} asg_tuning;

/* Test hook (no counterpart in the reference): adds `skew` to every target of
 * the counter barriers of the cooperative plane kernels (xy_sync = 2), so that
 * their bounded waits (one second) run out and the run ends with
 * ASG_ERR_TIMEOUT; 0 restores normal operation. */
int asg_debug_set_barrier_skew(asg_plan* plan, int skew);

/* Effective launch shapes (defaults resolved). */
int asg_get_tuning(asg_plan* plan, asg_tuning* out);

/* Sets launch shapes; ASG_ERR_ARG for a shape this grid does not support. */
int asg_set_tuning(asg_plan* plan, const asg_tuning* tuning);

/* Times every candidate of every shape on `steps` march steps from `field`
 * (host, nX*nY*nT floats) with step dz, keeps the fastest of each and returns
 * the result in *chosen (may be null). The plan's outputs are overwritten:
 * tune before the run whose outputs are wanted. */
int asg_autotune(asg_plan* plan, const float* field, double dz, int steps, asg_tuning* chosen);

/* One step operator on a host field in place (uses the slot-0 operators):
 * op = 1 full diffraction (HH, abl), 2 half diffraction (HH_half, abl_half),
 *      3 full attenuation, 4 half attenuation, 5 frequency-weighted boundary,
 *      6 super-absorbing boundary, 7 phase screen `screen_index`,
 *      8 beam-obliquity scalar (result in *scalar_out, field unchanged). */
int asg_apply_operator(asg_plan* plan, int op, float* field, int screen_index,
                       double* scalar_out);

/* Burgers step on ncols independent columns of length nT (host in/out).  With
 * cfl_target > 0 each column is sub-cycled at that CFL; a column that needs more
 * than max_subcycles makes the call return ASG_ERR_SUBCYCLES (out is written). */
int asg_flux_columns(const float* in, float* out, int ncols, int nT, int flux, double n_coef,
                     double dz, double dt, double beta_tvd, double cfl_target, int max_subcycles);

/* The same Burgers step on DEVICE buffers (ncols x nT floats each, column-major
 * as above; overlapping d_in and d_out ranges are rejected with ASG_ERR_ARG),
 * queued on `stream` (a cudaStream_t; NULL = the legacy default stream). No
 * counterpart in the reference: it exists for callers that must not allocate
 * device memory (memory owned by their own pool, loops where a synchronising
 * cudaMalloc/cudaFree is not allowed).
 * It allocates nothing: its scratch (a status word and the sub-cycle cap
 * counters, which it clears on `stream` before each launch, and a twiddle area)
 * is a fixed 16,640-byte array in the library. Its device address is looked up
 * on every call; the first call on a device also loads the library's kernels
 * there, so make that first call before any stream capture. nT above 2048 is
 * rejected with ASG_ERR_SHAPE; an error left pending by earlier CUDA work is
 * reported (ASG_ERR_CUDA) without launching and without clearing it. Returns
 * once the work is queued; the result is ready when `stream` is. Two calls in
 * flight at once on one device (different streams or host threads) share the
 * scratch and race: order them on one stream. */
int asg_flux_columns_device(const float* d_in, float* d_out, int ncols, int nT, int flux,
                            double n_coef, double dz, double dt, double beta_tvd,
                            double cfl_target, int max_subcycles, void* stream);

/* Sub-cycle cap counters of the last asg_flux_columns_device call on the current
 * device, read after `stream` (the stream that call used) completes: the number
 * of columns whose sub-cycle count was capped at max_subcycles (they ran above
 * cfl_target) and, if max_needed is not NULL, the largest count one of them
 * needed.  No counterpart in the reference. */
int asg_flux_columns_device_clamped(void* stream, unsigned* n_clamped, unsigned* max_needed);

/* ---- learned KT corrector (no counterpart in the reference) ------------------
 * A 1-D convolutional network along t (1 -> 64 -> 64 -> 64 -> 1 channels,
 * kernel 5, GELU, zero padding per column) whose two 64x64 layers run as BF16
 * tensor-core GEMMs with FP32 accumulation; FP32 master parameters, Adam.
 * Batches are ncols device columns of nT samples (nT a multiple of 128). */
typedef struct asg_net asg_net;
int asg_net_param_count(void);   /* length of the FP32 parameter vector */
int asg_net_create(asg_net** out);
int asg_net_destroy(asg_net* net);
/* Parameter vector layout: W1[64][5] b1[64] W2[64][64][5] b2[64] W3[64][64][5]
 * b3[64] W4[64][5] b4[1] (W[out][in][tap]); setting resets the Adam state. */
int asg_net_set_params(asg_net* net, const float* theta, int count);
int asg_net_get_params(asg_net* net, float* theta, int count);
/* y = net(x) on device buffers of ncols*nT floats, queued on `stream`. */
int asg_net_forward(asg_net* net, const float* d_x, float* d_y, int ncols, int nT, void* stream);
/* One step on a device batch: masked MSE loss of net(x) against target and its
 * gradients (to h_grad, host, asg_net_param_count() floats, when not NULL);
 * lr > 0 then applies an Adam update.  Synchronous. */
int asg_net_train_step(asg_net* net, const float* d_x, const float* d_target,
                       const float* d_mask, int ncols, int nT, float lr, double* loss_out,
                       float* h_grad);

/* Output scale gamma of the learned step (fitted on the training data):
 * out = coarse + s * gamma * cfl^3 * net(coarse * n_coef/dt * dz / 0.3),
 * s = max|u| of the column, cfl = n_coef/dt * s * dz its CFL number. */
int asg_net_set_output_scale(asg_net* net, float gamma);

/* Learned KT step on device columns (in -> out, ncols x nT floats, nT a
 * multiple of 128 up to 1024; in != out).  Per column: s = max|u|, the plain
 * KT sub-cycle count n_sub at cfl_target, and the steepness max|u[t+1]-u[t]|.
 * When n_sub >= min_subcycles, the steepness is at most shock_ratio * s and the
 * column's CFL number n_coef/dt * s * dz is at most 0.5 (the stability bound of
 * the coarse step),
 * one coarse KT step of the full dz plus the scaled correction above; otherwise
 * the plain sub-cycled KT step (the fallback).  Synchronous; *n_learned
 * receives the number of corrected columns. */
int asg_flux_columns_learned(asg_net* net, const float* d_in, float* d_out, int ncols, int nT,
                             int flux, double n_coef, double dz, double dt, double cfl_target,
                             int max_subcycles, int min_subcycles, float shock_ratio,
                             int* n_learned, void* stream);

/* Learned KT stage in the march (no counterpart in the reference): with a
 * network set, the nonlinear stage of every step takes, per column, the gated
 * learned step of asg_flux_columns_learned (one coarse KT step plus the
 * network's correction where the plain step would need at least min_subcycles
 * sub-cycles and the column is smooth: max|u[t+1]-u[t]| <= shock_ratio max|u|),
 * and the plain KT step sub-cycled at the plan's kt_cfl_target elsewhere (its
 * fallback).  Needs kt_cfl_target > 0, a KT flux and nT a multiple of 128 up to
 * 1024; steps then launch eagerly (the gate's count is read on the host).  The
 * net must outlive the plan's runs; NULL switches the stage off. */
int asg_set_learned(asg_plan* plan, asg_net* net, int min_subcycles, float shock_ratio);
/* Columns that took the learned path, and column steps in all, of the last run. */
int asg_learned_stats(asg_plan* plan, long* learned_columns, long* column_steps);

/* Message of the last error on this thread. */
const char* asg_last_error(void);

/* Library build description (arch, kernels compiled in). */
const char* asg_version(void);

#ifdef __cplusplus
}
#endif
#endif /* ASG_GB300_H */
