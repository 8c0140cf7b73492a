// C ABI of the GB300 angular-spectrum march: plan management, operator
// tables, screens/sources, and the host driver of the march.
//
// The driver reproduces the control flow of the reference's
// angular_spectrum_solve (angular_spectrum_solver.py:1408-1567):
//   z bookkeeping with sum(zvec) as a sequential double sum, partial last
//   step (:1413-1415, :1447-1450), stability test before each step (:1418-1420;
//   an error here, where the reference restarts forever), Strang or Lie
//   splitting (:1454-1492), freq-weighted and super-absorbing boundaries
//   (:1495-1502), screens crossed in (z, z+dZ] (:1505-1518), sources crossed
//   in (z, z+dZ] (:1521-1527), accumulators (:1529-1536), callback
//   (:1547-1548) and the trimmed outputs (:1556-1567).
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <mutex>
#include <string>
#include <vector>

#include "asg_generic.cuh"
#include "asg_internal.h"

// ---------------------------------------------------------------------------
// error reporting
// ---------------------------------------------------------------------------
static thread_local std::string g_err;

static int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define CK(call)                                                                    \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess)                                                          \
      return fail(ASG_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                  __FILE__, __LINE__);                                              \
  } while (0)

#define CKS(expr)                                                              \
  do {                                                                         \
    int s_ = (expr);                                                           \
    if (s_ != ASG_OK) {                                                        \
      if (g_err.empty()) fail(s_, "%s failed (%d)", #expr, s_);                \
      return s_;                                                               \
    }                                                                          \
  } while (0)

template <typename T>
static int dalloc(T** p, size_t n) {
  if (n == 0) n = 1;
  if (cudaMalloc((void**)p, n * sizeof(T)) != cudaSuccess)
    return fail(ASG_ERR_NOMEM, "cudaMalloc of %zu bytes failed", n * sizeof(T));
  return ASG_OK;
}
template <typename T>
static int h2d(T* d, const T* h, size_t n, cudaStream_t st) {
  CK(cudaMemcpyAsync(d, h, n * sizeof(T), cudaMemcpyHostToDevice, st));
  return ASG_OK;
}

// Copy between a large caller buffer on the host and the device.  The host
// buffer is page-locked for the copy (cudaHostRegister), so that it runs at the
// host link's rate instead of going through the driver's staging buffers, and
// unlocked again once the copy is done; a buffer that cannot be registered
// (already registered, for one) takes the pageable copy.
// Whether the current device reads pageable host memory through the host's page
// tables (address translation services, as on Grace-based systems): copies from
// and to pageable memory then run at the link's full rate and page-locking a
// buffer first only costs time.
static bool pageable_is_direct() {
  static int cached[ASG_MAX_DEVICES] = {};  // 0 unknown, 1 no, 2 yes
  const int dev = asg_device_slot();
  if (cached[dev] == 0) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) !=
        cudaSuccess) {
      (void)cudaGetLastError();
      v = 0;
    }
    cached[dev] = v ? 2 : 1;
  }
  return cached[dev] == 2;
}

static int copy_host(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind,
                     cudaStream_t st) {
  void* host = kind == cudaMemcpyHostToDevice ? const_cast<void*>(src) : dst;
  bool reg = false;
  if (bytes >= ((size_t)32 << 20) && !pageable_is_direct()) {
    reg = cudaHostRegister(host, bytes, cudaHostRegisterDefault) == cudaSuccess;
    if (!reg) (void)cudaGetLastError();
  }
  CK(cudaMemcpyAsync(dst, src, bytes, kind, st));
  if (reg) {
    const cudaError_t e = cudaStreamSynchronize(st);
    cudaHostUnregister(host);
    if (e != cudaSuccess) return fail(ASG_ERR_CUDA, "host copy: %s", cudaGetErrorString(e));
  }
  return ASG_OK;
}

// ---------------------------------------------------------------------------
// host FFT plan helpers
// ---------------------------------------------------------------------------
static GenPlan make_gen_plan(int n) {
  GenPlan p;
  memset(&p, 0, sizeof(p));
  p.n = n;
  int m = n;
  const int pref[4] = {8, 4, 2, 3};
  for (int r : pref) {
    while (m % r == 0 && p.nrad < 24) {
      p.rad[p.nrad++] = r;
      m /= r;
    }
  }
  for (int r = 5; m > 1 && p.nrad < 24; r += 2) {
    while (m % r == 0) {
      p.rad[p.nrad++] = r;
      m /= r;
    }
  }
  return p;
}

static void roots(int n, std::vector<float2>& out) {
  out.resize(n);
  for (int k = 0; k < n; ++k) {
    const double a = -2.0 * M_PI * (double)k / (double)n;
    out[k] = make_float2((float)cos(a), (float)sin(a));
  }
}

static constexpr int L2_MAX_CLUSTERS = 64;

// four-step slot order of a fast line of length n (n = n1*n2)
static void fast_factors(int n, int* n1, int* n2) {
  switch (n) {
    case 32: *n1 = 4; *n2 = 8; break;
    case 64: *n1 = 8; *n2 = 8; break;
    case 96: *n1 = 8; *n2 = 12; break;
    case 128: *n1 = 8; *n2 = 16; break;
    case 192: *n1 = 12; *n2 = 16; break;
    case 256: *n1 = 16; *n2 = 16; break;
    case 384: *n1 = 16; *n2 = 24; break;
    case 512: *n1 = 16; *n2 = 32; break;
    case 768: *n1 = 24; *n2 = 32; break;
    case 1024: *n1 = 32; *n2 = 32; break;
    default: *n1 = 0; *n2 = 0; break;
  }
}

// ---------------------------------------------------------------------------
// Python's built-in sum() over a list of floats (CPython >= 3.12): the first
// item enters exactly (0 + x0), later items with Neumaier compensation, and
// the compensation is added at the end when it is finite and non-zero.  The
// reference's control flow reads sum(zvec) (:1413-1414, :1506, :1522, :1548).
// ---------------------------------------------------------------------------
struct PySum {
  double f = 0.0, c = 0.0;
  long n = 0;
  void add(double x) {
    if (n == 0) {
      f = 0.0 + x;
    } else {
      const double t = f + x;
      if (fabs(f) >= fabs(x)) c += (f - t) + x;
      else c += (x - t) + f;
      f = t;
    }
    ++n;
  }
  double value() const {
    double r = f;
    if (c != 0.0 && isfinite(c)) r += c;
    return r;
  }
};

// ---------------------------------------------------------------------------
// plan
// ---------------------------------------------------------------------------
struct Slot {
  bool ready = false;
  double dz = 0.0;
  double beta_tvd = 1.0;
  float2* tabA = nullptr;  // Strang: H(dz/2) A(1/2)  | Lie: H(dz)
  float2* tabB = nullptr;  // Strang: H(dz/2)
  float2* tabC = nullptr;  // Strang: A(1/2)          | Lie: A(1)
  // 1-D vectors kept for single-operator application
  double* kt_prop = nullptr;
  double* km_att = nullptr;
  double* alpha = nullptr;
  double* astar = nullptr;
  double kstart = 0, kmax_t = 0;
  int att_obl = 1, att_clip = 0;
};

struct Screen {
  double z;
  float* phase;
  float* amp;
};
struct Source {
  double z;
  int* map;
  float* val;
  int nactive;
};

struct asg_plan {
  asg_config cfg;
  int X, Y, T, ncols, F, M;
  bool tfast, xyfast;
  bool split;  // half-plane transforms: the column pass applies the first radix-2 x stage
  bool l2;     // plane kernel with the x exchange through an L2-resident scratch
  int G, nsub;
  int t_cols[3] = {0, 0, 0};  // columns per block: flux, taper-only, statistics column passes
  int xy_clusters = 0;        // resident-cluster cap of the L2 plane kernel (0 = all)
  int xy_clusters_c = 0;      // the same for the closing-stage kernel
  int xy_bulk = 1;            // HBM row loads of the L2 plane kernels (XYParams::bulk_rows);
                              // set from default_bulk() at plan creation
  int t_prefetch = 0;         // column passes: L2 prefetch of a later tile (TParams::prefetch)
  int xy_rows = 0;            // rows per diffraction CTA in a cooperative launch (asg_tuning
                              // xy_rows: 0 default, 1 sixteen, 2 eight)
  int xy_sync = 0;            // group barrier of the L2 plane kernels: 0 default,
                              // 1 thread-block cluster, 2 counters in a cooperative launch
  int batch_refs = 0;         // batches holding the plan (they use cluster barriers)
  unsigned* grp_cnt = nullptr;  // [L2_MAX_CLUSTERS] counters of the cooperative launch
  unsigned barrier_skew = 0;    // test hook: added to the group-barrier targets
  // CUDA graph of a regular march step (slot 0, no screen, source, callback,
  // profiling or output write); rebuilt when `gen` moves on
  bool use_graphs = true;
  cudaGraphExec_t step_graph = nullptr;
  long gen = 0, graph_gen = -1;
  long graph_launches[ASG_NKINDS] = {};
  float2* l2_scratch = nullptr;
  int* l2_cls_x = nullptr;
  float2* spec2 = nullptr;  // whole-plane output of the epilogue pass (DSMEM split path)
  float2* nyq_tmp = nullptr;  // one plane: epilogue of the Nyquist plane (L2 path)
  int nyq_plane = -1;         // plane holding bin nT/2, or -1
  GenPlan gp_t, gp_x, gp_y;
  cudaStream_t st;
  cudaEvent_t ev0, ev1;
  float2* spec = nullptr;
  float* real = nullptr;
  // learned KT stage (asg_set_learned): the network, its gate, the second real
  // buffer and the counts of the last run
  asg_net* learned_net = nullptr;
  int learned_min_sub = 0;
  float learned_shock = 0.f;
  float* real2 = nullptr;
  long learned_cols = 0, learned_col_steps = 0;
  float2 *twT = nullptr, *twM = nullptr, *twX = nullptr, *twY = nullptr;
  int *f_of_plane = nullptr, *cls_x = nullptr, *cls_y = nullptr;
  int ncx, ncy;
  double *kx2 = nullptr, *ky2 = nullptr;
  std::vector<int> h_f_of_plane;
  std::vector<int> h_cls_x, h_cls_y;
  std::vector<int> h_rep_x, h_rep_y;  // centred-grid index of each class
  Slot slot[2];
  float2* tab_scratch = nullptr;
  // tapers
  float *abl_xy_half = nullptr, *abl_t_half = nullptr, *abl_xy_full = nullptr,
        *abl_t_full = nullptr;
  bool have_ops = false;
  // epilogue data
  float *fw_lx = nullptr, *fw_ly = nullptr, *fw_exp = nullptr;
  float *sa_wx = nullptr, *sa_wy = nullptr, *sa_coef = nullptr;
  float* screen_fscale = nullptr;
  float* obl_tab = nullptr;
  double* power_acc = nullptr;
  // screens / sources
  std::vector<Screen> screens;
  std::vector<Source> sources;
  ScreenDev* d_screens = nullptr;  // per-step list (max 64)
  SourceEvent* d_src = nullptr;    // per-step list (max 64)
  // state
  int* d_step = nullptr;
  unsigned *d_max_cur = nullptr, *d_max_next = nullptr, *d_status = nullptr;
  int* d_status_step = nullptr;
  double* d_iprev = nullptr;
  unsigned* d_hist = nullptr;
  unsigned* d_clamp = nullptr;     // [2] columns capped at kt_max_subcycles, largest need
  // outputs
  float *o_pnp = nullptr, *o_ppp = nullptr, *o_pI = nullptr, *o_pIloss = nullptr, *o_pax = nullptr;
  int o_cap = 0;
  std::vector<double> zaxis;
  int nsteps = 0;
  double run_ms = 0.0;
  double N = 0.0;
  // per-kernel accounting: launch counts always, CUDA-event times when enabled
  bool prof = false;
  long launches[ASG_NKINDS] = {0};
  double kms[ASG_NKINDS] = {0};
  std::vector<cudaEvent_t> ev_pool;
  std::vector<int> ev_kind;  // kind of event pair i (events 2i, 2i+1)
};

// Default HBM row loads of the plane kernels: 16-byte cp.async where the
// diffraction kernel runs 8-row CTAs in a cooperative launch (from 256-wide
// planes: 1-4 % faster than bulk copies there), bulk copies in the diffraction
// kernel otherwise.
static int default_bulk(const asg_plan* p) { return (p->l2 && p->Y >= 256) ? 0 : 1; }

// launch accounting around one kernel launch of `kind`
struct KScope {
  asg_plan* p;
  int kind;
  KScope(asg_plan* p_, int k) : p(p_), kind(k) {
    p->launches[kind]++;
    if (p->prof) {
      const size_t i = p->ev_kind.size();
      while (p->ev_pool.size() < 2 * (i + 1)) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        p->ev_pool.push_back(e);
      }
      p->ev_kind.push_back(kind);
      cudaEventRecord(p->ev_pool[2 * i], p->st);
    }
  }
  ~KScope() {
    if (p->prof) cudaEventRecord(p->ev_pool[2 * (p->ev_kind.size() - 1) + 1], p->st);
  }
};

static void collect_kernel_times(asg_plan* p) {
  if (!p->prof) return;
  cudaStreamSynchronize(p->st);
  for (size_t i = 0; i < p->ev_kind.size(); ++i) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p->ev_pool[2 * i], p->ev_pool[2 * i + 1]) == cudaSuccess)
      p->kms[p->ev_kind[i]] += ms;
  }
  p->ev_kind.clear();
}

static void free_slot(Slot& s) {
  cudaFree(s.tabA);
  cudaFree(s.tabB);
  cudaFree(s.tabC);
  cudaFree(s.kt_prop);
  cudaFree(s.km_att);
  cudaFree(s.alpha);
  cudaFree(s.astar);
  s = Slot();
}

static void free_outputs(asg_plan* p) {
  cudaFree(p->o_pnp);
  cudaFree(p->o_ppp);
  cudaFree(p->o_pI);
  cudaFree(p->o_pIloss);
  cudaFree(p->o_pax);
  p->o_pnp = p->o_ppp = p->o_pI = p->o_pIloss = p->o_pax = nullptr;
  p->o_cap = 0;
}

extern "C" int asg_plan_destroy(asg_plan* p) {
  if (!p) return ASG_OK;
  cudaStreamSynchronize(p->st);
  for (auto& s : p->slot) free_slot(s);
  for (auto& s : p->screens) {
    cudaFree(s.phase);
    cudaFree(s.amp);
  }
  for (auto& s : p->sources) {
    cudaFree(s.map);
    cudaFree(s.val);
  }
  if (p->step_graph) cudaGraphExecDestroy(p->step_graph);
  void* ptrs[] = {p->l2_scratch, p->l2_cls_x, p->grp_cnt, p->spec, p->spec2, p->nyq_tmp, p->real, p->real2, p->twT, p->twM, p->twX, p->twY, p->f_of_plane, p->cls_x,
                  p->cls_y, p->kx2, p->ky2, p->tab_scratch, p->abl_xy_half, p->abl_t_half,
                  p->abl_xy_full, p->abl_t_full, p->fw_lx, p->fw_ly, p->fw_exp, p->sa_wx,
                  p->sa_wy, p->sa_coef, p->screen_fscale, p->obl_tab, p->power_acc,
                  p->d_screens, p->d_src, p->d_step, p->d_max_cur, p->d_max_next,
                  p->d_status, p->d_status_step, p->d_iprev, p->d_hist, p->d_clamp};
  for (void* q : ptrs) cudaFree(q);
  free_outputs(p);
  cudaEventDestroy(p->ev0);
  cudaEventDestroy(p->ev1);
  for (auto e : p->ev_pool) cudaEventDestroy(e);
  cudaStreamDestroy(p->st);
  delete p;
  return ASG_OK;
}

static bool g_roots_done[ASG_MAX_DEVICES] = {};
static int upload_roots() {
  const int dev = asg_device_slot();
  if (g_roots_done[dev]) return ASG_OK;
  std::vector<float2> w192, w64;
  roots(192, w192);
  roots(64, w64);
  if (asg_roots_upload_t(w192.data(), w64.data()) != 0 ||
      asg_roots_upload_xy(w192.data(), w64.data()) != 0 ||
      asg_roots_upload_l2(w192.data(), w64.data()) != 0)
    return fail(ASG_ERR_CUDA, "upload of the constant root tables failed");
  g_roots_done[dev] = true;
  return ASG_OK;
}

static int plan_create_impl(const asg_config* cfg, asg_plan* p) {
  p->cfg = *cfg;
  const int X = cfg->nX, Y = cfg->nY, T = cfg->nT;
  if (X < 2 || Y < 2 || T < 3) return fail(ASG_ERR_SHAPE, "grid %dx%dx%d too small", X, Y, T);
  p->X = X;
  p->Y = Y;
  p->T = T;
  p->ncols = X * Y;
  p->F = T / 2 + 1;
  p->M = T / 2;
  p->N = cfg->beta / (2.0 * cfg->c0 * cfg->c0 * cfg->c0 * cfg->rho0);
  p->tfast = asg_t_fast_supported(T) && X % 2 == 0 && Y % 4 == 0;
  int Gs = 0, Gl = 0;
  p->l2 = p->tfast && asg_xy_l2_supported(X, Y, 2, &Gl);
  p->xy_bulk = default_bulk(p);
  p->split = p->l2 || (p->tfast && asg_xy_split_supported(X, Y, &Gs));
  p->xyfast = p->split || asg_xy_fast_supported(X, Y, &p->G);
  p->nsub = 1;
  if (p->split) {
    p->G = p->l2 ? Gl : Gs;
    p->nsub = 2;
  }
  if (!p->xyfast) {
    p->G = 1;
    // planes larger than one CTA's shared memory take the generic row/column
    // passes over HBM (their column pass holds whole columns: nX <= 1024)
    if (asg_xy_generic_smem(X, Y) > ASG_XY_GENERIC_MAX_SMEM && X > 1024)
      return fail(ASG_ERR_SHAPE, "grid %dx%d: nX > 1024 without a fast plane transform", X, Y);
  }
  if (!p->tfast && asg_t_generic_smem(T) > 200 * 1024)
    return fail(ASG_ERR_SHAPE, "nT=%d too long for the generic column transform", T);
  if (!p->tfast && (T + 31) / 32 > 64)
    return fail(ASG_ERR_SHAPE, "nT=%d too long for the generic column transform", T);
  if (Y > 1024) return fail(ASG_ERR_SHAPE, "nY=%d > 1024", Y);
  p->gp_t = make_gen_plan(T);
  p->gp_x = make_gen_plan(X);
  p->gp_y = make_gen_plan(Y);
  CK(cudaStreamCreateWithFlags(&p->st, cudaStreamNonBlocking));
  CK(cudaEventCreate(&p->ev0));
  CK(cudaEventCreate(&p->ev1));
  CKS(upload_roots());

  // ---- planes ----
  p->h_f_of_plane.resize(p->F);
  if (p->tfast) {
    int n1, n2;
    fast_factors(p->M, &n1, &n2);
    for (int q = 0; q < p->M; ++q) p->h_f_of_plane[q] = (q / n2) + n1 * (q % n2);
    p->h_f_of_plane[p->M] = p->M;
  } else {
    for (int q = 0; q < p->F; ++q) p->h_f_of_plane[q] = q;
  }
  // ---- x/y slot -> natural bin, and mirror classes ----
  // natural bin held by each x slot (row order of the plane kernels) and by
  // each y slot (the fast kernels keep y in four-step slot order)
  std::vector<int> binx(X), biny(Y);
  for (int s = 0; s < X; ++s) {
    if (p->split) {
      const int Xs = X / 2, R = 16, h = s / Xs, sg = s % Xs;
      binx[s] = 2 * ((sg / R) + p->G * (sg % R)) + h;
    } else if (p->xyfast) {
      const int R = 32;
      binx[s] = (s / R) + p->G * (s % R);
    } else {
      binx[s] = s;
    }
  }
  for (int s = 0; s < Y; ++s) {
    if (p->xyfast) {
      int n1, n2;
      fast_factors(Y, &n1, &n2);
      biny[s] = (s / n2) + n1 * (s % n2);
    } else {
      biny[s] = s;
    }
  }
  // x classes: centred-grid index pair {i, X-1-i} (equal kx^2), id = min
  p->ncx = (X + 1) / 2;
  p->h_cls_x.resize(X);
  p->h_rep_x.resize(p->ncx);
  for (int c = 0; c < p->ncx; ++c) p->h_rep_x[c] = c;
  for (int s = 0; s < X; ++s) {
    const int i = (binx[s] + X / 2) % X;
    p->h_cls_x[s] = i < X - 1 - i ? i : X - 1 - i;
  }
  // y classes: the smaller slot of each mirror pair, so consecutive slots read
  // consecutive table entries
  auto classes = [](int n, const std::vector<int>& bin, std::vector<int>& cls, int& ncls,
                    std::vector<int>& rep) {
    std::vector<int> slot_of_cent(n), cent(n);
    for (int s = 0; s < n; ++s) {
      cent[s] = (bin[s] + n / 2) % n;
      slot_of_cent[cent[s]] = s;
    }
    std::vector<int> raw(n), id(n, -1);
    for (int s = 0; s < n; ++s) {
      const int s2 = slot_of_cent[n - 1 - cent[s]];
      raw[s] = s < s2 ? s : s2;
    }
    ncls = 0;
    rep.clear();
    for (int s = 0; s < n; ++s)
      if (raw[s] == s) {
        id[s] = ncls++;
        rep.push_back(cent[s]);
      }
    cls.resize(n);
    for (int s = 0; s < n; ++s) cls[s] = id[raw[s]];
  };
  classes(Y, biny, p->h_cls_y, p->ncy, p->h_rep_y);

  // ---- device buffers ----
  const size_t nspec = (size_t)p->F * p->ncols;
  CKS(dalloc(&p->spec, nspec));
  const bool big = !p->xyfast && asg_xy_generic_smem(X, Y) > ASG_XY_GENERIC_MAX_SMEM;
  if ((p->split && !p->l2) || big) CKS(dalloc(&p->spec2, nspec));
  for (int q = 0; q < p->F; ++q)
    if (2 * p->h_f_of_plane[q] == T) p->nyq_plane = q;
  if (p->l2 && p->nyq_plane >= 0) CKS(dalloc(&p->nyq_tmp, (size_t)X * Y));
  if (p->l2) {
    // scratch for up to L2_MAX_CLUSTERS clusters, two half-planes each
    const int Xs = X / 2;
    CKS(dalloc(&p->l2_scratch, (size_t)L2_MAX_CLUSTERS * 2 * Xs * Y));
    int n1, n2;
    fast_factors(Xs, &n1, &n2);
    std::vector<int> cl(2 * Xs);
    for (int h = 0; h < 2; ++h)
      for (int sl = 0; sl < Xs; ++sl) {
        const int kxs = (sl / n2) + n1 * (sl % n2);  // bin of the Xs-point FFT in slot sl
        const int kx = 2 * kxs + h;
        const int i = (kx + X / 2) % X;
        // the class's row offset in the (x class, y class) multiplier tables
        cl[h * Xs + sl] = (i < X - 1 - i ? i : X - 1 - i) * p->ncy;
      }
    CKS(dalloc(&p->l2_cls_x, 2 * Xs));
    CKS(h2d(p->l2_cls_x, cl.data(), 2 * Xs, p->st));
    CKS(dalloc(&p->grp_cnt, 2 * L2_MAX_CLUSTERS));
  }
  CKS(dalloc(&p->real, (size_t)p->ncols * T));
  std::vector<float2> w;
  roots(T, w);
  CKS(dalloc(&p->twT, T));
  CKS(h2d(p->twT, w.data(), T, p->st));
  roots(p->M > 0 ? p->M : 1, w);
  CKS(dalloc(&p->twM, w.size()));
  CKS(h2d(p->twM, w.data(), w.size(), p->st));
  roots(X, w);
  CKS(dalloc(&p->twX, X));
  CKS(h2d(p->twX, w.data(), X, p->st));
  roots(Y, w);
  CKS(dalloc(&p->twY, Y));
  CKS(h2d(p->twY, w.data(), Y, p->st));
  CKS(dalloc(&p->f_of_plane, p->F));
  CKS(h2d(p->f_of_plane, p->h_f_of_plane.data(), p->F, p->st));
  CKS(dalloc(&p->cls_x, X));
  CKS(h2d(p->cls_x, p->h_cls_x.data(), X, p->st));
  CKS(dalloc(&p->cls_y, Y));
  CKS(h2d(p->cls_y, p->h_cls_y.data(), Y, p->st));
  CKS(dalloc(&p->kx2, p->ncx));
  CKS(dalloc(&p->ky2, p->ncy));
  const size_t ntab = (size_t)p->F * p->ncx * p->ncy;
  CKS(dalloc(&p->tab_scratch, ntab));
  CKS(dalloc(&p->abl_xy_half, p->ncols));
  CKS(dalloc(&p->abl_xy_full, p->ncols));
  CKS(dalloc(&p->abl_t_half, T));
  CKS(dalloc(&p->abl_t_full, T));
  CKS(dalloc(&p->fw_lx, X));
  CKS(dalloc(&p->fw_ly, Y));
  CKS(dalloc(&p->fw_exp, p->F));
  CKS(dalloc(&p->sa_wx, X));
  CKS(dalloc(&p->sa_wy, Y));
  CKS(dalloc(&p->sa_coef, p->F));
  CKS(dalloc(&p->screen_fscale, p->F));
  CKS(dalloc(&p->power_acc, 2));
  CKS(dalloc(&p->d_screens, 64));
  CKS(dalloc(&p->d_src, 64));
  CKS(dalloc(&p->d_step, 1));
  CKS(dalloc(&p->d_max_cur, 1));
  CKS(dalloc(&p->d_max_next, 1));
  CKS(dalloc(&p->d_status, 1));
  CKS(dalloc(&p->d_status_step, 1));
  CKS(dalloc(&p->d_iprev, p->ncols));
  CKS(dalloc(&p->d_hist, 64));
  CKS(dalloc(&p->d_clamp, 2));
  CK(cudaMemsetAsync(p->d_clamp, 0, 2 * sizeof(unsigned), p->st));
  CK(cudaMemsetAsync(p->d_status, 0, sizeof(unsigned), p->st));
  CK(cudaMemsetAsync(p->d_hist, 0, 64 * sizeof(unsigned), p->st));

  // per-plane constants that do not depend on the step
  {
    const double dT = cfg->dT;
    std::vector<float> sac(p->F), fsc(p->F);
    const double w1 = 2.0 * M_PI * (1.0 / (T * dT));  // omega of bin 1
    const double f0_bin = cfg->f0 / (1.0 / (T * dT));
    for (int q = 0; q < p->F; ++q) {
      const int f = p->h_f_of_plane[q];
      const double om = 2.0 * M_PI * ((double)f / (T * dT));
      sac[q] = (fabs(om) > 0.5 * w1) ? (float)(cfg->c0 / om) : 0.f;
      fsc[q] = (float)((double)(float)f / fmax(f0_bin, 1.0));
    }
    CKS(h2d(p->sa_coef, sac.data(), p->F, p->st));
    CKS(h2d(p->screen_fscale, fsc.data(), p->F, p->st));
  }
  CK(cudaStreamSynchronize(p->st));
  return ASG_OK;
}

extern "C" int asg_plan_create(const asg_config* cfg, asg_plan** out) {
  g_err.clear();
  if (!cfg || !out) return fail(ASG_ERR_ARG, "null argument");
  asg_plan* p = new asg_plan();
  int s = plan_create_impl(cfg, p);
  if (s != ASG_OK) {
    std::string e = g_err;
    asg_plan_destroy(p);
    g_err = e;
    *out = nullptr;
    return s;
  }
  *out = p;
  return ASG_OK;
}

// ---------------------------------------------------------------------------
// operators
// ---------------------------------------------------------------------------
// One pass over the modes writes the tables of a step size: out_pa = P A,
// out_p = P, out_a = A (P the propagator of dz_prop, A the attenuation of
// dz_att; null outputs are skipped, a null factor is not formed).
static int build_tables(asg_plan* p, Slot& s, float2* out_pa, float2* out_p, float2* out_a,
                        double dz_prop, double dz_att) {
  TableParams tp;
  memset(&tp, 0, sizeof(tp));
  tp.nplanes = p->F;
  tp.ncx = p->ncx;
  tp.ncy = p->ncy;
  tp.kx2 = p->kx2;
  tp.ky2 = p->ky2;
  tp.kt_prop = s.kt_prop;
  tp.km_att = s.km_att;
  tp.alpha = s.alpha;
  tp.astar = s.astar;
  tp.f_of_plane = p->f_of_plane;
  tp.nT = p->T;
  tp.dz_prop = dz_prop;
  tp.dz_att = dz_att;
  tp.kstart = s.kstart;
  tp.kmax_t = s.kmax_t;
  tp.use_prop = out_pa != nullptr || out_p != nullptr;
  tp.use_att = out_pa != nullptr || out_a != nullptr;
  tp.obliquity = s.att_obl;
  tp.clip_negative = s.att_clip;
  // the plane kernels transform X/nsub-row (sub-)planes
  tp.norm = 1.0 / ((double)(p->X / p->nsub) * (double)p->Y);
  tp.out_pa = out_pa;
  tp.out_p = out_p;
  tp.out_a = out_a;
  return asg_launch_table(tp, p->st);
}

extern "C" int asg_set_step_operators(asg_plan* p, int slot, const asg_step_operators* o) {
  g_err.clear();
  if (!p || !o || slot < 0 || slot > 1) return fail(ASG_ERR_ARG, "bad argument");
  if (!o->kx || !o->ky || !o->kt || !o->alpha || !o->alpha_star || !o->abl_x || !o->abl_y ||
      !o->abl_t)
    return fail(ASG_ERR_ARG, "missing operator vector");
  p->gen++;  // tables (and possibly their addresses) change
  const int X = p->X, Y = p->Y, T = p->T, F = p->F;
  Slot& s = p->slot[slot];
  s.dz = o->dz;
  s.beta_tvd = o->beta_tvd;
  s.kstart = o->kfilt_start;
  s.kmax_t = o->kfilt_max;
  s.att_obl = o->atten_obliquity;
  s.att_clip = o->atten_clip_negative;
  // class wavenumbers (shared by both slots)
  {
    std::vector<double> kx2(p->ncx), ky2(p->ncy);
    for (int c = 0; c < p->ncx; ++c) kx2[c] = o->kx[p->h_rep_x[c]] * o->kx[p->h_rep_x[c]];
    for (int c = 0; c < p->ncy; ++c) ky2[c] = o->ky[p->h_rep_y[c]] * o->ky[p->h_rep_y[c]];
    CKS(h2d(p->kx2, kx2.data(), p->ncx, p->st));
    CKS(h2d(p->ky2, ky2.data(), p->ncy, p->st));
  }
  // per-plane vectors
  std::vector<double> ktp(F), kma(F), al(F), as(F);
  for (int q = 0; q < F; ++q) {
    const int f = p->h_f_of_plane[q];
    ktp[q] = o->kt[(f + T / 2) % T];
    kma[q] = 2.0 * M_PI * ((double)f / (T * p->cfg.dT)) / p->cfg.c0;
    al[q] = o->alpha[f];
    as[q] = o->alpha_star[f];
  }
  if (!s.kt_prop) {
    CKS(dalloc(&s.kt_prop, F));
    CKS(dalloc(&s.km_att, F));
    CKS(dalloc(&s.alpha, F));
    CKS(dalloc(&s.astar, F));
  }
  CKS(h2d(s.kt_prop, ktp.data(), F, p->st));
  CKS(h2d(s.km_att, kma.data(), F, p->st));
  CKS(h2d(s.alpha, al.data(), F, p->st));
  CKS(h2d(s.astar, as.data(), F, p->st));
  const size_t ntab = (size_t)F * p->ncx * p->ncy;
  if (!s.tabA) {
    CKS(dalloc(&s.tabA, ntab));
    CKS(dalloc(&s.tabC, ntab));
    if (p->cfg.split_step) CKS(dalloc(&s.tabB, ntab));
  }
  const double dz = o->dz;
  if (p->cfg.split_step) {
    // A = atten(dz/2) diff(dz/2), B = diff(dz/2), C = atten(dz/2)
    CKS(build_tables(p, s, s.tabA, s.tabB, s.tabC, dz / 2, dz * 0.5));
  } else {
    // A = diff(dz), C = atten(dz)
    CKS(build_tables(p, s, nullptr, s.tabA, s.tabC, dz, dz * 1.0));
  }
  // tapers (slot independent)
  {
    std::vector<float> axh(p->ncols), axf(p->ncols), ath(T), atf(T);
    for (int x = 0; x < X; ++x)
      for (int y = 0; y < Y; ++y) {
        const double v = o->abl_x[x] * o->abl_y[y];
        axf[(size_t)x * Y + y] = (float)v;
        axh[(size_t)x * Y + y] = (float)sqrt(v);
      }
    for (int t = 0; t < T; ++t) {
      atf[t] = (float)o->abl_t[t];
      ath[t] = (float)sqrt(o->abl_t[t]);
    }
    CKS(h2d(p->abl_xy_half, axh.data(), p->ncols, p->st));
    CKS(h2d(p->abl_xy_full, axf.data(), p->ncols, p->st));
    CKS(h2d(p->abl_t_half, ath.data(), T, p->st));
    CKS(h2d(p->abl_t_full, atf.data(), T, p->st));
  }
  // freq-weighted mask factors
  if (o->fw_exponent && o->fw_taper_x && o->fw_taper_y) {
    std::vector<float> lx(X), ly(Y), fe(F);
    for (int x = 0; x < X; ++x) lx[x] = (float)log2(o->fw_taper_x[x]);
    for (int y = 0; y < Y; ++y) ly[y] = (float)log2(o->fw_taper_y[y]);
    for (int q = 0; q < F; ++q) fe[q] = (float)o->fw_exponent[p->h_f_of_plane[q]];
    CKS(h2d(p->fw_lx, lx.data(), X, p->st));
    CKS(h2d(p->fw_ly, ly.data(), Y, p->st));
    CKS(h2d(p->fw_exp, fe.data(), F, p->st));
  }
  if (o->sa_wx && o->sa_wy) {
    std::vector<float> wx(X), wy(Y);
    for (int x = 0; x < X; ++x) wx[x] = (float)o->sa_wx[x];
    for (int y = 0; y < Y; ++y) wy[y] = (float)o->sa_wy[y];
    CKS(h2d(p->sa_wx, wx.data(), X, p->st));
    CKS(h2d(p->sa_wy, wy.data(), Y, p->st));
  }
  if (p->cfg.nonlinear_obliquity && !p->obl_tab) {
    CKS(dalloc(&p->obl_tab, ntab));
    TableParams tp;
    memset(&tp, 0, sizeof(tp));
    tp.nplanes = F;
    tp.ncx = p->ncx;
    tp.ncy = p->ncy;
    tp.kx2 = p->kx2;
    tp.ky2 = p->ky2;
    tp.km_att = s.km_att;
    CKS(asg_launch_obl_table(tp, p->obl_tab, p->st));
  }
  CK(cudaStreamSynchronize(p->st));
  s.ready = true;
  if (slot == 0) p->have_ops = true;
  return ASG_OK;
}

extern "C" int asg_add_screen(asg_plan* p, double z, const float* phase, const float* amp) {
  g_err.clear();
  if (!p || !phase) return fail(ASG_ERR_ARG, "null argument");
  Screen s;
  s.z = z;
  s.phase = nullptr;
  s.amp = nullptr;
  CKS(dalloc(&s.phase, p->ncols));
  CK(cudaMemcpy(s.phase, phase, p->ncols * sizeof(float), cudaMemcpyHostToDevice));
  if (amp) {
    CKS(dalloc(&s.amp, p->ncols));
    CK(cudaMemcpy(s.amp, amp, p->ncols * sizeof(float), cudaMemcpyHostToDevice));
  }
  p->screens.push_back(s);
  return ASG_OK;
}

extern "C" int asg_add_source(asg_plan* p, double z, const float* plane) {
  g_err.clear();
  if (!p || !plane) return fail(ASG_ERR_ARG, "null argument");
  const int T = p->T;
  std::vector<int> map(p->ncols, -1);
  std::vector<float> vals;
  int na = 0;
  for (int c = 0; c < p->ncols; ++c) {
    const float* col = plane + (size_t)c * T;
    bool nz = false;
    for (int t = 0; t < T; ++t)
      if (col[t] != 0.f) {
        nz = true;
        break;
      }
    if (nz) {
      map[c] = na++;
      vals.insert(vals.end(), col, col + T);
    }
  }
  Source s;
  s.z = z;
  s.nactive = na;
  s.map = nullptr;
  s.val = nullptr;
  CKS(dalloc(&s.map, p->ncols));
  CK(cudaMemcpy(s.map, map.data(), p->ncols * sizeof(int), cudaMemcpyHostToDevice));
  CKS(dalloc(&s.val, (size_t)(na > 0 ? na : 1) * T));
  if (na > 0)
    CK(cudaMemcpy(s.val, vals.data(), vals.size() * sizeof(float), cudaMemcpyHostToDevice));
  p->sources.push_back(s);
  return ASG_OK;
}

extern "C" int asg_add_source_compact(asg_plan* p, double z, const int* cols, int ncols_active,
                                      const float* values) {
  g_err.clear();
  if (!p || ncols_active < 0 || (ncols_active > 0 && (!cols || !values)))
    return fail(ASG_ERR_ARG, "bad argument");
  const int T = p->T;
  std::vector<int> map(p->ncols, -1);
  for (int i = 0; i < ncols_active; ++i) {
    if (cols[i] < 0 || cols[i] >= p->ncols)
      return fail(ASG_ERR_ARG, "source column %d outside the grid", cols[i]);
    if (map[cols[i]] >= 0) return fail(ASG_ERR_ARG, "source column %d given twice", cols[i]);
    map[cols[i]] = i;
  }
  Source s;
  s.z = z;
  s.nactive = ncols_active;
  s.map = nullptr;
  s.val = nullptr;
  CKS(dalloc(&s.map, p->ncols));
  CK(cudaMemcpy(s.map, map.data(), p->ncols * sizeof(int), cudaMemcpyHostToDevice));
  CKS(dalloc(&s.val, (size_t)(ncols_active > 0 ? ncols_active : 1) * T));
  if (ncols_active > 0)
    CK(cudaMemcpy(s.val, values, (size_t)ncols_active * T * sizeof(float), cudaMemcpyHostToDevice));
  p->sources.push_back(s);
  return ASG_OK;
}

// ---------------------------------------------------------------------------
// kernel parameter helpers
// ---------------------------------------------------------------------------
static TParams tparams(asg_plan* p) {
  TParams t;
  memset(&t, 0, sizeof(t));
  t.spec = p->spec;
  t.spec_out = nullptr;
  t.ncols = p->ncols;
  t.nT = p->T;
  t.X = p->X;
  t.Y = p->Y;
  t.twX = p->twX;
  t.split_in = p->split;
  t.split_out = p->split;
  t.tw = p->twT;
  t.twM = p->twM;
  t.status = p->d_status;
  t.op.flux = FLUX_NONE;
  t.op.step = p->d_step;
  t.op.ncols = p->ncols;
  t.op.iprev = p->d_iprev;
  t.op.max_next = p->d_max_next;
  t.op.pnp = p->o_pnp;
  t.op.ppp = p->o_ppp;
  t.op.pI = p->o_pI;
  t.op.pIloss = p->o_pIloss;
  t.op.pax = p->o_pax;
  t.op.pax_col = p->cfg.pax_x * p->Y + p->cfg.pax_y;
  t.op.max_subcycles = p->cfg.kt_max_subcycles > 0 ? p->cfg.kt_max_subcycles : 1024;
  t.op.cfl_target = (float)p->cfg.kt_cfl_target;
  t.op.subcycle_hist = p->d_hist;
  t.op.subcycle_clamp = p->d_clamp;
  return t;
}

// Group barrier of the L2 plane kernels: by default the counter barriers of a
// cooperative launch, split into arrive and wait in the diffraction kernel
// (3; 3 % faster than 2 at 512-wide planes), for groups of 12 and 16 CTAs (large clusters leave SMs
// idle, since a cluster must fit in one GPC: 14 clusters of 16 are resident on
// a GB300, 224 of 304 CTA slots; measured 20 % faster at 512-wide planes, 2 %
// at 384) and from 256-wide planes up, where a cooperative launch runs the
// diffraction kernel with 8-row CTAs (256 x 256 x 1024: 2.02 -> 1.90 ms per
// step against clusters); thread-block clusters for smaller planes, which pack
// well, and inside a batch, whose plans run side by side.
static int xy_sync_of(const asg_plan* p) {
  if (!p->l2) return 0;
  if (p->batch_refs > 0) return 1;
  if (p->xy_sync != 0) return p->xy_sync;
  return (p->G >= 12 || p->Y >= 256) ? 3 : 1;
}

static XYParams xyparams(asg_plan* p, const float2* table, bool zero_dc_nyq) {
  XYParams x;
  memset(&x, 0, sizeof(x));
  x.spec = p->spec;
  x.X = p->X;
  x.Y = p->Y;
  x.G = p->G;
  x.nsub = p->nsub;
  x.nplanes = p->F;
  x.nT = p->T;
  x.f_of_plane = p->f_of_plane;
  x.table = table;
  x.ncx = p->ncx;
  x.ncy = p->ncy;
  x.cls_x = p->cls_x;
  x.cls_y = p->cls_y;
  x.zero_dc_nyq = zero_dc_nyq;
  x.twX = p->twX;
  x.twY = p->twY;
  x.status = p->d_status;
  x.status_step = p->d_status_step;
  x.step = p->d_step;
  x.max_cur = p->d_max_cur;
  x.fw_lx = p->fw_lx;
  x.fw_ly = p->fw_ly;
  x.fw_exp = p->fw_exp;
  x.sa_wx = p->sa_wx;
  x.sa_wy = p->sa_wy;
  x.sa_coef = p->sa_coef;
  x.sa_strength = (float)p->cfg.super_absorbing_strength;
  x.sa_inv2dx = (float)(1.0 / (2.0 * p->cfg.dX));
  x.sa_invdx = (float)(1.0 / p->cfg.dX);
  x.sa_inv2dy = (float)(1.0 / (2.0 * p->cfg.dY));
  x.sa_invdy = (float)(1.0 / p->cfg.dY);
  x.screen_fscale = p->screen_fscale;
  x.obl_table = p->obl_tab;
  x.power_acc = p->power_acc;
  x.l2_scratch = p->l2_scratch;
  x.l2_cls_x = p->l2_cls_x;
  x.l2_max_clusters = (p->xy_clusters > 0 && p->xy_clusters < L2_MAX_CLUSTERS)
                          ? p->xy_clusters : L2_MAX_CLUSTERS;
  x.coop = xy_sync_of(p) >= 2 ? 1 : 0;
  x.pipe = xy_sync_of(p) == 3 ? 1 : 0;
  x.bulk_rows = p->xy_bulk;
  x.rows8 = p->xy_rows != 1 ? 1 : 0;  // used from 256-wide planes in cooperative launches
  x.grp_cnt = p->grp_cnt;
  x.grp_skew = p->barrier_skew;
  x.spec_tmp = p->spec2;
  x.skip_plane = -1;
  return x;
}

// which tuning slot a column pass uses: 0 Burgers step, 1 taper only, 2 statistics
static int t_slot(const TParams& t) {
  if (t.stats) return 2;
  return t.op.flux != FLUX_NONE ? 0 : 1;
}

static int run_t(asg_plan* p, const TParams& t, int kind = ASG_K_OTHER) {
  KScope k(p, kind);
  if (!p->tfast) return asg_launch_t(t, false, p->gp_t, p->st);
  TParams tt = t;
  tt.cols_per_block = p->t_cols[t_slot(t)];
  tt.prefetch = p->t_prefetch;
  return asg_launch_t(tt, true, p->gp_t, p->st);
}
static int run_xy(asg_plan* p, const XYParams& x, int kind = ASG_K_OTHER) {
  KScope k(p, kind);
  if (p->l2 && x.epi == 0 && x.nscreens == 0) return asg_launch_xy_l2(x, p->st);
  return asg_launch_xy(x, p->xyfast, p->gp_x, p->gp_y, p->st);
}

static void set_flux(asg_plan* p, TParams& t, double dz, double beta_tvd, int flux) {
  t.op.flux = flux;
  t.op.dz = (float)dz;
  t.op.beta_tvd = (float)beta_tvd;
  t.op.coef_rus = (float)(p->N * dz / p->cfg.dT);
  t.op.coef_kt = (float)(p->N / p->cfg.dT);
  t.op.n_rus64 = p->N * dz / p->cfg.dT;
  t.op.n_kt64 = p->N / p->cfg.dT;
}

// the nonlinear step of the current stage, with the optional beam-obliquity
// scaling of N (march_step_*_obl, :923-965)
static int nonlinear_stage(asg_plan* p, double dz, double beta_tvd, const float* axy,
                           const float* at) {
  const int flux = p->cfg.split_step ? p->cfg.flux : ASG_FLUX_RUSANOV;
  if (p->N == 0.0) {
    // linear medium (beta = 0): every flux adds -0 * dZ/dT * (flux difference)
    // to the field, the identity for finite values (the KT step's halvings
    // aside, which change only subnormal samples), so the pass only tapers
    TParams t = tparams(p);
    t.op.abl_xy = axy;
    t.op.abl_t = at;
    t.do_r2c = 1;
    return run_t(p, t, ASG_K_T_NONLIN);
  }
  if (p->learned_net != nullptr && !p->cfg.nonlinear_obliquity &&
      (flux == ASG_FLUX_KT || flux == ASG_FLUX_KT_MINMOD)) {
    // learned KT stage: (1) inverse transform and taper into real columns,
    // (2) per column the gated learned step (one coarse KT step plus the
    // network's correction) or the plain sub-cycled KT step as its fallback,
    // (3) forward transform of the result
    {
      TParams t = tparams(p);
      t.op.abl_xy = axy;
      t.op.abl_t = at;
      t.write_real = 1;
      t.real_out = p->real;
      t.do_r2c = 0;
      CKS(run_t(p, t, ASG_K_T_NONLIN));
    }
    {
      KScope k(p, ASG_K_T_NONLIN);
      int nl = 0;
      const int s = asg_flux_columns_learned(
          p->learned_net, p->real, p->real2, p->ncols, p->T, flux, p->N, dz, p->cfg.dT,
          p->cfg.kt_cfl_target, p->cfg.kt_max_subcycles > 0 ? p->cfg.kt_max_subcycles : 1024,
          p->learned_min_sub, p->learned_shock, &nl, p->st);
      if (s != ASG_OK) return s;
      p->learned_cols += nl;
      p->learned_col_steps += p->ncols;
    }
    TParams t = tparams(p);
    t.in_real = 1;
    t.real_in = p->real2;
    t.do_r2c = 1;
    return run_t(p, t, ASG_K_T_NONLIN);
  }
  if (!p->cfg.nonlinear_obliquity) {
    TParams t = tparams(p);
    t.op.abl_xy = axy;
    t.op.abl_t = at;
    set_flux(p, t, dz, beta_tvd, flux);
    t.do_r2c = 1;
    return run_t(p, t, ASG_K_T_NONLIN);
  }
  // (1) taper only, (2) power sums of the tapered field, (3) flux with N_eff
  {
    TParams t = tparams(p);
    t.op.abl_xy = axy;
    t.op.abl_t = at;
    t.do_r2c = 1;
    CKS(run_t(p, t));
  }
  CK(cudaMemsetAsync(p->power_acc, 0, 2 * sizeof(double), p->st));
  {
    XYParams x = xyparams(p, nullptr, false);
    x.power_only = 1;
    CKS(run_xy(p, x));
  }
  TParams t = tparams(p);
  set_flux(p, t, dz, beta_tvd, flux);
  t.op.n_scale = p->power_acc;  // ratio formed in the column code
  t.do_r2c = 1;
  return run_t(p, t, ASG_K_T_NONLIN);
}

static int ensure_outputs(asg_plan* p, int cap) {
  if (p->o_cap >= cap) return ASG_OK;
  p->gen++;  // the step graph holds the old output pointers
  free_outputs(p);
  const size_t n = (size_t)cap * p->ncols;
  CKS(dalloc(&p->o_pnp, n));
  CKS(dalloc(&p->o_ppp, n));
  CKS(dalloc(&p->o_pI, n));
  CKS(dalloc(&p->o_pIloss, n));
  CKS(dalloc(&p->o_pax, (size_t)cap * p->T));
  p->o_cap = cap;
  return ASG_OK;
}

static int status_to_error(asg_plan* p) {
  unsigned st = 0;
  int sstep = 0;
  CK(cudaMemcpy(&st, p->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost));
  if (st == 0) return ASG_OK;
  CK(cudaMemcpy(&sstep, p->d_status_step, sizeof(int), cudaMemcpyDeviceToHost));
  const int code = -(int)st;
  if (code == ASG_ERR_STABILITY)
    return fail(code,
                "stability criterion violated before step %d (N*dZ/dT*max|p| > "
                "stabilityThreshold); the step cannot shrink below dZmin",
                sstep);
  if (code == ASG_ERR_NAN) return fail(code, "non-finite field value before step %d", sstep);
  return fail(code, "device status %d at step %d", code, sstep);
}

// one march step; `last` -> write the real field, no forward transform
// closing plane pass + (x, y, omega) epilogue, then the column pass that
// ends the step (or, for asg_apply_operator, just returns to real space)
static int closing_stage(asg_plan* p, const float2* table, int epi, int nscr, int kind,
                         TParams& t_after) {
  XYParams x = xyparams(p, table, false);
  if (!p->split) {
    x.epi = epi;
    x.nscreens = nscr;
    x.screens = p->d_screens;
    CKS(run_xy(p, x, kind));
    t_after.split_in = 0;
    return ASG_OK;
  }
  if (p->l2 && (epi != 0 || nscr > 0)) {
    // both half-planes of a plane in one cluster, epilogue fused, whole planes
    // out in place; the Nyquist plane (Re() before the boundary corrections)
    // goes through the epilogue pass on its own
    x.epi = epi;
    x.nscreens = nscr;
    x.screens = p->d_screens;
    x.skip_plane = p->nyq_plane;
    x.l2_max_clusters = (p->xy_clusters_c > 0 && p->xy_clusters_c < L2_MAX_CLUSTERS)
                            ? p->xy_clusters_c : L2_MAX_CLUSTERS;
    {
      KScope k(p, kind);
      CKS(asg_launch_xy_l2_closing(x, p->st));
    }
    if (p->nyq_plane >= 0) {
      const int pl = p->nyq_plane;
      const size_t pe = (size_t)p->X * p->Y;
      XYParams e = xyparams(p, nullptr, false);
      e.epi = epi;
      e.nscreens = nscr;
      e.screens = p->d_screens;
      e.nplanes = 1;
      e.f_of_plane = p->f_of_plane + pl;
      if (e.fw_exp) e.fw_exp += pl;
      if (e.sa_coef) e.sa_coef += pl;
      if (e.screen_fscale) e.screen_fscale += pl;
      KScope k(p, ASG_K_OTHER);
      CKS(asg_launch_epilogue_pass(e, p->spec + pl * pe, p->nyq_tmp, 0, p->st));
      CK(cudaMemcpyAsync(p->spec + pl * pe, p->nyq_tmp, pe * sizeof(float2),
                         cudaMemcpyDeviceToDevice, p->st));
    }
    t_after.split_in = 0;
    return ASG_OK;
  }
  CKS(run_xy(p, x, kind));
  if (epi != 0 || nscr > 0) {
    // half-planes -> whole planes with the epilogue applied, into spec2
    XYParams e = xyparams(p, nullptr, false);
    e.epi = epi;
    e.nscreens = nscr;
    e.screens = p->d_screens;
    KScope k(p, ASG_K_OTHER);
    CKS(asg_launch_epilogue_pass(e, p->spec, p->spec2, 1, p->st));
    t_after.spec = p->spec2;
    t_after.spec_out = p->spec;
    t_after.split_in = 0;
  } else {
    t_after.split_in = 1;
  }
  return ASG_OK;
}

static int march_step(asg_plan* p, const Slot& s, double dzs, double btvd, int nscr, int nsrc,
                      bool last, bool want_real) {
  const bool strang = p->cfg.split_step != 0;
  const float* axy = strang ? p->abl_xy_half : p->abl_xy_full;
  const float* at = strang ? p->abl_t_half : p->abl_t_full;
  // stage A (+ stability test)
  {
    XYParams x = xyparams(p, s.tabA, true);
    x.check_stability = 1;
    x.stab_coef = p->N * dzs / p->cfg.dT;
    x.stab_thr = p->cfg.stability_threshold;
    CKS(run_xy(p, x, ASG_K_XY_A));
  }
  CKS(nonlinear_stage(p, dzs, btvd, axy, at));
  if (strang) {
    XYParams x = xyparams(p, s.tabB, true);
    CKS(run_xy(p, x, ASG_K_XY_B));
    TParams t = tparams(p);
    t.op.abl_xy = axy;
    t.op.abl_t = at;
    t.do_r2c = 1;
    CKS(run_t(p, t, ASG_K_T_MID));
  }
  // closing stage: attenuation + (x, y, omega) epilogue, then the step end
  const int epi = (p->cfg.freq_weighted ? EPI_FREQW : 0) | (p->cfg.super_absorbing ? EPI_SUPERABS : 0);
  TParams t = tparams(p);
  CKS(closing_stage(p, s.tabC, epi, nscr, ASG_K_XY_C, t));
  t.stats = 1;
  t.op.nsrc = nsrc;
  t.op.src = p->d_src;
  t.write_real = (last || want_real) ? 1 : 0;
  t.real_out = p->real;
  t.do_r2c = last ? 0 : 1;
  CKS(run_t(p, t, ASG_K_T_END));
  KScope k(p, ASG_K_OTHER);
  return asg_launch_advance(p->d_step, p->d_max_cur, p->d_max_next, p->st);
}

// A regular step replays the captured graph of one march step.  The first
// regular step of a run without a valid graph runs eagerly (one-time launcher
// set-up such as shared-memory attributes happens outside any capture), the
// next one is captured and instantiated.  Kernels take the step index and the
// stability maxima from device memory, so every regular step is the same
// sequence of launches with the same arguments.
static int regular_step(asg_plan* p, const Slot& s, double dzs, double btvd, bool& seen) {
  if (p->step_graph && p->graph_gen == p->gen) {
    CK(cudaGraphLaunch(p->step_graph, p->st));
    for (int i = 0; i < ASG_NKINDS; ++i) p->launches[i] += p->graph_launches[i];
    return ASG_OK;
  }
  if (!seen) {
    seen = true;
    return march_step(p, s, dzs, btvd, 0, 0, false, false);
  }
  if (p->step_graph) {
    cudaGraphExecDestroy(p->step_graph);
    p->step_graph = nullptr;
  }
  long before[ASG_NKINDS];
  for (int i = 0; i < ASG_NKINDS; ++i) before[i] = p->launches[i];
  CK(cudaStreamBeginCapture(p->st, cudaStreamCaptureModeThreadLocal));
  const int st = march_step(p, s, dzs, btvd, 0, 0, false, false);
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(p->st, &g);
  if (st != ASG_OK || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    if (st != ASG_OK) return st;
    return fail(ASG_ERR_CUDA, "step capture failed: %s", cudaGetErrorString(e));
  }
  cudaGraphExec_t ex = nullptr;
  const cudaError_t e2 = cudaGraphInstantiate(&ex, g, 0);
  cudaGraphDestroy(g);
  if (e2 != cudaSuccess) return fail(ASG_ERR_CUDA, "graph instantiation: %s", cudaGetErrorString(e2));
  p->step_graph = ex;
  p->graph_gen = p->gen;
  for (int i = 0; i < ASG_NKINDS; ++i) p->graph_launches[i] = p->launches[i] - before[i];
  CK(cudaGraphLaunch(ex, p->st));
  return ASG_OK;
}

extern "C" int asg_set_graphs(asg_plan* p, int enable) {
  if (!p) return fail(ASG_ERR_ARG, "null plan");
  p->use_graphs = enable != 0;
  return ASG_OK;
}

// State of one run between its steps.
struct RunState {
  std::vector<double> steps;    // step sizes
  std::vector<double> zbefore;  // sum(zvec) before each step
  double dz = 0.0;
  double zcum = 0.0;            // np.cumsum(zvec): plain sequential sum (:1562)
  PySum zsum;
  bool regular_seen = false;
};

// Validation, the step sequence, state reset, field upload and the initial
// column pass (accumulator baselines and the first forward transform).
static int prepare_run(asg_plan* p, const float* init, double prop_dist, double dz,
                       RunState& rs) {
  if (!p || !init) return fail(ASG_ERR_ARG, "null argument");
  if (!p->slot[0].ready) return fail(ASG_ERR_STATE, "asg_set_step_operators(slot 0) not called");
  if (fabs(p->slot[0].dz - dz) != 0.0)
    return fail(ASG_ERR_STATE, "slot-0 operators were built for dz=%.17g, run asks %.17g",
                p->slot[0].dz, dz);
  rs = RunState();
  rs.dz = dz;
  // the step sequence, exactly as the reference's while loop forms it
  {
    PySum zs;
    while (zs.value() < prop_dist - 1e-15) {
      const double rem = prop_dist - zs.value();
      const double d = dz < rem ? dz : rem;
      rs.zbefore.push_back(zs.value());
      rs.steps.push_back(d);
      zs.add(d);
      if (rs.steps.size() > 100000000) return fail(ASG_ERR_ARG, "too many steps");
    }
  }
  const int cap = (int)ceil(prop_dist / dz) + 100;
  if ((int)rs.steps.size() > cap) return fail(ASG_ERR_ARG, "step count exceeds output capacity");
  for (size_t k = 0; k < rs.steps.size(); ++k) {
    const double dzs = rs.steps[k];
    if (fabs(dzs - dz) > 1e-15 && (!p->slot[1].ready || p->slot[1].dz != dzs))
      return fail(ASG_ERR_STATE, "partial step dz=%.17g needs asg_set_step_operators(slot 1)",
                  dzs);
  }
  CKS(ensure_outputs(p, cap));
  // state
  CK(cudaMemsetAsync(p->d_status, 0, sizeof(unsigned), p->st));
  CK(cudaMemsetAsync(p->d_step, 0, sizeof(int), p->st));
  CK(cudaMemsetAsync(p->d_max_cur, 0, sizeof(unsigned), p->st));
  CK(cudaMemsetAsync(p->d_max_next, 0, sizeof(unsigned), p->st));
  CK(cudaMemsetAsync(p->d_status_step, 0, sizeof(int), p->st));
  CK(cudaMemsetAsync(p->d_clamp, 0, 2 * sizeof(unsigned), p->st));
  CKS(copy_host(p->real, init, (size_t)p->ncols * p->T * sizeof(float), cudaMemcpyHostToDevice,
                p->st));
  // initial upload: iprev, stability max, forward transform
  {
    TParams t = tparams(p);
    t.in_real = 1;
    t.real_in = p->real;
    t.stats = 1;
    t.op.init_stats = 1;
    t.do_r2c = 1;
    CKS(run_t(p, t));
    // max_cur <- max_next, step stays 0
    CKS(asg_launch_advance(p->d_step, p->d_max_cur, p->d_max_next, p->st));
    CK(cudaMemsetAsync(p->d_step, 0, sizeof(int), p->st));
  }
  p->zaxis.clear();
  p->learned_cols = p->learned_col_steps = 0;
  for (int i = 0; i < ASG_NKINDS; ++i) {
    p->launches[i] = 0;
    p->kms[i] = 0.0;
  }
  p->ev_kind.clear();
  return ASG_OK;
}

// Whether step k can replay the step graph: a full step with no screen or
// source crossing, not the last, no callback, profiling off.
static bool step_is_regular(const asg_plan* p, const RunState& rs, size_t k, bool has_cb) {
  if (!p->use_graphs || has_cb || p->prof || k + 1 == rs.steps.size()) return false;
  if (p->learned_net != nullptr) return false;  // the learned stage reads a count on the host
  const double dzs = rs.steps[k], z = rs.zbefore[k];
  if (fabs(dzs - rs.dz) > 1e-15) return false;
  for (auto& sc : p->screens)
    if (z < sc.z && sc.z <= z + dzs) return false;
  for (auto& so : p->sources)
    if (z < so.z && so.z <= z + dzs) return false;
  return true;
}

static double step_btvd(const asg_plan* p, double dzs) {
  const double norm_step = dzs / (p->cfg.c0 / p->cfg.f0);
  return fmax(1.0, 2.0 - p->cfg.adaptive_filter_strength * norm_step * 10);
}

// Step k launched eagerly (screens and sources crossed in (z, z+dZ] uploaded).
static int eager_step(asg_plan* p, const RunState& rs, size_t k, bool want_real) {
  const double dzs = rs.steps[k];
  const double z = rs.zbefore[k];
  const bool partial = fabs(dzs - rs.dz) > 1e-15;
  const Slot* s = partial ? &p->slot[1] : &p->slot[0];
  std::vector<ScreenDev> scr;
  for (auto& sc : p->screens)
    if (z < sc.z && sc.z <= z + dzs) scr.push_back(ScreenDev{sc.phase, sc.amp});
  std::vector<SourceEvent> src;
  for (auto& so : p->sources)
    if (z < so.z && so.z <= z + dzs) src.push_back(SourceEvent{so.map, so.val});
  if (scr.size() > 64 || src.size() > 64)
    return fail(ASG_ERR_ARG, "more than 64 screens or sources in one step");
  if (!scr.empty()) CKS(h2d(p->d_screens, scr.data(), scr.size(), p->st));
  if (!src.empty()) CKS(h2d(p->d_src, src.data(), src.size(), p->st));
  const bool last = (k + 1 == rs.steps.size());
  return march_step(p, *s, dzs, step_btvd(p, dzs), (int)scr.size(), (int)src.size(), last,
                    want_real);
}

static void step_done(asg_plan* p, RunState& rs, size_t k) {
  rs.zcum += rs.steps[k];
  rs.zsum.add(rs.steps[k]);
  p->zaxis.push_back(rs.zcum);
}

// Columns whose per-column KT sub-cycle count was capped at kt_max_subcycles
// ran above the CFL target: the run finished (outputs are complete) but is
// reported, not passed off as meeting the target.
static int clamp_to_error(const unsigned* d_clamp, int max_subcycles, cudaStream_t st) {
  unsigned c[2] = {0u, 0u};
  CK(cudaMemcpyAsync(c, d_clamp, sizeof(c), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (c[0] == 0u) return ASG_OK;
  return fail(ASG_ERR_SUBCYCLES,
              "%u column steps needed more KT sub-cycles than the cap of %d (up to %u) and ran "
              "above the CFL target; raise the cap or the target",
              c[0], max_subcycles, c[1]);
}

static int finish_run(asg_plan* p, const RunState& rs) {
  collect_kernel_times(p);
  p->nsteps = (int)rs.steps.size();
  CKS(status_to_error(p));
  if (p->cfg.kt_cfl_target > 0.0)
    return clamp_to_error(p->d_clamp,
                          p->cfg.kt_max_subcycles > 0 ? p->cfg.kt_max_subcycles : 1024, p->st);
  return ASG_OK;
}

// ---------------------------------------------------------------------------
// Batched march: independent plans (grids of any size) advanced together.
// Step k of every plan whose step k is regular is issued as ONE graph launch:
// the graph forks from the batch stream to every plan's stream, holds one
// march step of each plan, and joins back, so the steps of all instances run
// concurrently and the hardware block scheduler balances their uneven work
// (per-column KT sub-cycle counts included: every column block is its own
// block).  Other steps (a plan's first, last or partial step, screen and
// source crossings) run eagerly on the plan's stream.  The graph is captured
// again when the set of plans in it, or one of their generations, changes.
// ---------------------------------------------------------------------------
struct asg_batch {
  std::vector<asg_plan*> plans;
  cudaStream_t master = nullptr;
  cudaEvent_t fork = nullptr, fork_cap = nullptr, ev0 = nullptr, ev1 = nullptr;
  std::vector<cudaEvent_t> join, join_cap;
  cudaGraphExec_t graph = nullptr;
  std::vector<int> graph_set;
  std::vector<long> graph_gens;
  std::vector<long> graph_launches;  // [plan in set][kind]
  bool use_graphs = true;
  double run_ms = 0.0;
};

extern "C" int asg_batch_create(asg_plan* const* plans, int n, asg_batch** out) {
  g_err.clear();
  if (!plans || n <= 0 || !out) return fail(ASG_ERR_ARG, "bad argument");
  for (int i = 0; i < n; ++i) {
    if (!plans[i]) return fail(ASG_ERR_ARG, "null plan %d", i);
    for (int j = 0; j < i; ++j)
      if (plans[j] == plans[i]) return fail(ASG_ERR_ARG, "plan %d appears twice", i);
  }
  asg_batch* b = new asg_batch();
  b->plans.assign(plans, plans + n);
  for (int i = 0; i < n; ++i) {
    plans[i]->batch_refs++;
    plans[i]->gen++;  // step graphs are captured again with cluster barriers
  }
  auto cleanup = [&](int code, const char* what) {
    cudaError_t e = cudaGetLastError();
    if (b->master) cudaStreamDestroy(b->master);
    for (cudaEvent_t ev : {b->fork, b->fork_cap, b->ev0, b->ev1})
      if (ev) cudaEventDestroy(ev);
    for (auto ev : b->join) cudaEventDestroy(ev);
    for (auto ev : b->join_cap) cudaEventDestroy(ev);
    for (asg_plan* q : b->plans) {
      q->batch_refs--;
      q->gen++;
    }
    delete b;
    return fail(code, "%s: %s", what, cudaGetErrorString(e));
  };
  if (cudaStreamCreateWithFlags(&b->master, cudaStreamNonBlocking) != cudaSuccess)
    return cleanup(ASG_ERR_CUDA, "stream");
  if (cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->fork_cap, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess)
    return cleanup(ASG_ERR_CUDA, "events");
  for (int i = 0; i < n; ++i) {
    cudaEvent_t a, c;
    if (cudaEventCreateWithFlags(&a, cudaEventDisableTiming) != cudaSuccess)
      return cleanup(ASG_ERR_CUDA, "events");
    b->join.push_back(a);
    if (cudaEventCreateWithFlags(&c, cudaEventDisableTiming) != cudaSuccess)
      return cleanup(ASG_ERR_CUDA, "events");
    b->join_cap.push_back(c);
  }
  *out = b;
  return ASG_OK;
}

extern "C" int asg_batch_destroy(asg_batch* b) {
  if (!b) return ASG_OK;
  if (b->graph) cudaGraphExecDestroy(b->graph);
  cudaStreamSynchronize(b->master);
  cudaStreamDestroy(b->master);
  for (cudaEvent_t ev : {b->fork, b->fork_cap, b->ev0, b->ev1}) cudaEventDestroy(ev);
  for (auto ev : b->join) cudaEventDestroy(ev);
  for (auto ev : b->join_cap) cudaEventDestroy(ev);
  for (asg_plan* q : b->plans) {
    q->batch_refs--;
    q->gen++;
  }
  delete b;
  return ASG_OK;
}

extern "C" int asg_batch_set_graphs(asg_batch* b, int enable) {
  if (!b) return fail(ASG_ERR_ARG, "null batch");
  b->use_graphs = enable != 0;
  return ASG_OK;
}

extern "C" int asg_batch_last_run_ms(asg_batch* b, double* ms) {
  if (!b || !ms) return fail(ASG_ERR_ARG, "null argument");
  *ms = b->run_ms;
  return ASG_OK;
}

// the batch stream waits for the listed plans' streams
static int batch_join(asg_batch* b, const std::vector<int>& set) {
  for (int i : set) {
    CK(cudaEventRecord(b->join[i], b->plans[i]->st));
    CK(cudaStreamWaitEvent(b->master, b->join[i], 0));
  }
  return ASG_OK;
}
// the listed plans' streams wait for the batch stream
static int batch_fork(asg_batch* b, const std::vector<int>& set) {
  CK(cudaEventRecord(b->fork, b->master));
  for (int i : set) CK(cudaStreamWaitEvent(b->plans[i]->st, b->fork, 0));
  return ASG_OK;
}

static int batch_capture(asg_batch* b, const std::vector<int>& set,
                         const std::vector<RunState>& rs, size_t k) {
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  std::vector<long> before(set.size() * ASG_NKINDS);
  for (size_t j = 0; j < set.size(); ++j)
    for (int q = 0; q < ASG_NKINDS; ++q) before[j * ASG_NKINDS + q] = b->plans[set[j]]->launches[q];
  CK(cudaStreamBeginCapture(b->master, cudaStreamCaptureModeThreadLocal));
  int st = ASG_OK;
  if (cudaEventRecord(b->fork_cap, b->master) != cudaSuccess) st = ASG_ERR_CUDA;
  for (int i : set) {
    asg_plan* p = b->plans[i];
    if (st == ASG_OK && cudaStreamWaitEvent(p->st, b->fork_cap, 0) != cudaSuccess) st = ASG_ERR_CUDA;
    if (st == ASG_OK) {
      const double dzs = rs[i].steps[k];
      st = march_step(p, p->slot[0], dzs, step_btvd(p, dzs), 0, 0, false, false);
    }
    // every stream that joined rejoins the batch stream, also after a failure
    cudaEventRecord(b->join_cap[i], p->st);
    cudaStreamWaitEvent(b->master, b->join_cap[i], 0);
  }
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(b->master, &g);
  if (st != ASG_OK || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    if (st != ASG_OK) return g_err.empty() ? fail(st, "batch step capture failed") : st;
    return fail(ASG_ERR_CUDA, "batch step capture: %s", cudaGetErrorString(e));
  }
  cudaGraphExec_t ex = nullptr;
  const cudaError_t e2 = cudaGraphInstantiate(&ex, g, 0);
  cudaGraphDestroy(g);
  if (e2 != cudaSuccess)
    return fail(ASG_ERR_CUDA, "batch graph instantiation: %s", cudaGetErrorString(e2));
  b->graph = ex;
  b->graph_set = set;
  b->graph_gens.clear();
  b->graph_launches.assign(set.size() * ASG_NKINDS, 0);
  for (size_t j = 0; j < set.size(); ++j) {
    asg_plan* p = b->plans[set[j]];
    b->graph_gens.push_back(p->gen);
    for (int q = 0; q < ASG_NKINDS; ++q) {
      b->graph_launches[j * ASG_NKINDS + q] = p->launches[q] - before[j * ASG_NKINDS + q];
      p->launches[q] = before[j * ASG_NKINDS + q];  // counted when the graph is launched
    }
  }
  return ASG_OK;
}

extern "C" int asg_batch_run(asg_batch* b, const float* const* fields, const double* prop_dist,
                             const double* dz, int* n_steps_out) {
  g_err.clear();
  if (!b || !fields || !prop_dist || !dz) return fail(ASG_ERR_ARG, "null argument");
  const int n = (int)b->plans.size();
  std::vector<RunState> rs(n);
  std::vector<int> all(n);
  size_t kmax = 0;
  for (int i = 0; i < n; ++i) {
    all[i] = i;
    const int st = prepare_run(b->plans[i], fields[i], prop_dist[i], dz[i], rs[i]);
    if (st != ASG_OK) {
      for (int j = 0; j < n; ++j) cudaStreamSynchronize(b->plans[j]->st);
      return st;
    }
    kmax = rs[i].steps.size() > kmax ? rs[i].steps.size() : kmax;
  }
  // the timed region starts once every plan is set up
  CKS(batch_join(b, all));
  CK(cudaEventRecord(b->ev0, b->master));
  CKS(batch_fork(b, all));
  std::vector<int> set;
  for (size_t k = 0; k < kmax; ++k) {
    set.clear();
    for (int i = 0; i < n; ++i) {
      if (k >= rs[i].steps.size()) continue;
      asg_plan* p = b->plans[i];
      if (b->use_graphs && step_is_regular(p, rs[i], k, false) && rs[i].regular_seen) {
        set.push_back(i);
      } else {
        if (step_is_regular(p, rs[i], k, false)) rs[i].regular_seen = true;
        CKS(eager_step(p, rs[i], k, false));
      }
    }
    if (!set.empty()) {
      bool same = b->graph != nullptr && b->graph_set == set;
      for (size_t j = 0; same && j < set.size(); ++j)
        same = b->graph_gens[j] == b->plans[set[j]]->gen;
      CKS(batch_join(b, set));
      if (!same) CKS(batch_capture(b, set, rs, k));
      CK(cudaGraphLaunch(b->graph, b->master));
      for (size_t j = 0; j < set.size(); ++j)
        for (int q = 0; q < ASG_NKINDS; ++q)
          b->plans[set[j]]->launches[q] += b->graph_launches[j * ASG_NKINDS + q];
      CKS(batch_fork(b, set));
    }
    for (int i = 0; i < n; ++i)
      if (k < rs[i].steps.size()) step_done(b->plans[i], rs[i], k);
  }
  CKS(batch_join(b, all));
  CK(cudaEventRecord(b->ev1, b->master));
  CK(cudaStreamSynchronize(b->master));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
  b->run_ms = ms;
  int first = ASG_OK;
  std::string msg;
  for (int i = 0; i < n; ++i) {
    const int st = finish_run(b->plans[i], rs[i]);
    if (n_steps_out) n_steps_out[i] = b->plans[i]->nsteps;
    if (st != ASG_OK && first == ASG_OK) {
      first = st;
      msg = "instance " + std::to_string(i) + ": " + g_err;
    }
  }
  if (first != ASG_OK) g_err = msg;
  return first;
}

extern "C" int asg_run(asg_plan* p, const float* init, double prop_dist, double dz,
                       asg_step_cb cb, void* user, int* n_steps_out) {
  g_err.clear();
  RunState rs;
  CKS(prepare_run(p, init, prop_dist, dz, rs));
  CK(cudaEventRecord(p->ev0, p->st));
  for (size_t k = 0; k < rs.steps.size(); ++k) {
    if (step_is_regular(p, rs, k, cb != nullptr))
      CKS(regular_step(p, p->slot[0], rs.steps[k], step_btvd(p, rs.steps[k]), rs.regular_seen));
    else
      CKS(eager_step(p, rs, k, cb != nullptr));
    step_done(p, rs, k);
    if (cb) {
      CK(cudaStreamSynchronize(p->st));
      CKS(status_to_error(p));
      cb(user, (int)k, rs.zsum.value(), p->real);
    }
  }
  CK(cudaEventRecord(p->ev1, p->st));
  CK(cudaStreamSynchronize(p->st));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, p->ev0, p->ev1));
  p->run_ms = ms;
  const int st = finish_run(p, rs);
  if (n_steps_out) *n_steps_out = p->nsteps;
  return st;
}

extern "C" int asg_get_outputs(asg_plan* p, float* field, float* pnp, float* ppp, float* pI,
                               float* pIloss, double* zaxis, float* pax) {
  g_err.clear();
  if (!p) return fail(ASG_ERR_ARG, "null plan");
  const int nz = p->nsteps;
  const size_t nc = p->ncols;
  if (field) {
    CKS(copy_host(field, p->real, nc * p->T * sizeof(float), cudaMemcpyDeviceToHost, p->st));
    CK(cudaStreamSynchronize(p->st));
  }
  if (nz > 0) {
    float* tmp = nullptr;
    CKS(dalloc(&tmp, (size_t)nz * (nc > (size_t)p->T ? nc : (size_t)p->T)));
    float* srcs[4] = {p->o_pnp, p->o_ppp, p->o_pI, p->o_pIloss};
    float* dsts[4] = {pnp, ppp, pI, pIloss};
    for (int i = 0; i < 4; ++i) {
      if (!dsts[i]) continue;
      CKS(asg_launch_transpose(srcs[i], tmp, nz, (int)nc, p->st));
      CKS(copy_host(dsts[i], tmp, (size_t)nz * nc * sizeof(float), cudaMemcpyDeviceToHost, p->st));
      CK(cudaStreamSynchronize(p->st));
    }
    if (pax) {
      CKS(asg_launch_transpose(p->o_pax, tmp, nz, p->T, p->st));
      CK(cudaMemcpyAsync(pax, tmp, (size_t)nz * p->T * sizeof(float), cudaMemcpyDeviceToHost,
                         p->st));
      CK(cudaStreamSynchronize(p->st));
    }
    cudaFree(tmp);
  }
  if (zaxis && nz > 0) memcpy(zaxis, p->zaxis.data(), nz * sizeof(double));
  return ASG_OK;
}

extern "C" int asg_set_profiling(asg_plan* p, int enable) {
  if (!p) return fail(ASG_ERR_ARG, "null plan");
  p->prof = enable != 0;
  return ASG_OK;
}

extern "C" int asg_kernel_stats(asg_plan* p, double* ms, long* launches, int nkinds) {
  if (!p || nkinds <= 0) return fail(ASG_ERR_ARG, "bad argument");
  for (int i = 0; i < nkinds && i < ASG_NKINDS; ++i) {
    if (ms) ms[i] = p->kms[i];
    if (launches) launches[i] = p->launches[i];
  }
  return ASG_OK;
}

// ---------------------------------------------------------------------------
// launch-shape tuning
// ---------------------------------------------------------------------------
extern "C" int asg_get_tuning(asg_plan* p, asg_tuning* out) {
  if (!p || !out) return fail(ASG_ERR_ARG, "null argument");
  const int flux = p->cfg.flux != 0;
  for (int i = 0; i < 3; ++i) {
    int c = p->t_cols[i];
    if (c == 0) c = p->tfast ? asg_t_default_cols(p->T, p->Y, i == 0 ? flux : 0) : 4;
    (&out->t_cols_flux)[i] = c;
  }
  int ncl = p->xy_clusters > 0 ? p->xy_clusters : L2_MAX_CLUSTERS;
  out->xy_clusters = p->l2 ? ncl : 0;
  ncl = p->xy_clusters_c > 0 ? p->xy_clusters_c : L2_MAX_CLUSTERS;
  out->xy_clusters_closing = p->l2 ? ncl : 0;
  out->xy_sync = xy_sync_of(p);
  out->xy_bulk = p->l2 ? p->xy_bulk + 1 : 0;
  out->xy_rows = (p->l2 && p->Y >= 256) ? (p->xy_rows == 1 ? 1 : 2) : 0;
  out->t_prefetch = p->tfast ? p->t_prefetch + 1 : 0;
  return ASG_OK;
}

extern "C" int asg_set_tuning(asg_plan* p, const asg_tuning* t) {
  g_err.clear();
  if (!p || !t) return fail(ASG_ERR_ARG, "null argument");
  const int cols[3] = {t->t_cols_flux, t->t_cols_plain, t->t_cols_stats};
  for (int i = 0; i < 3; ++i) {
    if (cols[i] == 0) continue;
    if (!p->tfast || !asg_t_cols_supported(p->T, p->Y, i == 0, cols[i]))
      return fail(ASG_ERR_ARG, "%d columns per block not available for nT=%d, nY=%d", cols[i],
                  p->T, p->Y);
  }
  if (t->xy_clusters < 0 || t->xy_clusters > L2_MAX_CLUSTERS ||
      t->xy_clusters_closing < 0 || t->xy_clusters_closing > L2_MAX_CLUSTERS)
    return fail(ASG_ERR_ARG, "cluster caps %d, %d outside 0..%d", t->xy_clusters,
                t->xy_clusters_closing, L2_MAX_CLUSTERS);
  if (t->xy_sync < 0 || t->xy_sync > 3) return fail(ASG_ERR_ARG, "xy_sync %d outside 0..3", t->xy_sync);
  if (t->xy_bulk < 0 || t->xy_bulk > 3) return fail(ASG_ERR_ARG, "xy_bulk %d outside 0..3", t->xy_bulk);
  if (t->xy_rows < 0 || t->xy_rows > 2) return fail(ASG_ERR_ARG, "xy_rows %d outside 0..2", t->xy_rows);
  if (t->t_prefetch < 0 || t->t_prefetch > 2)
    return fail(ASG_ERR_ARG, "t_prefetch %d outside 0..2", t->t_prefetch);
  for (int i = 0; i < 3; ++i) p->t_cols[i] = cols[i];
  p->xy_clusters = t->xy_clusters;
  p->xy_clusters_c = t->xy_clusters_closing;
  p->xy_sync = t->xy_sync;
  p->xy_bulk = t->xy_bulk == 0 ? default_bulk(p) : t->xy_bulk - 1;
  p->xy_rows = t->xy_rows;
  p->t_prefetch = t->t_prefetch == 0 ? 0 : t->t_prefetch - 1;
  p->gen++;
  return ASG_OK;
}

// Times each candidate of each knob on `steps` march steps from `field` and
// keeps the fastest (per-kind device time of the passes the knob drives).
extern "C" int asg_autotune(asg_plan* p, const float* field, double dz, int steps,
                            asg_tuning* chosen) {
  g_err.clear();
  if (!p || !field || !(dz > 0.0) || steps < 1) return fail(ASG_ERR_ARG, "bad argument");
  if (!p->slot[0].ready) return fail(ASG_ERR_STATE, "operators not set");
  const bool prof = p->prof;
  p->prof = true;
  auto trial = [&](int kind, double* ms) -> int {
    int n = 0;
    int s = asg_run(p, field, steps * dz, dz, nullptr, nullptr, &n);
    if (s != ASG_OK) return s;
    *ms = p->launches[kind] > 0 ? p->kms[kind] / p->launches[kind] : 0.0;
    return ASG_OK;
  };
  int status = ASG_OK;
  if (p->tfast) {
    const int kinds[3] = {ASG_K_T_NONLIN, ASG_K_T_MID, ASG_K_T_END};
    for (int i = 0; i < 3 && status == ASG_OK; ++i) {
      if (i == 1 && !p->cfg.split_step) continue;  // no taper-only pass in the Lie march
      double best = 1e300;
      int best_c = 0;
      for (int c : {8, 16}) {
        if (!asg_t_cols_supported(p->T, p->Y, i == 0, c)) continue;
        p->t_cols[i] = c;
        double ms = 0.0;
        status = trial(kinds[i], &ms);
        if (status != ASG_OK) break;
        if (ms < best) {
          best = ms;
          best_c = c;
        }
      }
      p->t_cols[i] = best_c;
    }
    // L2 prefetch of later tiles: the three column passes together
    double best = 1e300;
    int best_f = 0;
    for (int f : {0, 1}) {
      if (status != ASG_OK) break;
      p->t_prefetch = f;
      double ms = 0.0;
      status = trial(ASG_K_T_NONLIN, &ms);
      if (status != ASG_OK) break;
      for (int k : {ASG_K_T_MID, ASG_K_T_END})
        if (p->launches[k] > 0) ms += p->kms[k] / p->launches[k];
      if (ms < best) {
        best = ms;
        best_f = f;
      }
    }
    p->t_prefetch = best_f;
  }
  if (p->l2 && status == ASG_OK && p->batch_refs == 0) {
    // group barrier: the plain diffraction pass and the closing pass together
    const bool closing = p->cfg.freq_weighted || p->cfg.super_absorbing;
    double best = 1e300;
    int best_s = 0;
    for (int sy : {1, 2, 3}) {
      p->xy_sync = sy;
      double ms = 0.0, ms_c = 0.0;
      status = trial(p->cfg.split_step ? ASG_K_XY_B : ASG_K_XY_A, &ms);
      if (status != ASG_OK) break;
      if (closing) {
        ms_c = p->launches[ASG_K_XY_C] > 0 ? p->kms[ASG_K_XY_C] / p->launches[ASG_K_XY_C] : 0.0;
      }
      if (ms + ms_c < best) {
        best = ms + ms_c;
        best_s = sy;
      }
    }
    p->xy_sync = best_s;
  }
  if (p->l2 && p->Y >= 256 && xy_sync_of(p) >= 2 && status == ASG_OK) {
    // tile shape of the cooperative diffraction kernel: 16-row or 8-row CTAs
    double best = 1e300;
    int best_r = 2;
    for (int r : {1, 2}) {
      p->xy_rows = r;
      double ms = 0.0;
      status = trial(p->cfg.split_step ? ASG_K_XY_B : ASG_K_XY_A, &ms);
      if (status != ASG_OK) break;
      if (ms < best) {
        best = ms;
        best_r = r;
      }
    }
    p->xy_rows = best_r;
  }
  if (p->l2 && status == ASG_OK) {
    double best = 1e300;
    int best_n = 0;
    for (int n : {0, 16, 12, 8}) {
      p->xy_clusters = n;
      double ms = 0.0;
      // the plain diffraction pass: B in the Strang march, A in the Lie march
      status = trial(p->cfg.split_step ? ASG_K_XY_B : ASG_K_XY_A, &ms);
      if (status != ASG_OK) break;
      if (ms < best) {
        best = ms;
        best_n = n;
      }
    }
    p->xy_clusters = best_n;
  }
  if (p->l2 && status == ASG_OK) {
    // HBM row loads of the plane kernels: cp.async, or bulk copies in the
    // diffraction kernel, or in both (diffraction and closing passes together)
    const bool closing = p->cfg.freq_weighted || p->cfg.super_absorbing;
    double best = 1e300;
    int best_b = 1;
    for (int b : {0, 1, 2}) {
      p->xy_bulk = b;
      double ms = 0.0, ms_c = 0.0;
      status = trial(p->cfg.split_step ? ASG_K_XY_B : ASG_K_XY_A, &ms);
      if (status != ASG_OK) break;
      if (closing)
        ms_c = p->launches[ASG_K_XY_C] > 0 ? p->kms[ASG_K_XY_C] / p->launches[ASG_K_XY_C] : 0.0;
      if (ms + ms_c < best) {
        best = ms + ms_c;
        best_b = b;
      }
    }
    p->xy_bulk = best_b;
  }
  // the closing-stage kernel runs when the step has a boundary epilogue
  if (p->l2 && (p->cfg.freq_weighted || p->cfg.super_absorbing) && status == ASG_OK) {
    double best = 1e300;
    int best_n = 0;
    for (int n : {0, 16, 12, 8}) {
      p->xy_clusters_c = n;
      double ms = 0.0;
      status = trial(ASG_K_XY_C, &ms);
      if (status != ASG_OK) break;
      if (ms < best) {
        best = ms;
        best_n = n;
      }
    }
    p->xy_clusters_c = best_n;
  }
  p->prof = prof;
  p->gen++;
  if (status != ASG_OK) return status;
  return chosen ? asg_get_tuning(p, chosen) : ASG_OK;
}

extern "C" int asg_set_learned(asg_plan* p, asg_net* net, int min_subcycles,
                               float shock_ratio) {
  g_err.clear();
  if (!p) return fail(ASG_ERR_ARG, "null argument");
  if (net == nullptr) {
    p->learned_net = nullptr;
    return ASG_OK;
  }
  if (!(p->cfg.kt_cfl_target > 0.0))
    return fail(ASG_ERR_STATE, "the learned KT stage needs per-column sub-cycling "
                               "(kt_cfl_target > 0): it defines the gate and the fallback");
  if (p->cfg.flux != ASG_FLUX_KT && p->cfg.flux != ASG_FLUX_KT_MINMOD)
    return fail(ASG_ERR_ARG, "the learned step corrects the KT schemes only");
  if (p->T % 128 != 0 || p->T > 1024)
    return fail(ASG_ERR_SHAPE, "learned step: nT a multiple of 128 up to 1024 (nT=%d)", p->T);
  if (min_subcycles < 1) return fail(ASG_ERR_ARG, "min_subcycles < 1");
  if (!p->real2) CKS(dalloc(&p->real2, (size_t)p->ncols * p->T));
  p->learned_net = net;
  p->learned_min_sub = min_subcycles;
  p->learned_shock = shock_ratio;
  p->gen++;
  return ASG_OK;
}

extern "C" int asg_learned_stats(asg_plan* p, long* learned_columns, long* column_steps) {
  if (!p) return fail(ASG_ERR_ARG, "null argument");
  if (learned_columns) *learned_columns = p->learned_cols;
  if (column_steps) *column_steps = p->learned_col_steps;
  return ASG_OK;
}

extern "C" int asg_debug_set_barrier_skew(asg_plan* p, int skew) {
  if (!p || skew < 0) return fail(ASG_ERR_ARG, "bad argument");
  p->barrier_skew = (unsigned)skew;
  p->gen++;
  return ASG_OK;
}

extern "C" int asg_last_run_ms(asg_plan* p, double* ms) {
  if (!p || !ms) return fail(ASG_ERR_ARG, "null argument");
  *ms = p->run_ms;
  return ASG_OK;
}

// ---------------------------------------------------------------------------
// single operators on a host field (parity tests of each stage)
// ---------------------------------------------------------------------------
extern "C" int asg_apply_operator(asg_plan* p, int op, float* field, int screen_index,
                                  double* scalar_out) {
  g_err.clear();
  if (!p || !field) return fail(ASG_ERR_ARG, "null argument");
  if (!p->slot[0].ready) return fail(ASG_ERR_STATE, "operators not set");
  Slot& s = p->slot[0];
  const size_t n = (size_t)p->ncols * p->T;
  CK(cudaMemsetAsync(p->d_status, 0, sizeof(unsigned), p->st));
  CK(cudaMemsetAsync(p->d_step, 0, sizeof(int), p->st));
  CK(cudaMemcpyAsync(p->real, field, n * sizeof(float), cudaMemcpyHostToDevice, p->st));
  {
    TParams t = tparams(p);
    t.in_real = 1;
    t.real_in = p->real;
    t.do_r2c = 1;
    CKS(run_t(p, t));
  }
  const float* axy = nullptr;
  const float* at = nullptr;
  const float2* table = nullptr;
  int zero = 0, epi = 0, nscr = 0;
  switch (op) {
    case 1:
    case 2:
      CKS(build_tables(p, s, nullptr, p->tab_scratch, nullptr, op == 1 ? s.dz : s.dz / 2, 0.0));
      table = p->tab_scratch;
      zero = 1;
      axy = op == 1 ? p->abl_xy_full : p->abl_xy_half;
      at = op == 1 ? p->abl_t_full : p->abl_t_half;
      break;
    case 3:
    case 4:
      CKS(build_tables(p, s, nullptr, nullptr, p->tab_scratch, 0.0, op == 3 ? s.dz : s.dz * 0.5));
      table = p->tab_scratch;
      break;
    case 5: epi = EPI_FREQW; break;
    case 6: epi = EPI_SUPERABS; break;
    case 7: {
      if (screen_index < 0 || screen_index >= (int)p->screens.size())
        return fail(ASG_ERR_ARG, "screen index %d out of range", screen_index);
      ScreenDev sd{p->screens[screen_index].phase, p->screens[screen_index].amp};
      CKS(h2d(p->d_screens, &sd, 1, p->st));
      nscr = 1;
      break;
    }
    case 8: {
      if (!p->obl_tab) return fail(ASG_ERR_STATE, "plan built without nonlinear obliquity");
      CK(cudaMemsetAsync(p->power_acc, 0, 2 * sizeof(double), p->st));
      XYParams x = xyparams(p, nullptr, false);
      x.power_only = 1;
      CKS(run_xy(p, x));
      double acc[2];
      CK(cudaMemcpyAsync(acc, p->power_acc, sizeof(acc), cudaMemcpyDeviceToHost, p->st));
      CK(cudaStreamSynchronize(p->st));
      if (scalar_out) *scalar_out = acc[0] / (acc[1] + 1e-30);
      return status_to_error(p);
    }
    default: return fail(ASG_ERR_ARG, "unknown operator %d", op);
  }
  TParams t = tparams(p);
  if (zero) {
    XYParams x = xyparams(p, table, true);
    CKS(run_xy(p, x));
  } else {
    CKS(closing_stage(p, table, epi, nscr, ASG_K_OTHER, t));
  }
  t.op.abl_xy = axy;
  t.op.abl_t = at;
  t.write_real = 1;
  t.real_out = p->real;
  t.do_r2c = 0;
  CKS(run_t(p, t));
  CK(cudaMemcpyAsync(field, p->real, n * sizeof(float), cudaMemcpyDeviceToHost, p->st));
  CK(cudaStreamSynchronize(p->st));
  return status_to_error(p);
}

extern "C" int asg_flux_columns(const float* in, float* out, int ncols, int nT, int flux,
                                double n_coef, double dz, double dt, double beta_tvd,
                                double cfl_target, int max_subcycles) {
  g_err.clear();
  if (!in || !out || ncols <= 0 || nT < 3) return fail(ASG_ERR_ARG, "bad argument");
  if ((nT + 31) / 32 > 64 || asg_t_generic_smem(nT) > 200 * 1024)
    return fail(ASG_ERR_SHAPE, "nT=%d too long", nT);
  if (flux < ASG_FLUX_RUSANOV || flux > ASG_FLUX_KT_MINMOD)
    return fail(ASG_ERR_ARG, "unknown flux %d", flux);
  CKS(upload_roots());
  float *d = nullptr, *dout = nullptr;
  unsigned* st = nullptr;
  float2* tw = nullptr;
  const size_t n = (size_t)ncols * nT;
  CKS(dalloc(&d, n));
  CKS(dalloc(&dout, n));
  CKS(dalloc(&st, 4));  // status word, then the sub-cycle cap counters [2]
  CKS(dalloc(&tw, nT));
  CK(cudaMemset(st, 0, 4 * sizeof(unsigned)));
  CK(cudaMemcpy(d, in, n * sizeof(float), cudaMemcpyHostToDevice));
  TParams t;
  memset(&t, 0, sizeof(t));
  t.ncols = ncols;
  t.nT = nT;
  t.in_real = 1;
  t.real_in = d;
  t.write_real = 1;
  t.real_out = dout;
  t.tw = tw;
  t.status = st;
  t.op.flux = flux;
  t.op.dz = (float)dz;
  t.op.beta_tvd = (float)beta_tvd;
  t.op.coef_rus = (float)(n_coef * dz / dt);
  t.op.coef_kt = (float)(n_coef / dt);
  t.op.n_rus64 = n_coef * dz / dt;
  t.op.n_kt64 = n_coef / dt;
  t.op.cfl_target = (float)cfl_target;
  t.op.max_subcycles = max_subcycles > 0 ? max_subcycles : 1024;
  t.op.subcycle_clamp = st + 1;
  GenPlan gp = make_gen_plan(nT);
  int s = asg_launch_t(t, false, gp, 0);
  cudaError_t e = cudaDeviceSynchronize();
  if (s == ASG_OK && e == cudaSuccess)
    e = cudaMemcpy(out, dout, n * sizeof(float), cudaMemcpyDeviceToHost);
  int sc = ASG_OK;
  if (s == ASG_OK && e == cudaSuccess && cfl_target > 0.0)
    sc = clamp_to_error(st + 1, t.op.max_subcycles, 0);
  cudaFree(d);
  cudaFree(dout);
  cudaFree(st);
  cudaFree(tw);
  if (s != ASG_OK) return fail(s, "flux kernel launch failed");
  if (e != cudaSuccess) return fail(ASG_ERR_CUDA, "%s", cudaGetErrorString(e));
  return sc;
}

// ---------------------------------------------------------------------------
// asg_flux_columns_device: the Burgers column step on the caller's device
// buffers and stream, allocating nothing.
//
// asg_flux_columns allocates and frees four device buffers on every call. Some
// callers cannot have that: a host framework whose device memory all belongs
// to its own pool, a real-time loop in which cudaMalloc/cudaFree (which
// synchronise the device) are not allowed, or code that queues work on a
// stream it must not stall. They call this entry point instead. Besides its
// input and output the column kernel touches three small global areas: a
// status word it reads first (it must be zero, or the kernel returns without
// work), the sub-cycle cap counters it adds to, and a twiddle area it copies
// into shared memory (unused here, since the columns go in and out as real
// samples with no transform). All live in the fixed array below.
// ---------------------------------------------------------------------------
static constexpr int FLUX_SCRATCH_MAX_NT = 2048;  // longest column of the kernel

struct FluxScratch {
  unsigned status;        // must read zero when the kernel starts
  unsigned clamp[2];      // columns capped at max_subcycles, largest count needed
  unsigned pad[61];       // keeps the twiddle area on its own 256-byte line
  float2 tw[FLUX_SCRATCH_MAX_NT];
};  // 16,640 bytes in all

static __device__ __align__(256) FluxScratch g_flux_scratch;

// Device address of the scratch in the current context.  Looked up on every
// call (cudaGetSymbolAddress allocates nothing): an address kept from an
// earlier call would be stale after cudaDeviceReset or under another context.
// The first call on a device also loads the library's kernels there, so make
// it before any stream capture.
static int flux_scratch_on_current_device(FluxScratch** out) {
  void* ptr = nullptr;
  CK(cudaGetSymbolAddress(&ptr, g_flux_scratch));
  *out = static_cast<FluxScratch*>(ptr);
  return ASG_OK;
}

extern "C" int asg_flux_columns_device(const float* d_in, float* d_out, int ncols, int nT,
                                       int flux, double n_coef, double dz, double dt,
                                       double beta_tvd, double cfl_target, int max_subcycles,
                                       void* stream) {
  g_err.clear();
  if (!d_in || !d_out || ncols <= 0 || nT < 3) return fail(ASG_ERR_ARG, "bad argument");
  if (nT > FLUX_SCRATCH_MAX_NT)
    return fail(ASG_ERR_SHAPE, "nT=%d exceeds the %d samples the fixed scratch holds", nT,
                FLUX_SCRATCH_MAX_NT);
  if (flux < ASG_FLUX_RUSANOV || flux > ASG_FLUX_KT_MINMOD)
    return fail(ASG_ERR_ARG, "unknown flux %d", flux);
  {
    // with overlapping ranges a block's output columns could overwrite input
    // columns that another block has not read yet
    const size_t bytes = (size_t)ncols * (size_t)nT * sizeof(float);
    const uintptr_t a = reinterpret_cast<uintptr_t>(d_in), b = reinterpret_cast<uintptr_t>(d_out);
    if (a < b + bytes && b < a + bytes)
      return fail(ASG_ERR_ARG, "d_in and d_out overlap (the step is not in place)");
  }
  {
    // an error left pending by earlier work is not this call's failure
    const cudaError_t pre = cudaPeekAtLastError();
    if (pre != cudaSuccess)
      return fail(ASG_ERR_CUDA, "a CUDA error was pending before this call: %s",
                  cudaGetErrorString(pre));
  }
  FluxScratch* scr = nullptr;
  CKS(flux_scratch_on_current_device(&scr));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CK(cudaMemsetAsync(scr, 0, 3 * sizeof(unsigned), st));  // status and cap counters
  TParams t;
  memset(&t, 0, sizeof(t));
  t.ncols = ncols;
  t.nT = nT;
  t.in_real = 1;
  t.real_in = const_cast<float*>(d_in);
  t.write_real = 1;
  t.real_out = d_out;
  t.tw = scr->tw;
  t.status = &scr->status;
  t.op.flux = flux;
  t.op.dz = (float)dz;
  t.op.beta_tvd = (float)beta_tvd;
  t.op.coef_rus = (float)(n_coef * dz / dt);
  t.op.coef_kt = (float)(n_coef / dt);
  t.op.n_rus64 = n_coef * dz / dt;
  t.op.n_kt64 = n_coef / dt;
  t.op.cfl_target = (float)cfl_target;
  t.op.max_subcycles = max_subcycles > 0 ? max_subcycles : 1024;
  t.op.subcycle_clamp = scr->clamp;
  GenPlan gp = make_gen_plan(nT);
  const int s = asg_launch_t(t, false, gp, st);
  if (s != ASG_OK) {
    const cudaError_t e = cudaGetLastError();  // this call's own launch error
    return fail(s, "flux kernel launch failed: %s", cudaGetErrorString(e));
  }
  return ASG_OK;
}

extern "C" int asg_flux_columns_device_clamped(void* stream, unsigned* n_clamped,
                                               unsigned* max_needed) {
  g_err.clear();
  if (!n_clamped) return fail(ASG_ERR_ARG, "null argument");
  FluxScratch* scr = nullptr;
  CKS(flux_scratch_on_current_device(&scr));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned c[2] = {0u, 0u};
  CK(cudaMemcpyAsync(c, scr->clamp, sizeof(c), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  *n_clamped = c[0];
  if (max_needed) *max_needed = c[1];
  return ASG_OK;
}

int asg_fail_message(int code, const char* msg) { return fail(code, "%s", msg); }

extern "C" const char* asg_last_error(void) { return g_err.c_str(); }

extern "C" const char* asg_version(void) {
  return "asg_gb300 1 (sm_103a; fast t sizes 128..2048, fast xy nY 64..512 with nX = 32*G)";
}
