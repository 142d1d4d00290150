// ati_api.cu — C ABI (include/ati.h) over the sm_103a kernels.
//
// One handle = one aerofoil case = every block of the multi-block grid in one
// GPU's HBM, with one CUDA stream.  The reference's MPI exchanges between
// blocks (src/Subroutines3D.f90:47-56, src/Main3D.f90:799-813 and 901-925,
// src/SingleTurbulence3D.f90:378-443) become reads of the neighbour block's
// face buffers inside the kernels.
//
// Arrays: an FP64 set (state, metrics, set-up work fields, the reference's
// rr/ss for the granular calls, and the FP64 stage intermediates) always
// exists; a case created with ATI_MIXED also owns an FP32 set of stage
// intermediates, metrics, face buffers and coefficients.
#include <cuda.h>  // CUtensorMap and its enumerations (the encoder itself is fetched from the driver at run time)
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <type_traits>
#include <memory>
#include <vector>

#include "../../include/ati.h"
#include "ati_internal.h"
#include "ati_kernels.h"
#include "ati_turb.h"
#include "ati_scheme.h"

using namespace ati;

namespace {

struct TaskRange {
  int off = 0, n = 0, maxline = 0;
};

constexpr int SPG_PER_BLOCK = 14;

thread_local std::string g_create_err;
thread_local std::string g_tma_err;  // a tensor-map encoding failure at creation

}  // namespace

struct ati_handle {
  ati_config_t cfg{};  // case 0; the numerics every case of a batch shares
  int nb = 0;
  bool mixed = false;
  std::vector<BlockDev> blk;
  SchemeHost sh{};     // case 0: scheme coefficients (shared) and its physics
  // a batch: cases 0..ncase-1, case c owns blocks [case_b0[c], case_b0[c] + 6)
  int ncase = 1;
  std::vector<ati_config_t> cfgs;
  std::vector<SchemeHost> shc;
  std::vector<int> case_b0;
  std::vector<TaskRange> tl_force_c;
  bool any_cfl = false;  // some case takes its dt from the CFL condition (dto < 0)
  bool tma[4] = {false, false, false, false};  // tensor maps exist for the mixed path's eta/zeta sweeps
  std::vector<TmaMap> htmaps;                   // host copy of the tensor maps (kept for the upload)
  bool tune = true;                             // time tile candidates at ati_init (ati_set_tuning)
  bool fused = false;                           // fused face chains (ati_set_options)
  bool fp64_at_point = true;                    // FP64 viscous fluxes with the stresses at the point (ati_set_options)
  unsigned spin_limit = 1u << 24;               // polls a device barrier wait may take (ati_set_spin_limit)
  int64_t *dcum = nullptr;                      // running face-line counts of the task list (fused chains)
  unsigned *dbar = nullptr;                     // grid-barrier counters of the fused chains
  int64_t task_lines(int off, int n) const {    // face lines of a task range
    int64_t t = 0;
    for (int q = off; q < off + n; q++) t += htasks[q].nline;
    return t;
  }
  std::vector<PTile> hpt;
  std::vector<LTile> hlt[4];
  std::vector<LTile> hlts[4];  // tiles of the segmented sweeps (mixed path), by class (segc)
  SegClass segc[4][SEG_NCLASS] = {};
  int nsegc[4] = {0, 0, 0, 0};
  size_t max_pt = 0, max_lt[4] = {0, 0, 0, 0};
  // point tiles of the candidate sizes (PT_CAND), uploaded once; pw_pt[kind] is a pointwise kernel's own timed
  // size (0: the shared queue of pt_points)
  std::vector<PTile> hptc[3];
  const PTile *dptc[3] = {nullptr, nullptr, nullptr};
  int pw_pt[PW_KINDS] = {};
  int sg_lines[4] = {XC_NL, XC_NL, SG_DEFAULT, SG_DEFAULT}, pt_points = PT_DEFAULT;  // tile shapes (timed at ati_init)
  int64_t N = 0, F = 0, nfac = 0, nsbcc = 0, nwall = 0;
  int maxlen[4] = {0, 0, 0, 0};
  int maxlines[4] = {0, 0, 0, 0};
  cudaStream_t st = nullptr;
  // side streams and events for the three directions' sweeps, which are independent within a stage
  cudaStream_t side[2] = {nullptr, nullptr};
  cudaEvent_t ev_fork = nullptr, ev_join[2] = {nullptr, nullptr};
  char *arena = nullptr;
  size_t arena_bytes = 0;
  Eng<double> ed{};  // FP64 arrays: set-up, granular calls, FP64 stage
  Eng<float> ef{};   // FP32 stage arrays (ATI_MIXED)
  double *rr = nullptr, *ss = nullptr;  // the reference's rr/ss (granular calls, set-up)
  double *fw1 = nullptr;                // FP64 forward scratch of the granular calls
  FaceTask *dtasks = nullptr;
  std::vector<FaceTask> htasks;
  TaskRange tl_mpigo, tl_mpigo_x, tl_gcbc, tl_gcbc_dir[4], tl_wall, tl_pack, tl_avg_dir[4], tl_force, tl_all;
  JunctionDev *djn = nullptr;
  int njct = 0, jnk = 0;
  double *area = nullptr, *wnor = nullptr, *dforce = nullptr, *dspg = nullptr;
  int64_t *dwoff = nullptr;
  std::vector<int> grid_set;
  bool inited = false;
  int64_t n_host = 0;
  std::string err;
  // CUDA graphs of one time step: [0] plain step, [1] step with a new dt target
  cudaGraphExec_t gexec[2] = {nullptr, nullptr};
  int64_t glaunches[2] = {0, 0};  // kernels held by each graph
  bool graphs_ok = true;
  int64_t steps_done = 0;
  // instrumentation
  int64_t launches = 0;
  bool profiling = false;
  double wait_timeout = 0.0;  // seconds a host wait may take (0: unbounded)
  struct Ev {
    cudaEvent_t a, b;
    int cls;
  };
  std::vector<Ev> ev_used, ev_free;
  double prof_ms[ATI_K_NSLOTS] = {0};
  int64_t prof_n[ATI_K_NSLOTS] = {0};
  // synthetic inflow turbulence: mode tables per case, gust points, their target deltas
  std::vector<float> hmodes;
  std::vector<TurbCase> htc;
  float *dmodes = nullptr, *ddelta = nullptr;
  TurbCase *dtc = nullptr;
  GustPt *dgust = nullptr;
  // the strict mode's FP64 synthesis: the gust points in FP64 and their target changes
  GustPt64 *dgust64 = nullptr;
  double *ddelta64 = nullptr;
  int64_t ngust = 0;
  // surface-pressure recorder (ring buffer of wall pressure on the mid-span lines)
  int probe_cap = 0;
  int64_t probe_npts = 0, probe_n0 = 0;
  double *probe_p = nullptr, *probe_t = nullptr;
};

static int autotune(ati_handle *h);

// error text for calls that have no handle (ati_last_error(NULL))
void ati_set_thread_error(const char *msg) { g_create_err = msg ? msg : ""; }
void ati_set_handle_error(ati_handle_t *h, const char *msg) {
  if (h) h->err = msg ? msg : "";
  else g_create_err = msg ? msg : "";
}

static int fail(ati_handle *h, int code, const std::string &msg) {
  if (h) h->err = msg;
  else g_create_err = msg;
  return code;
}

#define CK(call)                                                                      \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess) return fail(h, ATI_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

#define CKL()                                                                         \
  do {                                                                                \
    cudaError_t e_ = cudaGetLastError();                                              \
    if (e_ != cudaSuccess) return fail(h, ATI_ECUDA, std::string("kernel launch: ") + cudaGetErrorString(e_)); \
  } while (0)

// every launch site is wrapped in prof_begin/prof_end; without profiling
// this only counts launches
static void prof_begin(ati_handle *h, int cls) {
  h->launches++;
  if (!h->profiling) return;
  ati_handle::Ev e;
  if (!h->ev_free.empty()) {
    e = h->ev_free.back();
    h->ev_free.pop_back();
  } else {
    cudaEventCreate(&e.a);
    cudaEventCreate(&e.b);
  }
  e.cls = cls;
  cudaEventRecord(e.a, h->st);
  h->ev_used.push_back(e);
}
static void prof_end(ati_handle *h) {
  if (!h->profiling || h->ev_used.empty()) return;
  cudaEventRecord(h->ev_used.back().b, h->st);
}
static void prof_drain(ati_handle *h) {
  for (auto &e : h->ev_used) {
    float ms = 0.f;
    cudaEventSynchronize(e.b);
    cudaEventElapsedTime(&ms, e.a, e.b);
    h->prof_ms[e.cls] += ms;
    h->prof_n[e.cls] += 1;
    h->ev_free.push_back(e);
  }
  h->ev_used.clear();
}
#define PROF(h, cls, launch) \
  do {                        \
    prof_begin(h, cls);       \
    launch;                   \
    prof_end(h);              \
  } while (0)

static const FaceTask *tp(const ati_handle *h, const TaskRange &r) { return h->dtasks + r.off; }

static void ijk_host(const BlockDev &B, int nn, int &i1, int &i2, int &i3) {
  if (nn == 1) { i1 = B.lxi; i2 = B.let; i3 = B.lze; }
  else if (nn == 2) { i1 = B.let; i2 = B.lze; i3 = B.lxi; }
  else { i1 = B.lze; i2 = B.lxi; i3 = B.let; }
}

// ---- set-up kernels (compiled without FMA contraction) ---------------------------
namespace {

__device__ __forceinline__ int64_t sidx3(int lxi, int let, int i, int j, int k, int nn) {
  if (nn == 1) return ((int64_t)k * (let + 1) + j) * (lxi + 1) + i;
  if (nn == 2) return ((int64_t)j * (let + 1) + i) * (lxi + 1) + k;
  return ((int64_t)i * (let + 1) + k) * (lxi + 1) + j;
}

__device__ __forceinline__ void sface(const BlockDev &B, int nn, int ip, int jk, int &i, int &j, int &k) {
  int a1, a2;
  if (nn == 1) { a1 = B.lxi; a2 = B.let; }
  else if (nn == 2) { a1 = B.let; a2 = B.lze; }
  else { a1 = B.lze; a2 = B.lxi; }
  j = jk % (a2 + 1);
  k = jk / (a2 + 1);
  i = ip * a1;
}

// face unit normals (src/Main3D.f90:429-439)
__global__ void k_cm(Eng<double> c, const FaceTask *tasks) {
  const FaceTask T = tasks[blockIdx.y];
  const int jk = blockIdx.x * blockDim.x + threadIdx.x;
  if (jk >= T.nline) return;
  const BlockDev &B = c.blk[T.b];
  int i, j, k;
  sface(B, T.nn, T.ip, jk, i, j, k);
  const int64_t g = B.off + sidx3(B.lxi, B.let, i, j, k, T.nn), N = c.N, nbs = T.nline;
  const double *mt = T.nn == 1 ? c.xim : (T.nn == 2 ? c.etm : c.zem);
  const double y = c.yaco[g];
  const double r1 = y * mt[g], r2 = y * mt[g + N], r3 = y * mt[g + 2 * N];
  const double f = 1.0 / sqrt(r1 * r1 + r2 * r2 + r3 * r3);
  double *cm = const_cast<double *>(c.cm) + B.face_off[T.nn] * 6;
  cm[jk + nbs * (0 + 3 * T.ip)] = f * r1;
  cm[jk + nbs * (1 + 3 * T.ip)] = f * r2;
  cm[jk + nbs * (2 + 3 * T.ip)] = f * r3;
}

// GCBC weights (src/Main3D.f90:460-480): visit counts, then weights
__global__ void k_sbcc_count(Eng<double> c, const FaceTask *tasks, double *cnt) {
  const FaceTask T = tasks[blockIdx.y];
  const int jk = blockIdx.x * blockDim.x + threadIdx.x;
  if (jk >= T.nline) return;
  const BlockDev &B = c.blk[T.b];
  int i, j, k;
  sface(B, T.nn, T.ip, jk, i, j, k);
  const int iq = 1 - 2 * T.ip;
  for (int ii = 0; ii <= MBCI; ii++) atomicAdd(&cnt[B.off + sidx3(B.lxi, B.let, i + iq * ii, j, k, T.nn)], 1.0);
}

__global__ void k_sbcc_weight(Eng<double> c, const FaceTask *tasks, const double *cnt, double s1, double s2, double s3) {
  const FaceTask T = tasks[blockIdx.y];
  const int jk = blockIdx.x * blockDim.x + threadIdx.x;
  if (jk >= T.nline) return;
  const BlockDev &B = c.blk[T.b];
  int i, j, k;
  sface(B, T.nn, T.ip, jk, i, j, k);
  const int iq = 1 - 2 * T.ip;
  const double res = 1.0 / c.yaco[B.off + sidx3(B.lxi, B.let, i, j, k, T.nn)];
  const double sb[4] = {0.0, s1, s2, s3};
  double *sbcc = const_cast<double *>(c.sbcc);
  for (int ii = 0; ii <= MBCI; ii++) {
    const double w = ii == 0 ? res : res * sb[ii];
    sbcc[T.sbcc_off + (int64_t)jk * (MBCI + 1) + ii] = w / cnt[B.off + sidx3(B.lxi, B.let, i + iq * ii, j, k, T.nn)];
  }
}

// sponge coefficients (spongeup, src/SingleTurbulence3D.f90:209-249); spg per
// block: [0..2] nsz(0,:)*szr(0,:), [3..5] szp(0,:), [6..8] nsz(1,:)*szr(1,:), [9..11] szp(1,:),
// [12] szco, [13] domlen of the block's case
__global__ void k_sponge(Eng<double> c, const double *xyz, const double *spg, double pi) {
  const BlockDev &B = c.blk[blockIdx.y];
  const double *P = spg + SPG_PER_BLOCK * blockIdx.y;
  const double szco = P[12], domlen = P[13];
  const int64_t N = c.N;
  const double ra1 = 0.25, ra2 = pi / (2.0 * domlen);
  double *asz = const_cast<double *>(c.asz), *bsz = const_cast<double *>(c.bsz);
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < B.npts; l += (int64_t)gridDim.x * blockDim.x) {
    const int64_t g = B.off + l;
    double r[3];
    for (int q = 0; q < 3; q++) {
      const double x = xyz[g + q * N];
      r[q] = P[q] * fmax(P[3 + q] - x, 0.0) + P[6 + q] * fmax(x - P[9 + q], 0.0);
    }
    const double sig = szco * (1.0 - 0.125 * (1.0 + cos(pi * r[0])) * (1.0 + cos(pi * r[1])) * (1.0 + cos(pi * r[2])));
    const double lam = ra1 + 0.5 * (1.0 - ra1) * (1.0 + cos(ra2 * (fmin(xyz[g], domlen) + domlen)));
    if (sig > 0.0) {
      const double res = 1.0 / c.yaco[g];
      asz[g] = res * sig * lam;
      bsz[g] = res * c.sc[B.cs].hamm1 * sig;
    } else {
      asz[g] = 0.0;
      bsz[g] = 0.0;
    }
  }
}

// wall area and normals (wallArea/walldir, src/rpt.f90:774-864), list order
// ll = k*(lxi+1) + i of the wall row
__global__ void k_wall_geom(Eng<double> c, const FaceTask *tasks, const int64_t *woff, double *area, double *wnor) {
  const FaceTask T = tasks[blockIdx.y];
  const BlockDev &B = c.blk[T.b];
  const int64_t nw = T.nline, N = c.N;
  const int64_t ll = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (ll >= nw) return;
  const int k = (int)(ll / (B.lxi + 1)), i = (int)(ll % (B.lxi + 1));
  const int j = T.ip * B.let;
  const double coef = T.ip == 0 ? 1.0 : -1.0;
  const int64_t g = B.off + ((int64_t)k * (B.let + 1) + j) * (B.lxi + 1) + i;
  const double a1 = c.qo[g], a3 = c.qo[g + 2 * N], b1 = c.qa[g], b3 = c.qa[g + 2 * N], d1 = c.de[g], d3 = c.de[g + 2 * N];
  const double g11 = a1 * a1 + b1 * b1 + d1 * d1, g33 = a3 * a3 + b3 * b3 + d3 * d3, g13 = a1 * a3 + b1 * b3 + d1 * d3;
  double ar = sqrt(g11 * g33 - g13 * g13);
  if (i == 0) ar = ar * 0.5;
  else if (i == B.lxi) ar = ar * 0.5;
  if (k == 0) ar = ar * 0.5;
  else if (k == B.lze) ar = ar * 0.5;
  const int64_t o = woff[blockIdx.y];
  area[o + ll] = ar;
  const double e1 = c.etm[g], e2 = c.etm[g + N], e3 = c.etm[g + 2 * N];
  const double tmp = coef / sqrt(e1 * e1 + e2 * e2 + e3 * e3);
  wnor[3 * o + ll] = e1 * tmp;
  wnor[3 * o + nw + ll] = e2 * tmp;
  wnor[3 * o + 2 * nw + ll] = e3 * tmp;
}

// initial condition of initialo (src/SingleTurbulence3D.f90:203)
__global__ void k_ic(Eng<double> c) {
  const int64_t N = c.N;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < N; g += (int64_t)gridDim.x * blockDim.x) {
    c.qa[g] = c.sc->rhooo;
    c.qa[g + N] = 0.0;
    c.qa[g + 2 * N] = 0.0;
    c.qa[g + 3 * N] = 0.0;
    c.qa[g + 4 * N] = c.sc->hamm1 * c.sc->poo;
  }
}

// FP64 -> FP32 copies for the mixed engine
__global__ void k_to_float(const double *src, float *dst, int64_t n) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x)
    dst[g] = (float)src[g];
}
// pressure coefficient of the current qa (getCp, src/rptPost.f90:1456-1465), one grid row per block
__global__ void k_cp(Eng<double> c, double *cp) {
  const BlockDev &B = c.blk[blockIdx.y];
  const Scheme &S = c.sc[B.cs];
  const int64_t N = c.N;
  const double ra0 = 2.0 / (S.amachoo * S.amachoo);
  for (int64_t g = B.off + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < B.off + B.npts;
       g += (int64_t)gridDim.x * blockDim.x) {
    const double q1 = c.qa[g], q2 = c.qa[g + N], q3 = c.qa[g + 2 * N], q4 = c.qa[g + 3 * N];
    const double pp = S.gamm1 * (c.qa[g + 4 * N] - 0.5 * (q2 * q2 + q3 * q3 + q4 * q4) / q1);
    cp[g] = (pp - S.poo) * ra0;
  }
}

// one record of the wall pressure (FP64, from qa) on the mid-span line of every
// wall face; record slot (n - n0 - 1) mod cap, n = steps done (already advanced)
__global__ void k_wall_probe(Eng<double> c, const FaceTask *tasks, int ntask, int64_t n0, int cap, int64_t npts,
                             double *pbuf, double *tbuf) {
  const Scheme &S = *c.sc;
  const int64_t N = c.N;
  const int64_t r = (c.scal->n - n0 - 1) % cap;
  int64_t base = 0;
  for (int q = 0; q < ntask; q++) {
    const FaceTask T = tasks[q];
    const BlockDev &B = c.blk[T.b];
    const int nx = B.lxi + 1;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nx; i += gridDim.x * blockDim.x) {
      const int j = T.ip * B.let, k = B.lze / 2;
      const int64_t g = B.off + ((int64_t)k * (B.let + 1) + j) * nx + i;
      const double q1 = c.qa[g], q2 = c.qa[g + N], q3 = c.qa[g + 2 * N], q4 = c.qa[g + 3 * N];
      pbuf[r * npts + base + i] = S.gamm1 * (c.qa[g + 4 * N] - 0.5 * (q2 * q2 + q3 * q3 + q4 * q4) / q1);
    }
    base += nx;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) tbuf[r] = c.scal->timo;
}

// sign of the Jacobian over each block: bit 0 some J > 0, bit 1 some J < 0, bit 2 J = 0 or not finite
__global__ void k_jac_sign(Eng<double> c, int *flags) {
  const BlockDev &B = c.blk[blockIdx.y];
  int f = 0;
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < B.npts; l += (int64_t)gridDim.x * blockDim.x) {
    const double y = c.yaco[B.off + l];
    if (y > 0.0 && y < 1e300) f |= 1;
    else if (y < 0.0 && y > -1e300) f |= 2;
    else f |= 4;
  }
  if (f) atomicOr(&flags[blockIdx.y], f);
}

__global__ void k_to_double(const float *src, double *dst, int64_t n, double add) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x)
    dst[g] = (double)src[g] + add;
}

}  // namespace

// ---- topology: domdcomp (src/SingleTurbulence3D.f90:121-164), npc = 1 ---------
static void topology(const ati_config_t &cfg, int mb, BlockDev &B, int nbcs[4], int nbce[4]) {
  const int bkx = cfg.bkx, bky = cfg.bky, mbk = cfg.bkx * cfg.bky * cfg.bkz - 1;
  const int bcw = 20 + 5 * cfg.nviscous, bcinout = 10, bcperiod = 45, bcinter = 30;
  int ms[4], me[4];
  const int ll = mb % bkx;
  if (ll == 0) { ms[1] = mb + (bkx - 1); me[1] = mb + 1; nbcs[1] = bcinout; nbce[1] = bcinter; }
  else if (ll == bkx - 1) { ms[1] = mb - 1; me[1] = mb - (bkx - 1); nbcs[1] = bcinter; nbce[1] = bcinout; }
  else { ms[1] = mb - 1; me[1] = mb + 1; nbcs[1] = bcinter; nbce[1] = bcinter; }
  if (mb < bkx) { ms[2] = mb + bkx * (bky - 1); me[2] = mb + bkx; nbcs[2] = bcinout; nbce[2] = bcinter; }
  else if (mb > mbk - bkx) { ms[2] = mb - bkx; me[2] = mb - bkx * (bky - 1); nbcs[2] = bcinter; nbce[2] = bcinout; }
  else { ms[2] = mb - bkx; me[2] = mb + bkx; nbcs[2] = bcinter; nbce[2] = bcinter; }
  nbcs[3] = bcperiod; nbce[3] = bcperiod; ms[3] = mb; me[3] = mb;
  if (mb == 1) nbce[2] = bcw;
  if (mb == 4) nbcs[2] = bcw;
  for (int nn = 1; nn <= 3; nn++) {
    B.nbc[0][nn] = nbcs[nn]; B.nbc[1][nn] = nbce[nn];
    B.ncd[0][nn] = ms[nn]; B.ncd[1][nn] = me[nn];
    for (int ip = 0; ip <= 1; ip++) {
      const int np = B.nbc[ip][nn];
      B.ndf[ip][nn] = (np == 35 || np == 40 || np == 45) ? 1 : 0;
    }
  }
}

static bool is_gcbc(int np) { return np == 10 || np == 20 || np == 25 || np == 30; }
static bool is_wall(int np) { return np == 20 || np == 25; }
static bool is_avg(int np) { return np == 30 || np == 35 || np == 45; }

// ---- lifetime --------------------------------------------------------------
extern "C" int ati_abi_version(void) { return ATI_ABI_VERSION; }

extern "C" const char *ati_last_error(const ati_handle_t *h) { return h ? h->err.c_str() : g_create_err.c_str(); }

// the candidate point-tile sizes of the pointwise kernels
static const int PT_CAND[3] = {PT_MIN, 4 * PT_MIN, PT_MAX};

// point tiles of pt points, each within one case
static void point_tiles(const ati_handle *h, int pt, std::vector<PTile> &out) {
  const int nbc = h->nb / h->ncase;
  out.clear();
  for (int cs = 0; cs < h->ncase; cs++) {
    const int64_t g0 = h->blk[h->case_b0[cs]].off;
    const BlockDev &Bl = h->blk[h->case_b0[cs] + nbc - 1];
    const int64_t g1 = Bl.off + Bl.npts;
    for (int64_t g = g0; g < g1; g += pt) out.push_back(PTile{cs, 0, g, std::min(g + pt, g1)});
  }
}

// point every engine's pointwise kinds at their own tiles (pw_pt), or at the shared queue
static void apply_pw_tiles(ati_handle *h) {
  for (int w = 0; w < PW_KINDS; w++) {
    const PTile *q = nullptr;
    int n = 0;
    for (int c = 0; c < 3; c++)
      if (h->pw_pt[w] == PT_CAND[c]) { q = h->dptc[c]; n = (int)h->hptc[c].size(); }
    h->ed.ptk[w] = h->ef.ptk[w] = q;
    h->ed.nptk[w] = h->ef.nptk[w] = n;
  }
}

// work queues: point tiles of pt points of one case, line tiles of one block
// (XC_NL xi lines, sg2 eta lines, sg3 zeta lines)
static void make_tiles(ati_handle *h, int sg2, int sg3, int pt) {
  point_tiles(h, pt, h->hpt);
  for (int nn = 1; nn <= 3; nn++) {
    h->hlt[nn].clear();
    const int step = nn == 1 ? XC_NL : (nn == 2 ? sg2 : sg3);
    for (int gb = 0; gb < h->nb; gb++)
      for (int t0 = 0; t0 < h->blk[gb].nbsize[nn]; t0 += step) h->hlt[nn].push_back(LTile{gb, t0});
  }
  h->sg_lines[2] = sg2;
  h->sg_lines[3] = sg3;
  h->pt_points = pt;
}

// copy the host work queues into the device arrays and point both engines at them
static int upload_tiles(ati_handle *h) {
  CK(cudaMemcpyAsync(const_cast<PTile *>(h->ed.pt), h->hpt.data(), sizeof(PTile) * h->hpt.size(), cudaMemcpyHostToDevice,
                     h->st));
  for (int nn = 1; nn <= 3; nn++)
    CK(cudaMemcpyAsync(const_cast<LTile *>(h->ed.lt[nn]), h->hlt[nn].data(), sizeof(LTile) * h->hlt[nn].size(),
                       cudaMemcpyHostToDevice, h->st));
  CK(cudaStreamSynchronize(h->st));
  h->ed.npt = h->ef.npt = (int)h->hpt.size();
  for (int nn = 1; nn <= 3; nn++) h->ed.nlt[nn] = h->ef.nlt[nn] = (int)h->hlt[nn].size();
  for (int nn = 0; nn < 4; nn++) h->ed.sg_lines[nn] = h->ef.sg_lines[nn] = h->sg_lines[nn];
  return ATI_OK;
}

// cuTensorMapEncodeTiled, fetched through the runtime (the library has no link-time dependency on the driver)
using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiled encode_tiled() {
  static EncodeTiled fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      return (EncodeTiled) nullptr;
    }
    return (EncodeTiled)p;
  }();
  return fn;
}

// Can every block's FP32 planes of direction nn (2: eta, 3: zeta) be described by a tensor map?  The base of each
// block's plane and every stride must be a multiple of 16 bytes (N, the block offsets and the row or plane sizes
// multiples of 4 floats), and a box spans the whole line (at most 256 points).
static bool tma_geometry(const ati_handle *h, int nn) {
  if (!h->mixed || h->N % 4 != 0) return false;
  for (int b = 0; b < h->nb; b++) {
    const BlockDev &B = h->blk[b];
    const int64_t nx = B.lxi + 1, ny = B.let + 1, nz = B.lze + 1;
    if (B.off % 4 != 0) return false;
    if (nn == 2 && (nx % 4 != 0 || ny > 256)) return false;
    if (nn == 3 && ((nx * ny) % 4 != 0 || nz > 256)) return false;
  }
  return encode_tiled() != nullptr;
}

// The tensor maps of the mixed path's eta/zeta derivative sweeps: per array (0: the four primitive planes u, v, w,
// T, plane stride N; 1: the five flux planes of direction nn, stride 3 N), direction and block.  eta lines of a
// block: 4-D (xi, eta, zeta, field), box 32 x ny x 1 x 1; zeta lines: 3-D (xi-eta plane, zeta, field), box 32 x nz
// x 1.  Tile-mode boxes, no swizzle, out-of-bounds points read as zero.
static int encode_tmaps(ati_handle *h, std::vector<TmaMap> &out) {
  const int64_t N = h->N;
  out.assign((size_t)4 * h->nb, TmaMap{});
  EncodeTiled enc = encode_tiled();
  for (int arr = 0; arr < 2; arr++)
    for (int nn = 2; nn <= 3; nn++) {
      if (!h->tma[nn]) continue;
      const int nf = arr == 0 ? 4 : 5;
      const int64_t fs = arr == 0 ? N : 3 * N;
      float *plane = arr == 0 ? h->ef.prim : h->ef.flx + (nn - 1) * N;
      for (int b = 0; b < h->nb; b++) {
        const BlockDev &B = h->blk[b];
        const uint64_t nx = B.lxi + 1, ny = B.let + 1, nz = B.lze + 1;
        void *g = plane + B.off;
        CUtensorMap *m = reinterpret_cast<CUtensorMap *>(&out[(size_t)(arr * 2 + nn - 2) * h->nb + b]);
        CUresult r;
        if (nn == 2) {
          const cuuint64_t dim[4] = {nx, ny, nz, (cuuint64_t)nf};
          const cuuint64_t str[3] = {nx * 4, nx * ny * 4, (cuuint64_t)fs * 4};
          const cuuint32_t box[4] = {(cuuint32_t)SEG_LINES, (cuuint32_t)ny, 1, 1}, es[4] = {1, 1, 1, 1};
          r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, g, dim, str, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        } else {
          const cuuint64_t dim[3] = {nx * ny, nz, (cuuint64_t)nf};
          const cuuint64_t str[2] = {nx * ny * 4, (cuuint64_t)fs * 4};
          const cuuint32_t box[3] = {(cuuint32_t)SEG_LINES, (cuuint32_t)nz, 1}, es[3] = {1, 1, 1};
          r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, g, dim, str, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        }
        if (r != CUDA_SUCCESS)
          return fail(h, ATI_ECUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ") for block " +
                                        std::to_string(b) + ", direction " + std::to_string(nn));
      }
    }
  return ATI_OK;
}

static int build_tables(ati_handle *h, std::vector<double> &facd, std::vector<double> &facf, std::vector<double> &spg) {
  int64_t off = 0, face = 0, fac = 0;
  spg.assign((size_t)SPG_PER_BLOCK * h->nb, 0.0);
  const int nbc = h->cfg.bkx * h->cfg.bky * h->cfg.bkz;  // blocks per case
  h->case_b0.assign(h->ncase, 0);
  for (int gb = 0; gb < h->nb; gb++) {
    const int cs = gb / nbc, mb = gb % nbc, b0 = cs * nbc;
    const ati_config_t &cfg = h->cfgs[cs];
    h->case_b0[cs] = b0;
    BlockDev &B = h->blk[gb];
    std::memset(&B, 0, sizeof(B));
    const int i = mb % cfg.bkx, j = (mb / cfg.bkx) % cfg.bky, k = mb / (cfg.bkx * cfg.bky);
    B.lxi = cfg.lxibk[i]; B.let = cfg.letbk[j]; B.lze = cfg.lzebk[k];
    if (B.lxi < 6 || B.let < 6 || B.lze < 12) return fail(h, ATI_EINVAL, "block sizes: lxi, let >= 6 and lze >= 12 required");
    int nbcs[4], nbce[4];
    topology(cfg, mb, B, nbcs, nbce);
    for (int nn = 1; nn <= 3; nn++) { B.ncd[0][nn] += b0; B.ncd[1][nn] += b0; }  // neighbours within the case
    B.cs = cs;
    B.off = off;
    B.npts = (int64_t)(B.lxi + 1) * (B.let + 1) * (B.lze + 1);
    off += B.npts;
    for (int nn = 1; nn <= 3; nn++) {
      int a1, a2, a3;
      ijk_host(B, nn, a1, a2, a3);
      B.nbsize[nn] = (a2 + 1) * (a3 + 1);
      B.face_off[nn] = face;
      face += B.nbsize[nn];
      B.fac_off[nn] = fac;
      fac += a1 + 1;
      h->maxlines[nn] = std::max(h->maxlines[nn], B.nbsize[nn]);
      h->maxlen[nn] = std::max(h->maxlen[nn], a1 + 1);
    }
    // sponge set-up constants (spongeup, src/SingleTurbulence3D.f90:211-222);
    // the literal 0.7e0 is default (single) precision in the reference
    const double p7 = (double)0.7f, dl = cfg.domlen;
    double szr[2][4] = {{0, 1 / cfg.szth1, 1 / cfg.szth2, 0}, {0, 1 / (cfg.szth1 + cfg.szxt), 1 / cfg.szth2, 0}};
    double szp[2][4] = {{0, -p7 * dl + cfg.szth1, -p7 * dl + cfg.szth2, 0},
                        {0, dl - cfg.szth1, dl + cfg.szxt - cfg.szth2, 0}};
    for (int nn = 1; nn <= 3; nn++) {
      const double n0 = nbcs[nn] == 10 ? 1.0 : 0.0, n1 = nbce[nn] == 10 ? 1.0 : 0.0;
      spg[SPG_PER_BLOCK * gb + (nn - 1)] = n0 * szr[0][nn];
      spg[SPG_PER_BLOCK * gb + 3 + (nn - 1)] = szp[0][nn];
      spg[SPG_PER_BLOCK * gb + 6 + (nn - 1)] = n1 * szr[1][nn];
      spg[SPG_PER_BLOCK * gb + 9 + (nn - 1)] = szp[1][nn];
    }
    spg[SPG_PER_BLOCK * gb + 12] = cfg.szco;
    spg[SPG_PER_BLOCK * gb + 13] = cfg.domlen;
  }
  h->N = off;
  h->F = face;
  h->nfac = fac;
  facd.assign((size_t)fac * 5, 0.0);
  facf.assign((size_t)fac * 5, 0.0);
  for (int mb = 0; mb < h->nb; mb++) {
    const BlockDev &B = h->blk[mb];
    for (int nn = 1; nn <= 3; nn++) {
      int a1, a2, a3;
      ijk_host(B, nn, a1, a2, a3);
      const int ns = B.ndf[0][nn], ne = B.ndf[1][nn];
      penta_factors(h->sh.albed[ns], h->sh.albed[ne], 0.5862704032801503, 0.09549533555017055, a1 + 1,
                    &facd[(size_t)B.fac_off[nn] * 5]);
      penta_factors(h->sh.albef[ns], h->sh.albef[ne], h->sh.alphf, h->sh.betf, a1 + 1, &facf[(size_t)B.fac_off[nn] * 5]);
    }
  }
  // face task lists
  auto &T = h->htasks;
  T.clear();
  auto add = [&](TaskRange &r, auto pred) {
    r.off = (int)T.size();
    for (int mb = 0; mb < h->nb; mb++)
      for (int nn = 1; nn <= 3; nn++)
        for (int ip = 0; ip <= 1; ip++) {
          const BlockDev &B = h->blk[mb];
          if (!pred(B, nn, ip)) continue;
          FaceTask t{};
          t.b = mb; t.nn = nn; t.ip = ip; t.bc = B.nbc[ip][nn]; t.nb_b = B.ncd[ip][nn];
          t.nline = B.nbsize[nn]; t.sbcc_off = -1; t.wall_off = -1;
          T.push_back(t);
          r.maxline = std::max(r.maxline, t.nline);
        }
    r.n = (int)T.size() - r.off;
  };
  add(h->tl_mpigo, [](const BlockDev &B, int nn, int ip) { return B.ndf[ip][nn] == 1; });
  // the mixed path's segmented derivative sweeps close faces periodic onto their own block themselves
  add(h->tl_mpigo_x, [h](const BlockDev &B, int nn, int ip) {
    const int gb = (int)(&B - h->blk.data());
    return B.ndf[ip][nn] == 1 && !(B.nbc[ip][nn] == 45 && B.ncd[ip][nn] == gb);
  });
  add(h->tl_gcbc, [](const BlockDev &B, int nn, int ip) { return is_gcbc(B.nbc[ip][nn]); });
  for (int d = 1; d <= 3; d++)
    add(h->tl_gcbc_dir[d], [d](const BlockDev &B, int nn, int ip) { return nn == d && is_gcbc(B.nbc[ip][nn]); });
  add(h->tl_wall, [](const BlockDev &B, int nn, int ip) { return is_wall(B.nbc[ip][nn]); });
  add(h->tl_pack, [](const BlockDev &B, int nn, int ip) { return is_avg(B.nbc[ip][nn]); });
  for (int d = 1; d <= 3; d++)
    add(h->tl_avg_dir[d], [d](const BlockDev &B, int nn, int ip) { return nn == d && is_avg(B.nbc[ip][nn]); });
  add(h->tl_all, [](const BlockDev &, int, int) { return true; });
  const int bcw = 20 + 5 * h->cfg.nviscous;
  add(h->tl_force, [bcw](const BlockDev &B, int nn, int ip) {
    if (nn != 2) return false;
    if (ip == 0) return B.nbc[0][2] == bcw;
    return B.nbc[0][2] != bcw && B.nbc[1][2] == bcw;
  });
  // GCBC weight and wall offsets, keyed by (block, nn, ip)
  std::vector<int64_t> sb_off((size_t)h->nb * 8, -1), w_off((size_t)h->nb * 8, -1);
  int64_t ns = 0, nw = 0;
  for (int mb = 0; mb < h->nb; mb++)
    for (int nn = 1; nn <= 3; nn++)
      for (int ip = 0; ip <= 1; ip++) {
        const BlockDev &B = h->blk[mb];
        const int np = B.nbc[ip][nn];
        if (is_gcbc(np)) { sb_off[mb * 8 + nn * 2 + ip] = ns; ns += (int64_t)B.nbsize[nn] * (MBCI + 1); }
        if (is_wall(np)) { w_off[mb * 8 + nn * 2 + ip] = nw; nw += B.nbsize[nn]; }
      }
  for (auto &t : T) {
    t.sbcc_off = sb_off[t.b * 8 + t.nn * 2 + t.ip];
    t.wall_off = w_off[t.b * 8 + t.nn * 2 + t.ip];
  }
  h->nsbcc = ns;
  h->nwall = nw;
  // wall faces of each case (contiguous: the task lists follow the block order)
  h->tl_force_c.assign(h->ncase, TaskRange{});
  for (int q = 0; q < h->tl_force.n; q++) {
    const int cs = h->blk[T[h->tl_force.off + q].b].cs;
    TaskRange &r = h->tl_force_c[cs];
    if (r.n == 0) r.off = h->tl_force.off + q;
    r.n++;
    r.maxline = std::max(r.maxline, T[h->tl_force.off + q].nline);
  }
  // work queues, at their finest tiles (the device arrays are sized for these)
  make_tiles(h, SG_MIN, SG_MIN, PT_MIN);
  h->max_pt = h->hpt.size();
  for (int c = 0; c < 3; c++) point_tiles(h, PT_CAND[c], h->hptc[c]);
  for (int nn = 1; nn <= 3; nn++) h->max_lt[nn] = h->hlt[nn].size();
  make_tiles(h, SG_DEFAULT, SG_DEFAULT, PT_DEFAULT);
  for (int nn = 2; nn <= 3; nn++) h->tma[nn] = tma_geometry(h, nn);
  for (int nn = 1; nn <= 3; nn++) {
    if (h->mixed && h->maxlen[nn] > SEG_LMAX)
      return fail(h, ATI_EINVAL, "mixed precision: lines of up to " + std::to_string(SEG_LMAX) + " points");
    // classes of the segmented sweeps: the distinct segment counts of the blocks' lines, ascending (beyond
    // SEG_NCLASS the largest counts share the last class, whose CTAs then idle a warp for the shorter lines)
    auto len = [&](const BlockDev &B) { return nn == 1 ? B.lxi + 1 : (nn == 2 ? B.let + 1 : B.lze + 1); };
    std::vector<int> counts;
    for (int gb = 0; gb < h->nb; gb++) counts.push_back(seg_count(len(h->blk[gb])));
    std::sort(counts.begin(), counts.end());
    counts.erase(std::unique(counts.begin(), counts.end()), counts.end());
    auto cls = [&](int L) {
      const int r = (int)(std::lower_bound(counts.begin(), counts.end(), seg_count(L)) - counts.begin());
      return std::min(r, SEG_NCLASS - 1);
    };
    h->nsegc[nn] = std::min((int)counts.size(), SEG_NCLASS);
    h->hlts[nn].clear();
    for (int c = 0; c < h->nsegc[nn]; c++) {
      SegClass C{(int)h->hlts[nn].size(), 0, 0, 1};
      for (int gb = 0; gb < h->nb; gb++)
        if (cls(len(h->blk[gb])) == c) C.maxlen = std::max(C.maxlen, len(h->blk[gb]));
      C.groups = seg_groups(C.maxlen);
      for (int gb = 0; gb < h->nb; gb++) {
        if (cls(len(h->blk[gb])) != c) continue;
        const BlockDev &B = h->blk[gb];
        // tiles of one-group CTAs come in runs of even length (a padding tile past the block's lines, on which
        // every CTA idles, evens an odd run): the paired sweeps take two consecutive tiles of a run a CTA
        auto even_run = [&](size_t start) {
          if (C.groups == 1 && (h->hlts[nn].size() - start) % 2) h->hlts[nn].push_back(LTile{gb, (int)B.nbsize[nn]});
        };
        if (nn == 2 && h->tma[2]) {
          // TMA eta tiles: the lines of one grid row (fixed zeta), from a multiple of 32 points along xi
          for (int ze = 0; ze <= B.lze; ze++) {
            const size_t start = h->hlts[nn].size();
            for (int xi0 = 0; xi0 <= B.lxi; xi0 += SEG_LINES * C.groups)
              h->hlts[nn].push_back(LTile{gb, ze * (B.lxi + 1) + xi0});
            even_run(start);
          }
          continue;
        }
        const size_t start = h->hlts[nn].size();
        for (int t0 = 0; t0 < B.nbsize[nn]; t0 += SEG_LINES * C.groups) h->hlts[nn].push_back(LTile{gb, t0});
        even_run(start);
      }
      C.n = (int)h->hlts[nn].size() - C.off;
      h->segc[nn][c] = C;
    }
  }
  return ATI_OK;
}

// Row tables of the segmented solves (k_sweep_seg), SEG_RT floats per row of
// one table of LU factors: the factors with the entries a row does not have
// set to zero, and the responses (g, h) = forward values of the row's segment
// from incoming v(s0-2) = 1 and from v(s0-1) = 1, (G, H) = its back-substituted
// values from b(s1) = 1 and from b(s1+1) = 1.  The first segment receives no
// forward values and the last no backward ones: their responses stay zero.
static void seg_tables(const ati_handle *h, const std::vector<double> &fac, std::vector<float> &out) {
  out.assign((size_t)h->nfac * SEG_RT, 0.f);
  for (int gb = 0; gb < h->nb; gb++) {
    const BlockDev &B = h->blk[gb];
    for (int nn = 1; nn <= 3; nn++) {
      const int L = nn == 1 ? B.lxi + 1 : (nn == 2 ? B.let + 1 : B.lze + 1);
      const double *fc = &fac[(size_t)B.fac_off[nn] * 5];
      float *o = &out[(size_t)B.fac_off[nn] * SEG_RT];
      auto l0 = [&](int i) { return i >= 2 ? fc[i * 5 + 0] : 0.0; };
      auto l1 = [&](int i) { return i >= 1 ? fc[i * 5 + 1] : 0.0; };
      auto c3 = [&](int i) { return i <= L - 2 ? fc[i * 5 + 3] : 0.0; };
      auto c4 = [&](int i) { return i <= L - 3 ? fc[i * 5 + 4] : 0.0; };
      for (int i = 0; i < L; i++) {
        float *r = o + (size_t)i * SEG_RT;
        r[0] = (float)l0(i); r[1] = (float)l1(i);
        r[6] = (float)fc[i * 5 + 2]; r[7] = (float)c3(i); r[10] = (float)c4(i);
      }
      const int S = seg_count(L);
      for (int k = 0; k < S; k++) {
        const int s0 = seg_start(k, L, S), s1 = seg_start(k + 1, L, S);
        if (k > 0) {
          double g2 = 1, g1 = 0, h2 = 0, h1 = 1;  // rows i-2, i-1
          for (int i = s0; i < s1; i++) {
            const double g = -l0(i) * g2 - l1(i) * g1, hh = -l0(i) * h2 - l1(i) * h1;
            o[(size_t)i * SEG_RT + 4] = (float)g;
            o[(size_t)i * SEG_RT + 5] = (float)hh;
            g2 = g1; g1 = g; h2 = h1; h1 = hh;
          }
        }
        if (k < S - 1) {
          double G1 = 1, G2 = 0, H1 = 0, H2 = 1;  // rows i+1, i+2
          for (int i = s1 - 1; i >= s0; i--) {
            const double G = -c3(i) * G1 - c4(i) * G2, H = -c3(i) * H1 - c4(i) * H2;
            o[(size_t)i * SEG_RT + 8] = (float)G;
            o[(size_t)i * SEG_RT + 9] = (float)H;
            G2 = G1; G1 = G; H2 = H1; H1 = H;
          }
        }
      }
    }
  }
}

// Dense zeta derivative operators of the mixed path (k_sweep_dense): on a block whose two zeta faces are periodic
// onto the block itself, the derivative of a zeta line is a fixed linear map d = M f of the line's L values: the
// closure values of the line ends are sums over the other end of the same line (k_mpigo's closure, taken inside the
// sweep), the end rows those of deriv's closures (line_ends), the interior rows the compact right-hand side, then
// the LU solve (src/Subroutines3D.f90:84-141).  Column j of M is that algorithm applied in FP64 to the unit line
// e_j; M is returned in FP64 (rounded to FP32 for the device), row-major in DENSE_MAX x DENSE_MAX storage per
// block.  Returns the largest line length, or 0 if some block's zeta lines do not qualify (a face of another kind,
// lines outside LMD + 2..DENSE_MAX).
static int dense_zeta(const ati_handle *h, const std::vector<double> &fac, std::vector<double> &out) {
  const Scheme &S = h->sh.s;
  int lmax = 0;
  for (int gb = 0; gb < h->nb; gb++) {
    const BlockDev &B = h->blk[gb];
    const int L = B.lze + 1;
    for (int ip = 0; ip <= 1; ip++)
      if (B.ndf[ip][3] != 1 || B.nbc[ip][3] != 45 || B.ncd[ip][3] != gb) return 0;
    if (L < LMD + 2 || L > DENSE_MAX) return 0;  // the closure sums reach LMD + 1 points in from the far end
    lmax = std::max(lmax, L);
  }
  out.assign((size_t)h->nb * DENSE_MAX * DENSE_MAX, 0.0);
  std::vector<double> f(DENSE_MAX), r(DENSE_MAX), v(DENSE_MAX), b(DENSE_MAX + 2);
  for (int gb = 0; gb < h->nb; gb++) {
    const BlockDev &B = h->blk[gb];
    const int L = B.lze + 1;
    const double *fc = &fac[(size_t)B.fac_off[3] * 5];
    for (int j = 0; j < L; j++) {
      std::fill(f.begin(), f.end(), 0.0);
      f[j] = 1.0;
      double rl[6];
      auto closure = [&](int r0, int dir, double *o) {  // the sums k_mpigo forms for the periodic face
        double c0 = 0, c1 = 0;
        for (int i = 0; i <= LMD; i++) {
          c0 += S.pbco[0][0][i] * f[r0 + i * dir];
          c1 += S.pbco[0][1][i] * f[r0 + i * dir];
        }
        o[0] = c0; o[1] = c1; o[2] = f[r0];
      };
      closure(L - 2, -1, rl);
      closure(1, 1, rl + 3);
      double s0 = 0, s1 = 0, e0 = 0, e1 = 0;
      for (int q = 0; q <= LMD; q++) {
        s0 += S.pbci[0][0][q] * f[q];
        s1 += S.pbci[0][1][q] * f[q];
        e0 += S.pbci[0][0][q] * f[L - 1 - q];
        e1 += S.pbci[0][1][q] * f[L - 1 - q];
      }
      r[0] = s0 + rl[0];
      r[1] = s1 + rl[1];
      r[2] = S.aa * (f[3] - f[1]) + S.ab * (f[4] - f[0]) + S.ac * (f[5] - rl[2]);
      for (int i = 3; i < L - 3; i++)
        r[i] = S.aa * (f[i + 1] - f[i - 1]) + S.ab * (f[i + 2] - f[i - 2]) + S.ac * (f[i + 3] - f[i - 3]);
      r[L - 3] = S.aa * (f[L - 2] - f[L - 4]) + S.ab * (f[L - 1] - f[L - 5]) + S.ac * (rl[5] - f[L - 6]);
      r[L - 2] = -e1 - rl[4];
      r[L - 1] = -e0 - rl[3];
      for (int i = 0; i < L; i++)
        v[i] = r[i] - (i >= 2 ? fc[i * 5 + 0] * v[i - 2] : 0.0) - (i >= 1 ? fc[i * 5 + 1] * v[i - 1] : 0.0);
      b[L] = b[L + 1] = 0.0;
      for (int i = L - 1; i >= 0; i--)
        b[i] = fc[i * 5 + 2] * v[i] - (i <= L - 2 ? fc[i * 5 + 3] * b[i + 1] : 0.0) -
               (i <= L - 3 ? fc[i * 5 + 4] * b[i + 2] : 0.0);
      for (int i = 0; i < L; i++) out[((size_t)gb * DENSE_MAX + i) * DENSE_MAX + j] = b[i];
    }
  }
  return lmax;
}

// Scaled-factor row tables of the FP64 fast path's line solves (solve_line_u,
// layout at FU_RT): forward factors rescaled to carry u = c2 v, the stencil
// weights k1..k3 times c2, the back-substitution factors with the entries past
// the line end set to zero, and c2 itself.
static void fu_tables(const ati_handle *h, const std::vector<double> &fac, double k1, double k2, double k3,
                      std::vector<double> &out) {
  out.assign((size_t)h->nfac * FU_RT, 0.0);
  for (int gb = 0; gb < h->nb; gb++) {
    const BlockDev &B = h->blk[gb];
    for (int nn = 1; nn <= 3; nn++) {
      const int L = nn == 1 ? B.lxi + 1 : (nn == 2 ? B.let + 1 : B.lze + 1);
      const double *fc = &fac[(size_t)B.fac_off[nn] * 5];
      double *o = &out[(size_t)B.fac_off[nn] * FU_RT];
      for (int i = 0; i < L; i++) {
        const double c2 = fc[i * 5 + 2];
        double *r = o + (size_t)i * FU_RT;
        r[0] = i >= 2 ? c2 * fc[i * 5 + 0] / fc[(i - 2) * 5 + 2] : 0.0;
        r[1] = i >= 1 ? c2 * fc[i * 5 + 1] / fc[(i - 1) * 5 + 2] : 0.0;
        r[2] = c2 * k1; r[3] = c2 * k2; r[4] = c2 * k3;
        r[5] = i <= L - 2 ? fc[i * 5 + 3] : 0.0;
        r[6] = i <= L - 3 ? fc[i * 5 + 4] : 0.0;
        r[7] = c2;
        r[8] = 2.0 * (r[2] + r[3] + r[4]);
      }
    }
  }
}

template <typename T>
static Coef<T> make_coef(const Scheme &S) {
  Coef<T> c;
  for (int r = 0; r < 3; r++)
    for (int q = 0; q < 6; q++) c.abc[r][q] = (T)S.abc[r][q];
  for (int a = 0; a < 2; a++)
    for (int b = 0; b < 2; b++) {
      for (int q = 0; q < 12; q++) { c.pbci[a][b][q] = (T)S.pbci[a][b][q]; c.pbco[a][b][q] = (T)S.pbco[a][b][q]; }
      c.pbcot[a][b] = (T)S.pbcot[a][b];
    }
  for (int q = 0; q < 3; q++) { c.fam[q] = (T)S.fam[q]; c.fbm[q] = (T)S.fbm[q]; c.fcm[q] = (T)S.fcm[q]; }
  c.fa = (T)S.fa; c.fb = (T)S.fb; c.fc = (T)S.fc;
  for (int q = 0; q < 4; q++) { c.fex[q] = (T)S.fex[q]; c.ffx[q] = (T)S.ffx[q]; }
  c.aa = (T)S.aa; c.ab = (T)S.ab; c.ac = (T)S.ac;
  return c;
}

static bool same_numerics(const ati_config_t &a, const ati_config_t &b) {
  return a.bkx == b.bkx && a.bky == b.bky && a.bkz == b.bkz && a.nkrk == b.nkrk && a.nviscous == b.nviscous &&
         a.les == b.les && a.precision == b.precision && a.fltk == b.fltk && a.fltkbc == b.fltkbc;
}

static int create_impl(const ati_config_t *cfgs, int ncase, ati_handle_t **out) {
  ati_handle *h = nullptr;
  if (!cfgs || !out || ncase < 1) return fail(h, ATI_EINVAL, "null argument or ncase < 1");
  *out = nullptr;
  for (int c = 0; c < ncase; c++) {
    const ati_config_t *cfg = &cfgs[c];
    if (cfg->bkx != 3 || cfg->bky != 2 || cfg->bkz != 1)
      return fail(h, ATI_EINVAL, "the aerofoil H-grid topology has bkx=3, bky=2, bkz=1 blocks");
    if (cfg->nkrk < 1 || cfg->nkrk > 8) return fail(h, ATI_EINVAL, "nkrk must be 1..8");
    if (cfg->precision != ATI_FP64 && cfg->precision != ATI_FP64_STRICT && cfg->precision != ATI_MIXED)
      return fail(h, ATI_EINVAL, "precision: ATI_FP64, ATI_FP64_STRICT or ATI_MIXED");
    if (!same_numerics(*cfg, cfgs[0]))
      return fail(h, ATI_EINVAL, "a batch shares its numerics: nkrk, nviscous, les, precision, fltk and fltkbc of "
                                 "every case must equal case 0's (case " + std::to_string(c) + " differs)");
  }
  if (6 * ncase > MAXB) return fail(h, ATI_EINVAL, "too many cases in one batch");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return fail(h, ATI_ECUDA, "no CUDA device: this library has no CPU fallback");
  h = new ati_handle();
  h->ncase = ncase;
  h->cfgs.assign(cfgs, cfgs + ncase);
  h->cfg = cfgs[0];
  h->mixed = h->cfg.precision == ATI_MIXED;
  h->nb = 6 * ncase;
  h->blk.resize(h->nb);
  h->grid_set.assign(h->nb, 0);
  h->shc.resize(ncase);
  for (int c = 0; c < ncase; c++) {
    build_scheme(cfgs[c], h->shc[c]);
    if (cfgs[c].dto < 0) h->any_cfl = true;
  }
  h->sh = h->shc[0];
  for (int c = 0; c < ncase; c++) {  // inflow-turbulence modes, concatenated over cases
    std::vector<float> m;
    build_modes(cfgs[c], m);
    TurbCase tc{};
    tc.off = (int)(h->hmodes.size() / 8);
    tc.n = (int)(m.size() / 8);
    for (int q = 0; q < 3; q++) tc.u[q] = h->shc[c].s.uoo[q + 1];
    h->htc.push_back(tc);
    h->hmodes.insert(h->hmodes.end(), m.begin(), m.end());
  }
  std::vector<double> facd, facf, spg;
  int rc = build_tables(h, facd, facf, spg);
  if (rc) {
    g_create_err = h->err;
    delete h;
    return rc;
  }
  const int64_t N = h->N, F = h->F;
  size_t bytes = 0;
  auto take = [&](size_t nbytes) {
    size_t o = bytes;
    bytes += (nbytes + 255) & ~(size_t)255;
    return o;
  };
  const size_t D8 = sizeof(double), F4 = sizeof(float);
  const size_t nforce = std::max<size_t>(h->tl_force.n, 1);
  // FP64 set: qa qo de(5) rr ss(3) xim etm zem(3) yaco p mu(1) tau(9) asz bsz(1) cnt(2) prim(4) dv(12) flx(15)
  // fw(3 x 5) fw1(1)
  const int np64 = 5 + 5 + 5 + 3 + 3 + 9 + 1 + 1 + 1 + 9 + 2 + 2 + 4 + 12 + 15 + 15 + 1;
  const size_t o_f = take((size_t)np64 * N * D8), o_drva = take(10 * F * D8), o_drvb = take(10 * F * D8),
               o_recv = take(30 * F * D8), o_cm = take(6 * F * D8), o_facd = take(facd.size() * D8),
               o_facf = take(facf.size() * D8), o_sbcc = take(std::max<int64_t>(h->nsbcc, 1) * D8),
               o_rpex = take(std::max<int64_t>(h->nwall, 1) * D8), o_area = take(std::max<int64_t>(h->nwall, 1) * D8),
               o_wnor = take(3 * std::max<int64_t>(h->nwall, 1) * D8), o_frc = take(2 * nforce * D8),
               o_spg = take(spg.size() * D8), o_blk = take(sizeof(BlockDev) * h->nb),
               o_sc = take(sizeof(Scheme) * ncase), o_cfd = take(sizeof(Coef<double>)),
               o_scal = take(sizeof(Scalars) * ncase), o_task = take(sizeof(FaceTask) * h->htasks.size()),
               o_cum = take(sizeof(int64_t) * (h->htasks.size() + 1)), o_bar = take(sizeof(unsigned) * 2),
               o_jn = take(sizeof(JunctionDev) * 2 * ncase), o_woff = take(nforce * sizeof(int64_t)),
               o_pt = take(sizeof(PTile) * h->max_pt), o_ptc0 = take(sizeof(PTile) * h->hptc[0].size()),
               o_ptc1 = take(sizeof(PTile) * h->hptc[1].size()), o_ptc2 = take(sizeof(PTile) * h->hptc[2].size()),
               o_lt1 = take(sizeof(LTile) * h->max_lt[1]),
               o_lt2 = take(sizeof(LTile) * h->max_lt[2]), o_lt3 = take(sizeof(LTile) * h->max_lt[3]),
               o_facud = take((size_t)h->nfac * FU_RT * D8), o_facuf = take((size_t)h->nfac * FU_RT * D8);
  // FP32 set (mixed): de(5) prim(4) mu p(1) dv(12) tau(9) flx(15) fw(3 x 5) xim etm zem(3) yaco asz bsz(1) gm(3)
  size_t o_ff = 0, o_fdrva = 0, o_fdrvb = 0, o_frecv = 0, o_fcm = 0, o_ffacd = 0, o_ffacf = 0, o_fsbcc = 0,
         o_frpex = 0, o_cff = 0, o_fdrvm = 0, o_lts[4] = {0, 0, 0, 0}, o_segd = 0, o_segf = 0, o_tmap = 0, o_dzm = 0;
  const int np32 = 5 + 4 + 1 + 1 + 12 + 9 + 15 + 15 + 9 + 1 + 1 + 1 + 3;
  if (h->mixed) {
    o_ff = take((size_t)np32 * N * F4);
    o_fdrva = take(10 * F * F4); o_fdrvb = take(10 * F * F4); o_frecv = take(30 * F * F4); o_fcm = take(6 * F * F4);
    o_fdrvm = take(10 * F * F4);
    o_ffacd = take(facd.size() * F4); o_ffacf = take(facf.size() * F4);
    o_fsbcc = take(std::max<int64_t>(h->nsbcc, 1) * F4); o_frpex = take(std::max<int64_t>(h->nwall, 1) * F4);
    o_cff = take(sizeof(Coef<float>));
    for (int nn = 1; nn <= 3; nn++) o_lts[nn] = take(sizeof(LTile) * std::max<size_t>(h->hlts[nn].size(), 1));
    // (SEG_PAD rows of padding before and after: the kernel reads a few rows ahead of its segment)
    o_segd = take((size_t)(h->nfac + 2 * SEG_PAD) * SEG_RT * F4);
    o_segf = take((size_t)(h->nfac + 2 * SEG_PAD) * SEG_RT * F4);
    o_tmap = take(sizeof(TmaMap) * 4 * (size_t)h->nb);
    o_dzm = take(sizeof(float) * DENSE_MAX * DENSE_MAX * (size_t)h->nb);
  }
  cudaError_t e = cudaMalloc(&h->arena, bytes);
  if (e != cudaSuccess) {
    g_create_err = std::string("cudaMalloc of ") + std::to_string(bytes) + " bytes: " + cudaGetErrorString(e);
    delete h;
    return ATI_ENOMEM;
  }
  h->arena_bytes = bytes;
  auto D = [&](size_t o) { return (double *)(h->arena + o); };
  auto Fp = [&](size_t o) { return (float *)(h->arena + o); };
  BlockDev *dblk = (BlockDev *)(h->arena + o_blk);
  Scheme *dsc = (Scheme *)(h->arena + o_sc);
  Scalars *dscal = (Scalars *)(h->arena + o_scal);
  const PTile *dpt = (const PTile *)(h->arena + o_pt);
  h->dptc[0] = (const PTile *)(h->arena + o_ptc0);
  h->dptc[1] = (const PTile *)(h->arena + o_ptc1);
  h->dptc[2] = (const PTile *)(h->arena + o_ptc2);
  const LTile *dlt[4] = {nullptr, (const LTile *)(h->arena + o_lt1), (const LTile *)(h->arena + o_lt2),
                         (const LTile *)(h->arena + o_lt3)};
  Eng<double> &d = h->ed;
  double *f = D(o_f);
  d.blk = dblk; d.sc = dsc; d.cf = (Coef<double> *)(h->arena + o_cfd); d.scal = dscal; d.N = N; d.F = F;
  d.ncase = ncase; d.pt = dpt; d.npt = (int)h->hpt.size();
  for (int nn = 0; nn < 4; nn++) d.sg_lines[nn] = h->sg_lines[nn];
  for (int nn = 0; nn < 4; nn++) d.maxlen[nn] = h->maxlen[nn];
  for (int nn = 1; nn <= 3; nn++) { d.lt[nn] = dlt[nn]; d.nlt[nn] = (int)h->hlt[nn].size(); }
  d.qa = f; f += 5 * N; d.qo = f; f += 5 * N; d.de = f; f += 5 * N;
  h->rr = f; f += 3 * N; h->ss = f; f += 3 * N;
  d.xim = f; f += 3 * N; d.etm = f; f += 3 * N; d.zem = f; f += 3 * N; d.yaco = f; d.yacod = f; f += N;
  d.p = f; f += N; d.mu = f; f += N; d.tau = f; f += 9 * N; d.asz = f; f += N; d.bsz = f; f += N;
  d.cnt = f; f += 2 * N; d.prim = f; f += 4 * N; d.dv = f; f += 12 * N; d.flx = f; f += 15 * N; d.fw = f; f += 15 * N;
  d.fw_dir = 5 * N;
  h->fw1 = f; f += N;
  d.drva = D(o_drva); d.drvb = D(o_drvb); d.recv = D(o_recv); d.cm = D(o_cm);
  d.facd = D(o_facd); d.facf = D(o_facf); d.sbcc = D(o_sbcc); d.rpex = D(o_rpex);
  d.facud = D(o_facud); d.facuf = D(o_facuf);
  h->area = D(o_area); h->wnor = D(o_wnor); h->dforce = D(o_frc); h->dspg = D(o_spg);
  h->dtasks = (FaceTask *)(h->arena + o_task);
  h->dcum = (int64_t *)(h->arena + o_cum);
  h->dbar = (unsigned *)(h->arena + o_bar);
  h->djn = (JunctionDev *)(h->arena + o_jn);
  h->dwoff = (int64_t *)(h->arena + o_woff);
  if (h->mixed) {
    Eng<float> &m = h->ef;
    float *g = Fp(o_ff);
    m.blk = dblk; m.sc = dsc; m.cf = (Coef<float> *)(h->arena + o_cff); m.scal = dscal; m.N = N; m.F = F;
    m.ncase = ncase; m.pt = dpt; m.npt = d.npt;
    for (int nn = 0; nn < 4; nn++) m.sg_lines[nn] = d.sg_lines[nn];
    for (int nn = 0; nn < 4; nn++) m.maxlen[nn] = h->maxlen[nn];
    for (int nn = 1; nn <= 3; nn++) { m.lt[nn] = dlt[nn]; m.nlt[nn] = d.nlt[nn]; }
    m.qa = d.qa; m.qo = d.qo; m.yacod = d.yacod; m.cnt = d.cnt;
    m.de = g; g += 5 * N; m.prim = g; g += 4 * N; m.mu = g; g += N; m.p = g; g += N; m.dv = g; g += 12 * N;
    m.tau = g; g += 9 * N; m.flx = g; g += 15 * N; m.fw = g; g += 15 * N;
    m.fw_dir = 5 * N;
    m.xim = g; g += 3 * N; m.etm = g; g += 3 * N; m.zem = g; g += 3 * N; m.yaco = g; g += N;
    m.asz = g; g += N; m.bsz = g; g += N; m.gm = g; g += 3 * N;
    m.drvm = Fp(o_fdrvm);
    m.drva = Fp(o_fdrva); m.drvb = Fp(o_fdrvb); m.recv = Fp(o_frecv); m.cm = Fp(o_fcm);
    m.facd = Fp(o_ffacd); m.facf = Fp(o_ffacf); m.sbcc = Fp(o_fsbcc); m.rpex = Fp(o_frpex);
    for (int nn = 1; nn <= 3; nn++) {
      m.lts[nn] = (const LTile *)(h->arena + o_lts[nn]);
      m.nsegc[nn] = h->nsegc[nn];
      for (int c = 0; c < SEG_NCLASS; c++) m.segc[nn][c] = h->segc[nn][c];
    }
    m.segd = Fp(o_segd) + SEG_PAD * SEG_RT; m.segf = Fp(o_segf) + SEG_PAD * SEG_RT;
    m.dzm = Fp(o_dzm);
    m.dense = false;
    m.tmaps = (const TmaMap *)(h->arena + o_tmap);
    m.nblk = h->nb;
    for (int nn = 0; nn < 4; nn++) m.tma[nn] = h->tma[nn];
    m.eta_rowtiles = h->tma[2];
    m.pairs = true;
  }
  // junctions (src/SingleTurbulence3D.f90:386-398), bkx = 3, bky = 2, per case
  std::vector<JunctionDev> jn;
  for (int cs = 0; cs < ncase; cs++) {
    const ati_config_t *cfg = &h->cfgs[cs];
    const int b0 = h->case_b0[cs];
    for (int nn = 0; nn <= (cfg->bkx - 1) * (cfg->bky - 1) - 1; nn++) {
      const int njct = nn + nn / (cfg->bkx - 1);
      const int mm[4] = {njct, njct + 1, njct + cfg->bkx, njct + cfg->bkx + 1};
      const int cip[4] = {1, 0, 1, 0}, cjp[4] = {1, 1, 0, 0};
      JunctionDev J{};
      for (int q = 0; q < 4; q++) {
        const BlockDev &B = h->blk[b0 + mm[q]];
        const int i = cip[q] * B.lxi, j = cjp[q] * B.let;
        J.base[q] = B.off + (int64_t)j * (B.lxi + 1) + i;
        J.kstr[q] = (int64_t)(B.lxi + 1) * (B.let + 1);
      }
      J.nk = h->blk[b0 + mm[0]].lze + 1;
      J.pa = (1 - nn) == 1 ? 2 : 1;
      J.pb = (1 - nn) == 1 ? 4 : 3;
      jn.push_back(J);
      h->jnk = std::max(h->jnk, J.nk);
    }
  }
  h->njct = (int)jn.size();
  std::vector<int64_t> woff;
  for (int q = 0; q < h->tl_force.n; q++) woff.push_back(h->htasks[h->tl_force.off + q].wall_off);
  const Coef<double> cfd = make_coef<double>(h->sh.s);
  const Coef<float> cff = make_coef<float>(h->sh.s);
  std::vector<Scheme> schemes;
  for (int c = 0; c < ncase; c++) schemes.push_back(h->shc[c].s);
  std::vector<float> facd32(facd.begin(), facd.end()), facf32(facf.begin(), facf.end()), segd32, segf32, dzm32;
  if (h->mixed) {
    seg_tables(h, facd, segd32);
    seg_tables(h, facf, segf32);
    std::vector<double> dzm;
    h->ef.dzl = dense_zeta(h, facd, dzm);
    dzm32.assign(dzm.begin(), dzm.end());
  }
  e = cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking);
  for (int q = 0; q < 2 && e == cudaSuccess; q++) e = cudaStreamCreateWithFlags(&h->side[q], cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming);
  for (int q = 0; q < 2 && e == cudaSuccess; q++) e = cudaEventCreateWithFlags(&h->ev_join[q], cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaMemsetAsync(h->arena, 0, bytes, h->st);
  auto up = [&](const void *dst, const void *src, size_t n) {
    if (e == cudaSuccess && n) e = cudaMemcpyAsync(const_cast<void *>(dst), src, n, cudaMemcpyHostToDevice, h->st);
  };
  up(d.facd, facd.data(), facd.size() * D8);
  up(d.facf, facf.data(), facf.size() * D8);
  std::vector<double> facud, facuf;
  fu_tables(h, facd, h->sh.s.aa, h->sh.s.ab, h->sh.s.ac, facud);
  fu_tables(h, facf, h->sh.s.fa, h->sh.s.fb, h->sh.s.fc, facuf);
  up(d.facud, facud.data(), facud.size() * D8);
  up(d.facuf, facuf.data(), facuf.size() * D8);
  up(h->dspg, spg.data(), spg.size() * D8);
  up(dblk, h->blk.data(), sizeof(BlockDev) * h->nb);
  up(dsc, schemes.data(), sizeof(Scheme) * ncase);
  up(d.cf, &cfd, sizeof(cfd));
  up(h->dtasks, h->htasks.data(), sizeof(FaceTask) * h->htasks.size());
  std::vector<int64_t> cum(h->htasks.size() + 1, 0);
  for (size_t q = 0; q < h->htasks.size(); q++) cum[q + 1] = cum[q] + h->htasks[q].nline;
  up(h->dcum, cum.data(), sizeof(int64_t) * cum.size());
  up(h->djn, jn.data(), sizeof(JunctionDev) * jn.size());
  up(h->dwoff, woff.data(), sizeof(int64_t) * woff.size());
  up(dpt, h->hpt.data(), sizeof(PTile) * h->hpt.size());
  for (int c = 0; c < 3; c++) up(h->dptc[c], h->hptc[c].data(), sizeof(PTile) * h->hptc[c].size());
  for (int nn = 1; nn <= 3; nn++) up(dlt[nn], h->hlt[nn].data(), sizeof(LTile) * h->hlt[nn].size());
  if (h->mixed) {
    up(h->ef.cf, &cff, sizeof(cff));
    up(h->ef.facd, facd32.data(), facd32.size() * F4);
    up(h->ef.facf, facf32.data(), facf32.size() * F4);
    up(h->ef.segd, segd32.data(), segd32.size() * F4);
    up(h->ef.segf, segf32.data(), segf32.size() * F4);
    up(h->ef.dzm, dzm32.data(), dzm32.size() * F4);
    if (h->tma[2] || h->tma[3]) {
      if (encode_tmaps(h, h->htmaps) != ATI_OK) {
        if (e == cudaSuccess) e = cudaErrorInvalidValue;
        g_tma_err = h->err;
      } else {
        up(h->ef.tmaps, h->htmaps.data(), sizeof(TmaMap) * h->htmaps.size());
      }
    }
    for (int nn = 1; nn <= 3; nn++) up(h->ef.lts[nn], h->hlts[nn].data(), sizeof(LTile) * h->hlts[nn].size());
    if (e == cudaSuccess) e = fast::seg_init();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
  if (e != cudaSuccess) {
    g_create_err = g_tma_err.empty() ? std::string("set-up copy: ") + cudaGetErrorString(e) : g_tma_err;
    g_tma_err.clear();
    cudaFree(h->arena);
    delete h;
    return ATI_ECUDA;
  }
  *out = h;
  return ATI_OK;
}

extern "C" int ati_create(const ati_config_t *cfg, ati_handle_t **out) { return create_impl(cfg, 1, out); }

// The dense zeta operator of one block, built on the host as ati_create builds it for ATI_OPT_DENSE_ZETA (scheme,
// topology and LU factors of the case, then dense_zeta), in FP64 and without a device.
extern "C" int ati_dense_zeta_operator(const ati_config_t *cfg, int blk, double *M, int32_t *L) {
  if (!cfg || !M || !L) return fail(nullptr, ATI_EINVAL, "ati_dense_zeta_operator: null argument");
  if (cfg->bkx != 3 || cfg->bky != 2 || cfg->bkz != 1)
    return fail(nullptr, ATI_EINVAL, "the aerofoil H-grid topology has bkx=3, bky=2, bkz=1 blocks");
  if (blk < 0 || blk >= 6) return fail(nullptr, ATI_EINVAL, "ati_dense_zeta_operator: block index out of range");
  std::unique_ptr<ati_handle> h(new ati_handle());
  h->ncase = 1;
  h->cfgs.assign(cfg, cfg + 1);
  h->cfg = *cfg;
  h->mixed = cfg->precision == ATI_MIXED;
  h->nb = 6;
  h->blk.resize(h->nb);
  h->grid_set.assign(h->nb, 0);
  h->shc.resize(1);
  build_scheme(*cfg, h->shc[0]);
  h->sh = h->shc[0];
  std::vector<double> facd, facf, spg, ops;
  if (int rc = build_tables(h.get(), facd, facf, spg)) {
    g_create_err = h->err;
    return rc;
  }
  if (!dense_zeta(h.get(), facd, ops))
    return fail(nullptr, ATI_EINVAL, "the zeta lines do not qualify: every zeta face periodic onto its own block "
                                     "and lines of LMD + 2 to DENSE_MAX points");
  const int n = h->blk[blk].lze + 1;
  *L = n;
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) M[(size_t)i * n + j] = ops[((size_t)blk * DENSE_MAX + i) * DENSE_MAX + j];
  return ATI_OK;
}

extern "C" int ati_create_batch(const ati_config_t *cfgs, int ncase, ati_handle_t **out) {
  return create_impl(cfgs, ncase, out);
}

static void probe_free(ati_handle *h) {
  if (h->probe_p) cudaFree(h->probe_p);
  if (h->probe_t) cudaFree(h->probe_t);
  h->probe_p = h->probe_t = nullptr;
  h->probe_cap = 0;
}

static void drop_graphs(ati_handle *h) {
  for (auto &g : h->gexec)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
}

extern "C" int ati_destroy(ati_handle_t *h) {
  if (!h) return ATI_OK;
  if (h->st) cudaStreamSynchronize(h->st);
  prof_drain(h);
  for (auto &e : h->ev_free) {
    cudaEventDestroy(e.a);
    cudaEventDestroy(e.b);
  }
  drop_graphs(h);
  probe_free(h);
  for (void *p : {(void *)h->dmodes, (void *)h->ddelta, (void *)h->dtc, (void *)h->dgust, (void *)h->dgust64,
                  (void *)h->ddelta64})
    if (p) cudaFree(p);
  if (h->arena) cudaFree(h->arena);
  if (h->st) cudaStreamDestroy(h->st);
  for (int q = 0; q < 2; q++) {
    if (h->side[q]) cudaStreamDestroy(h->side[q]);
    if (h->ev_join[q]) cudaEventDestroy(h->ev_join[q]);
  }
  if (h->ev_fork) cudaEventDestroy(h->ev_fork);
  delete h;
  return ATI_OK;
}

// Waits for the handle's stream: unbounded by default, or polling until the handle's wait limit, after which it
// returns ATI_ETIMEDOUT with the work still in flight (a later wait picks it up; nothing is cancelled).
static int wait_stream(ati_handle *h) {
  if (h->wait_timeout <= 0.0) {
    CK(cudaStreamSynchronize(h->st));
    return ATI_OK;
  }
  const auto t0 = std::chrono::steady_clock::now();
  for (;;) {
    const cudaError_t e = cudaStreamQuery(h->st);
    if (e == cudaSuccess) return ATI_OK;
    if (e != cudaErrorNotReady) return fail(h, ATI_ECUDA, std::string("cudaStreamQuery: ") + cudaGetErrorString(e));
    const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (dt >= h->wait_timeout)
      return fail(h, ATI_ETIMEDOUT, "the handle's work did not finish within the wait limit of " +
                                        std::to_string(h->wait_timeout) + " s (still in flight)");
    std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
}

extern "C" int ati_synchronize(ati_handle_t *h) {
  if (!h) return ATI_EINVAL;
  return wait_stream(h);
}

extern "C" int ati_set_wait_timeout(ati_handle_t *h, double seconds) {
  if (!h || !(seconds >= 0.0)) return fail(h, ATI_EINVAL, "ati_set_wait_timeout: bad argument");
  h->wait_timeout = seconds;
  return ATI_OK;
}

extern "C" int ati_block_dims(ati_handle_t *h, int blk, int32_t dims[3], int64_t *npts) {
  if (!h || blk < 0 || blk >= h->nb || !dims) return fail(h, ATI_EINVAL, "ati_block_dims: bad argument");
  dims[0] = h->blk[blk].lxi; dims[1] = h->blk[blk].let; dims[2] = h->blk[blk].lze;
  if (npts) *npts = h->blk[blk].npts;
  return ATI_OK;
}

// ---- field copies ----------------------------------------------------------
// In a mixed case de, p and the stresses of the last stage live in FP32: they
// are widened on the device before the copy; set_field writes the FP64 arrays.
static double *field_base(ati_handle *h, int field, int &ncomp, const float **f32) {
  Eng<double> &c = h->ed;
  *f32 = nullptr;
  switch (field) {
    case ATI_F_QA: ncomp = 5; return c.qa;
    case ATI_F_QO: ncomp = 5; return c.qo;
    case ATI_F_DE: ncomp = 5; if (h->mixed) *f32 = h->ef.de; return c.de;
    case ATI_F_RR: ncomp = 3; return h->rr;
    case ATI_F_SS: ncomp = 3; return h->ss;
    case ATI_F_XIM: ncomp = 3; return const_cast<double *>(c.xim);
    case ATI_F_ETM: ncomp = 3; return const_cast<double *>(c.etm);
    case ATI_F_ZEM: ncomp = 3; return const_cast<double *>(c.zem);
    case ATI_F_P: ncomp = 1; if (h->mixed) *f32 = h->ef.p; return c.p;
    case ATI_F_YACO: ncomp = 1; return const_cast<double *>(c.yaco);
    case ATI_F_STRESS: ncomp = 9; if (h->mixed) *f32 = h->ef.tau; return c.tau;
    case ATI_F_SPONGE: ncomp = 2; return const_cast<double *>(c.asz);  // asz and bsz are adjacent planes
    case ATI_F_CP: ncomp = 1; return h->fw1;  // derived into the granular scratch plane by copy_field
    default: ncomp = 0; return nullptr;
  }
}

// The mixed path's step takes the viscous stresses inside its flux kernel and keeps no stress planes: the
// forces and the stress output rebuild the last stage's planes (k_visc) from the derivative planes, viscosity
// and primitives that stage left, which nothing changes until the next stage.
// The step's viscous fluxes take the stresses at the point (no stress planes in a stage): the mixed path, and the
// FP64 fast path without the LES term (whose stresses read rho of the stage's state)
static bool stress_at_point(const ati_handle *h) {
  return h->cfg.nviscous == 1 && (h->mixed || (h->cfg.precision == ATI_FP64 && h->cfg.les != 1 && h->fp64_at_point));
}
// ... the stress planes are then made on demand, from the last stage's derivative planes
static void stress_planes(ati_handle *h) {
  if (!stress_at_point(h)) return;
  if (h->mixed) fast::pointwise_f(h->ef, h->st, PW_VISC);
  else fast::pointwise_d(h->ed, h->st, PW_VISC);
}

static int copy_field(ati_handle *h, int blk, int field, double *host, bool to_dev) {
  if (!h || blk < 0 || blk >= h->nb || !host) return fail(h, ATI_EINVAL, "field copy: bad argument");
  int nc = 0;
  const float *f32 = nullptr;
  double *base = field_base(h, field, nc, &f32);
  if (!base) return fail(h, ATI_EINVAL, "unknown field id");
  const BlockDev &B = h->blk[blk];
  const size_t w = (size_t)B.npts * sizeof(double), dp = (size_t)h->N * sizeof(double);
  if (field == ATI_F_CP) {
    if (to_dev) return fail(h, ATI_EINVAL, "ATI_F_CP is derived: ati_get_field only");
    if (!h->inited) return fail(h, ATI_ESTATE, "ATI_F_CP needs ati_init");
    k_cp<<<dim3(64, h->nb), 256, 0, h->st>>>(h->ed, base);
    CKL();
  }
  if (to_dev) {
    CK(cudaMemcpy2DAsync(base + B.off, dp, host, w, w, nc, cudaMemcpyHostToDevice, h->st));
  } else {
    if (field == ATI_F_STRESS) stress_planes(h);
    if (f32) {  // widen the FP32 stage field into the FP64 array first (the mixed pressure plane holds p - p_inf)
      const double add = field == ATI_F_P ? h->sh.s.poo : 0.0;
      k_to_double<<<256, 256, 0, h->st>>>(f32, base, (int64_t)nc * h->N, add);
      CKL();
    }
    CK(cudaMemcpy2DAsync(host, w, base + B.off, dp, w, nc, cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
  }
  return ATI_OK;
}

extern "C" int ati_set_field(ati_handle_t *h, int blk, int field, const double *v) {
  return copy_field(h, blk, field, const_cast<double *>(v), true);
}
extern "C" int ati_get_field(ati_handle_t *h, int blk, int field, double *v) { return copy_field(h, blk, field, v, false); }
extern "C" int ati_set_state(ati_handle_t *h, int blk, const double *q) {
  return copy_field(h, blk, ATI_F_QA, const_cast<double *>(q), true);
}
extern "C" int ati_get_state(ati_handle_t *h, int blk, double *q) { return copy_field(h, blk, ATI_F_QA, q, false); }

// the state planes qa are one contiguous [5][N] array: the whole state is one copy
extern "C" int ati_set_state_all(ati_handle_t *h, const double *q) {
  if (!h || !q) return fail(h, ATI_EINVAL, "ati_set_state_all: bad argument");
  CK(cudaMemcpyAsync(h->ed.qa, q, sizeof(double) * 5 * h->N, cudaMemcpyHostToDevice, h->st));
  return ATI_OK;
}
extern "C" int ati_get_state_all(ati_handle_t *h, double *q) {
  if (!h || !q) return fail(h, ATI_EINVAL, "ati_get_state_all: bad argument");
  CK(cudaMemcpyAsync(q, h->ed.qa, sizeof(double) * 5 * h->N, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  return ATI_OK;
}
extern "C" int ati_points_total(ati_handle_t *h, int64_t *n) {
  if (!h || !n) return fail(h, ATI_EINVAL, "ati_points_total: bad argument");
  *n = h->N;
  return ATI_OK;
}

extern "C" int ati_get_face(ati_handle_t *h, int blk, int which, int nn, double *v) {
  if (!h || blk < 0 || blk >= h->nb || nn < 1 || nn > 3 || !v) return fail(h, ATI_EINVAL, "ati_get_face: bad argument");
  const BlockDev &B = h->blk[blk];
  const double *src;
  int nc;
  switch (which) {
    case ATI_FACE_DRVA: src = h->ed.drva; nc = 10; break;
    case ATI_FACE_DRVB: src = h->ed.drvb; nc = 10; break;
    case ATI_FACE_RECV: src = h->ed.recv; nc = 6; break;
    case ATI_FACE_CM: src = h->ed.cm; nc = 6; break;
    default: return fail(h, ATI_EINVAL, "unknown face buffer");
  }
  CK(cudaMemcpyAsync(v, src + B.face_off[nn] * nc, sizeof(double) * nc * B.nbsize[nn], cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  return ATI_OK;
}

static int case_time(ati_handle *h, int cs, ati_time_t *t) {
  if (!h || !t || cs < 0 || cs >= h->ncase) return fail(h, ATI_EINVAL, "time: bad argument");
  Scalars s;
  CK(cudaMemcpyAsync(&s, h->ed.scal + cs, sizeof(s), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  t->n = s.n; t->ndt = s.ndt; t->dt = s.dt; t->dts = s.dts; t->dte = s.dte; t->timo = s.timo;
  return ATI_OK;
}

static int case_set_time(ati_handle *h, int cs, const ati_time_t *t) {
  if (!h || !t || cs < 0 || cs >= h->ncase) return fail(h, ATI_EINVAL, "set time: bad argument");
  if (h->ncase > 1 && t->n != h->n_host)
    return fail(h, ATI_EINVAL, "the cases of a batch step together: n must equal the batch's step count");
  Scalars s;
  CK(cudaMemcpyAsync(&s, h->ed.scal + cs, sizeof(s), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  s.n = t->n; s.ndt = t->ndt; s.dt = t->dt; s.dts = t->dts; s.dte = t->dte; s.timo = t->timo;
  CK(cudaMemcpyAsync(h->ed.scal + cs, &s, sizeof(s), cudaMemcpyHostToDevice, h->st));
  CK(cudaStreamSynchronize(h->st));
  h->n_host = t->n;
  return ATI_OK;
}

extern "C" int ati_get_time(ati_handle_t *h, ati_time_t *t) { return case_time(h, 0, t); }

extern "C" int ati_set_time(ati_handle_t *h, const ati_time_t *t) {
  if (!h || !t) return fail(h, ATI_EINVAL, "ati_set_time: bad argument");
  const int64_t n0 = h->n_host;
  h->n_host = t->n;  // every case at once: the batch keeps one step count
  for (int c = 0; c < h->ncase; c++) {
    int rc = case_set_time(h, c, t);
    if (rc) {
      h->n_host = n0;
      return rc;
    }
  }
  return ATI_OK;
}

extern "C" int ati_turbulence_modes(ati_handle_t *h, int cs, float *modes, int32_t *nmodes) {
  if (!h || !nmodes || cs < 0 || cs >= h->ncase) return fail(h, ATI_EINVAL, "ati_turbulence_modes: bad argument");
  *nmodes = h->htc[cs].n;
  if (modes) std::memcpy(modes, h->hmodes.data() + 8 * (size_t)h->htc[cs].off, sizeof(float) * 8 * h->htc[cs].n);
  return ATI_OK;
}

extern "C" int ati_turbulence_sample(ati_handle_t *h, int cs, double t, int64_t n, const double *xyz, double *v) {
  if (!h || cs < 0 || cs >= h->ncase || n < 0 || (n > 0 && (!xyz || !v)))
    return fail(h, ATI_EINVAL, "ati_turbulence_sample: bad argument");
  if (!h->inited) return fail(h, ATI_ESTATE, "ati_init not called");
  if (!h->dtc || h->htc[cs].n == 0) return fail(h, ATI_EINVAL, "ati_turbulence_sample: the case has no inflow turbulence");
  if (n == 0) return ATI_OK;
  double *d = nullptr;
  if (cudaMalloc(&d, sizeof(double) * 6 * n) != cudaSuccess) {
    cudaGetLastError();
    return fail(h, ATI_ENOMEM, "ati_turbulence_sample: device allocation failed");
  }
  cudaError_t e = cudaMemcpyAsync(d, xyz, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, h->st);
  if (e == cudaSuccess) {
    turb_sample(h->st, h->dtc, cs, h->dmodes, t, n, d, d + 3 * n);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(v, d + 3 * n, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, h->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
  cudaFree(d);
  if (e != cudaSuccess) return fail(h, ATI_ECUDA, std::string("ati_turbulence_sample: ") + cudaGetErrorString(e));
  return ATI_OK;
}

extern "C" int ati_jacobian_sign(ati_handle_t *h, int32_t *flags) {
  if (!h || !flags) return fail(h, ATI_EINVAL, "ati_jacobian_sign: bad argument");
  if (!h->inited) return fail(h, ATI_ESTATE, "ati_init not called");
  int *d = reinterpret_cast<int *>(h->fw1);  // the granular scratch plane is free outside granular calls
  CK(cudaMemsetAsync(d, 0, sizeof(int) * h->nb, h->st));
  k_jac_sign<<<dim3(64, h->nb), 256, 0, h->st>>>(h->ed, d);
  CKL();
  std::vector<int> f(h->nb);
  CK(cudaMemcpyAsync(f.data(), d, sizeof(int) * h->nb, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  for (int b = 0; b < h->nb; b++) flags[b] = f[b];
  return ATI_OK;
}

extern "C" int ati_tiles(ati_handle_t *h, int32_t out[4]) {
  if (!h || !out) return fail(h, ATI_EINVAL, "ati_tiles: bad argument");
  out[0] = XC_NL;
  out[1] = h->sg_lines[2];
  out[2] = h->sg_lines[3];
  out[3] = h->pt_points;
  return ATI_OK;
}

extern "C" int ati_set_tiles(ati_handle_t *h, const int32_t in[4]) {
  if (!h || !in) return fail(h, ATI_EINVAL, "ati_set_tiles: bad argument");
  if (!h->inited) return fail(h, ATI_ESTATE, "ati_set_tiles: handle not initialised");
  const int sg2 = in[1] ? in[1] : h->sg_lines[2], sg3 = in[2] ? in[2] : h->sg_lines[3];
  const int pt = in[3] ? in[3] : h->pt_points;
  auto sg_ok = [](int v) { return v >= SG_MIN && v <= SG_MAX && v % 32 == 0; };
  if ((in[0] && in[0] != XC_NL) || !sg_ok(sg2) || !sg_ok(sg3) || pt < PT_MIN || pt > PT_MAX || pt % PT_MIN)
    return fail(h, ATI_EINVAL, "ati_set_tiles: xi lines per CTA are fixed; eta/zeta lines per CTA must be multiples "
                               "of 32 in [32, 256] and points per tile multiples of 256 in [256, 4096]");
  CK(cudaStreamSynchronize(h->st));  // steps in flight read the queues
  make_tiles(h, sg2, sg3, pt);
  if (int rc = upload_tiles(h)) return rc;
  std::fill(h->pw_pt, h->pw_pt + PW_KINDS, 0);  // every pointwise kernel on the pinned tiles
  apply_pw_tiles(h);
  drop_graphs(h);  // the step graphs hold the old grid shapes
  return ATI_OK;
}

extern "C" int ati_set_tuning(ati_handle_t *h, int enable) {
  if (!h) return fail(h, ATI_EINVAL, "null handle");
  h->tune = enable != 0;
  return ATI_OK;
}

static_assert(ATI_TILE_PLAN == 4 + PW_KINDS, "a tile plan: the four shapes of ati_tiles, then one entry per pointwise kind");
extern "C" int ati_get_tile_plan(ati_handle_t *h, int32_t plan[ATI_TILE_PLAN]) {
  if (!h || !plan) return fail(h, ATI_EINVAL, "ati_get_tile_plan: bad argument");
  if (int rc = ati_tiles(h, plan)) return rc;
  for (int k = 0; k < PW_KINDS; k++) plan[4 + k] = h->pw_pt[k];
  return ATI_OK;
}

extern "C" int ati_set_tile_plan(ati_handle_t *h, const int32_t plan[ATI_TILE_PLAN]) {
  if (!h || !plan) return fail(h, ATI_EINVAL, "ati_set_tile_plan: bad argument");
  if (!h->inited) return fail(h, ATI_ESTATE, "ati_set_tile_plan: handle not initialised");
  for (int k = 0; k < PW_KINDS; k++) {
    const int v = plan[4 + k];
    if (v != 0 && v != PT_CAND[0] && v != PT_CAND[1] && v != PT_CAND[2])
      return fail(h, ATI_EINVAL, "ati_set_tile_plan: a pointwise kernel's tile must be 0 or one of the timed sizes");
  }
  if (int rc = ati_set_tiles(h, plan)) return rc;  // (validates and applies the shapes; pins the shared queue)
  for (int k = 0; k < PW_KINDS; k++) h->pw_pt[k] = plan[4 + k];
  apply_pw_tiles(h);
  h->pt_points = plan[3];
  return ATI_OK;
}

extern "C" int ati_set_options(ati_handle_t *h, int flags, int32_t *active) {
  if (!h) return fail(h, ATI_EINVAL, "null handle");
  if (flags & ~(ATI_OPT_TMA | ATI_OPT_FUSED_FACES | ATI_OPT_PAIRED_LINES | ATI_OPT_STRESS_AT_POINT | ATI_OPT_DENSE_ZETA))
    return fail(h, ATI_EINVAL, "ati_set_options: unknown flag");
  CK(cudaStreamSynchronize(h->st));
  drop_graphs(h);
  for (int nn = 2; nn <= 3; nn++) h->ef.tma[nn] = (flags & ATI_OPT_TMA) != 0 && h->tma[nn];
  h->fused = (flags & ATI_OPT_FUSED_FACES) != 0;
  h->ef.pairs = (flags & ATI_OPT_PAIRED_LINES) != 0;
  h->fp64_at_point = (flags & ATI_OPT_STRESS_AT_POINT) != 0;
  h->ef.dense = (flags & ATI_OPT_DENSE_ZETA) != 0 && h->ef.dzl > 0;
  if (active)
    *active = (h->ef.tma[2] || h->ef.tma[3] ? ATI_OPT_TMA : 0) | (h->fused ? ATI_OPT_FUSED_FACES : 0) |
              (h->ef.tma[2] ? ATI_OPT_TMA_ETA : 0) | (h->ef.tma[3] ? ATI_OPT_TMA_ZETA : 0) |
              (h->ef.pairs ? ATI_OPT_PAIRED_LINES : 0) | (h->fp64_at_point ? ATI_OPT_STRESS_AT_POINT : 0) |
              (h->ef.dense ? ATI_OPT_DENSE_ZETA : 0);
  return ATI_OK;
}

extern "C" int ati_set_spin_limit(ati_handle_t *h, int64_t polls) {
  if (!h || polls < 0 || polls > 0xffffffffLL) return fail(h, ATI_EINVAL, "ati_set_spin_limit: bad argument");
  CK(cudaStreamSynchronize(h->st));
  drop_graphs(h);  // (the limit is a launch argument captured in the step graphs)
  h->spin_limit = polls == 0 ? (1u << 24) : (unsigned)polls;
  return ATI_OK;
}

extern "C" int ati_case_count(ati_handle_t *h, int *ncase) {
  if (!h || !ncase) return fail(h, ATI_EINVAL, "ati_case_count: bad argument");
  *ncase = h->ncase;
  return ATI_OK;
}

extern "C" int ati_case_blocks(ati_handle_t *h, int cs, int *first_block, int *nblocks) {
  if (!h || cs < 0 || cs >= h->ncase || !first_block || !nblocks) return fail(h, ATI_EINVAL, "ati_case_blocks: bad argument");
  *first_block = h->case_b0[cs];
  *nblocks = h->nb / h->ncase;
  return ATI_OK;
}

extern "C" int ati_case_time(ati_handle_t *h, int cs, ati_time_t *t) { return case_time(h, cs, t); }
extern "C" int ati_case_set_time(ati_handle_t *h, int cs, const ati_time_t *t) { return case_set_time(h, cs, t); }

extern "C" int ati_set_grid(ati_handle_t *h, int blk, const double *xyz) {
  int rc = copy_field(h, blk, ATI_F_SS, const_cast<double *>(xyz), true);
  if (rc == ATI_OK) h->grid_set[blk] = 1;
  return rc;
}

// ---- granular calls (strict build: the reference's rounding) ---------------------
static int granular_sweep(ati_handle *h, int nn, bool filt, const double *in, double *out, int m) {
  Eng<double> e = h->ed;
  e.fw = h->fw1;
  e.fw_dir = 0;
  SweepIO<double, double> io{in, 0, out, 0, nullptr, 1, m, !filt};
  PROF(h, (filt ? ATI_K_FILTER_XI : ATI_K_DERIV_XI) + nn - 1,
       strict::sweep_ddd(e, h->st, nn, filt, io));
  CKL();
  return ATI_OK;
}

extern "C" int ati_mpigo(ati_handle_t *h, int nt, int nrt, int n45) {
  if (!h || nt < 0 || nt > 1 || nrt < 0 || nrt > 1 || n45 < 0 || n45 > 1) return fail(h, ATI_EINVAL, "ati_mpigo: bad selector");
  const int64_t N = h->N;
  const double *r = h->rr;
  // nz = (1-nrt)*(nn-1)+1 (src/Subroutines3D.f90:23)
  const double *s2 = nrt == 1 ? r : r + N, *s3 = nrt == 1 ? r : r + 2 * N;
  PROF(h, ATI_K_MPIGO,
       strict::mpigo_ddd(h->ed, h->st, tp(h, h->tl_mpigo), h->tl_mpigo.n, h->tl_mpigo.maxline, nt, n45, r, s2, s3, 0, 1));
  CKL();
  return ATI_OK;
}

extern "C" int ati_deriv(ati_handle_t *h, int nn, int nz, int m) {
  if (!h || nn < 1 || nn > 3 || nz < 1 || nz > 3 || m < 1 || m > 5) return fail(h, ATI_EINVAL, "ati_deriv: bad selector");
  const int64_t N = h->N;
  return granular_sweep(h, nn, false, h->rr + (nz - 1) * N, h->rr + (nn - 1) * N, m);
}

extern "C" int ati_filte(ati_handle_t *h, int nn, int nz) {
  if (!h || nn < 1 || nn > 3 || nz < 1 || nz > 3) return fail(h, ATI_EINVAL, "ati_filte: bad selector");
  const int64_t N = h->N;
  return granular_sweep(h, nn, true, h->rr + (nz - 1) * N, h->rr + (nz - 1) * N, 0);
}

// ---- set-up: metrics, normals, GCBC weights, sponge, wall, IC ---------------
static int to_float(ati_handle *h, const double *src, const float *dst, int64_t n) {
  if (n <= 0) return ATI_OK;
  k_to_float<<<512, 256, 0, h->st>>>(src, const_cast<float *>(dst), n);
  CKL();
  return ATI_OK;
}

// gust points of the inflow-turbulence cases: sponge points of the inflow zone
// (x < -0.7 domlen + szth1, spongeup src/SingleTurbulence3D.f90:252-258), with
// the streamwise ramp atz = sin^2(min(pi (x + domlen) / szth1, pi / 2)); each
// case's list is padded to whole CTAs of the evaluation kernel
static int setup_gust(ati_handle *h) {
  for (void **p : {(void **)&h->dmodes, (void **)&h->ddelta, (void **)&h->dtc, (void **)&h->dgust,
                   (void **)&h->dgust64, (void **)&h->ddelta64}) {  // (a second ati_init)
    if (*p) cudaFree(*p);
    *p = nullptr;
  }
  h->ngust = 0;
  if (h->hmodes.empty()) return ATI_OK;
  const int64_t N = h->N;
  const bool fp64 = h->cfg.precision == ATI_FP64_STRICT;
  std::vector<double> xyz((size_t)3 * N), asz(N);
  CK(cudaMemcpyAsync(xyz.data(), h->ss, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost, h->st));
  CK(cudaMemcpyAsync(asz.data(), h->ed.asz, sizeof(double) * N, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  const double pi = std::acos(-1.0);
  std::vector<GustPt> pts;
  std::vector<GustPt64> p64;
  const int nbc = h->nb / h->ncase;
  for (int cs = 0; cs < h->ncase; cs++) {
    if (h->htc[cs].n == 0) continue;
    const ati_config_t &cfg = h->cfgs[cs];
    const double xg = -(double)0.7f * cfg.domlen + cfg.szth1, ra0 = pi / cfg.szth1;
    const size_t first = pts.size();
    for (int b = h->case_b0[cs]; b < h->case_b0[cs] + nbc; b++) {
      const BlockDev &B = h->blk[b];
      for (int64_t g = B.off; g < B.off + B.npts; g++) {
        const double x = xyz[g];
        if (asz[g] == 0.0 || !(x < xg)) continue;  // asz carries the sign of 1/J
        const double s = std::sin(std::fmin(ra0 * (x + cfg.domlen), 0.5 * pi));
        pts.push_back(GustPt{g, (float)x, (float)xyz[g + N], (float)xyz[g + 2 * N], (float)(s * s), cs, 0});
        p64.push_back(GustPt64{x, xyz[g + N], xyz[g + 2 * N], s * s});
      }
    }
    while ((pts.size() - first) % 256) {
      pts.push_back(GustPt{-1, 0.f, 0.f, 0.f, 0.f, cs, 0});
      p64.push_back(GustPt64{0.0, 0.0, 0.0, 0.0});
    }
  }
  h->ngust = (int64_t)pts.size();
  if (h->ngust == 0) return ATI_OK;
  auto alloc = [&](void **p, size_t n) { return cudaMalloc(p, n) == cudaSuccess; };
  if (!alloc((void **)&h->dgust, sizeof(GustPt) * pts.size()) || !alloc((void **)&h->ddelta, sizeof(float) * 5 * pts.size()) ||
      !alloc((void **)&h->dmodes, sizeof(float) * h->hmodes.size()) || !alloc((void **)&h->dtc, sizeof(TurbCase) * h->ncase) ||
      (fp64 && (!alloc((void **)&h->dgust64, sizeof(GustPt64) * p64.size()) ||
                !alloc((void **)&h->ddelta64, sizeof(double) * 5 * p64.size())))) {
    cudaGetLastError();
    return fail(h, ATI_ENOMEM, "inflow turbulence: device allocation failed");
  }
  CK(cudaMemcpyAsync(h->dgust, pts.data(), sizeof(GustPt) * pts.size(), cudaMemcpyHostToDevice, h->st));
  CK(cudaMemcpyAsync(h->dmodes, h->hmodes.data(), sizeof(float) * h->hmodes.size(), cudaMemcpyHostToDevice, h->st));
  CK(cudaMemcpyAsync(h->dtc, h->htc.data(), sizeof(TurbCase) * h->ncase, cudaMemcpyHostToDevice, h->st));
  CK(cudaMemsetAsync(h->ddelta, 0, sizeof(float) * 5 * pts.size(), h->st));
  if (fp64) {
    CK(cudaMemcpyAsync(h->dgust64, p64.data(), sizeof(GustPt64) * p64.size(), cudaMemcpyHostToDevice, h->st));
    CK(cudaMemsetAsync(h->ddelta64, 0, sizeof(double) * 5 * p64.size(), h->st));
  }
  CK(cudaStreamSynchronize(h->st));
  return ATI_OK;
}

extern "C" int ati_init(ati_handle_t *h) {
  if (!h) return fail(h, ATI_EINVAL, "null handle");
  for (int b = 0; b < h->nb; b++)
    if (!h->grid_set[b]) return fail(h, ATI_ESTATE, "ati_init: grid of block " + std::to_string(b) + " not set");
  Eng<double> &c = h->ed;
  const int64_t N = h->N;
  drop_graphs(h);
  // coordinate derivatives (src/Main3D.f90:365-375)
  double *dst[3] = {c.qo, c.qa, c.de};
  for (int m = 1; m <= 3; m++) {
    CK(cudaMemcpyAsync(h->rr, h->ss + (m - 1) * N, sizeof(double) * N, cudaMemcpyDeviceToDevice, h->st));
    int rc = ati_mpigo(h, 0, 1, 1);
    if (!rc) rc = ati_deriv(h, 3, 1, m);
    if (!rc) rc = ati_deriv(h, 2, 1, m);
    if (!rc) rc = ati_deriv(h, 1, 1, m);
    if (rc) return rc;
    CK(cudaMemcpyAsync(dst[m - 1], h->rr, sizeof(double) * 3 * N, cudaMemcpyDeviceToDevice, h->st));
  }
  strict::metrics(c, h->st, nullptr);
  CKL();
  // wall area and normals (from the coordinate derivatives still in qo/qa/de)
  if (h->tl_force.n) {
    k_wall_geom<<<dim3((h->tl_force.maxline + 127) / 128, h->tl_force.n), 128, 0, h->st>>>(
        c, tp(h, h->tl_force), h->dwoff, h->area, h->wnor);
    CKL();
  }
  k_cm<<<dim3((h->tl_all.maxline + 127) / 128, h->tl_all.n), 128, 0, h->st>>>(c, tp(h, h->tl_all));
  CKL();
  // GCBC weights: visit counts in the granular scratch plane
  CK(cudaMemsetAsync(h->fw1, 0, sizeof(double) * N, h->st));
  if (h->tl_gcbc.n) {
    dim3 g((h->tl_gcbc.maxline + 127) / 128, h->tl_gcbc.n);
    k_sbcc_count<<<g, 128, 0, h->st>>>(c, tp(h, h->tl_gcbc), h->fw1);
    k_sbcc_weight<<<g, 128, 0, h->st>>>(c, tp(h, h->tl_gcbc), h->fw1, h->sh.sbci[1], h->sh.sbci[2], h->sh.sbci[3]);
    CKL();
  }
  // sponge (the grid coordinates are still in ss)
  k_sponge<<<dim3(64, h->nb), 256, 0, h->st>>>(c, h->ss, h->dspg, std::acos(-1.0));
  CKL();
  if (h->mixed) {  // FP32 copies of everything the mixed stage reads
    Eng<float> &m = h->ef;
    int rc = to_float(h, c.xim, m.xim, 3 * N);
    if (!rc) rc = to_float(h, c.etm, m.etm, 3 * N);
    if (!rc) rc = to_float(h, c.zem, m.zem, 3 * N);
    if (!rc) rc = to_float(h, c.yaco, m.yaco, N);
    if (!rc) rc = to_float(h, c.asz, m.asz, N);
    if (!rc) rc = to_float(h, c.bsz, m.bsz, N);
    if (!rc) rc = to_float(h, c.cm, m.cm, 6 * h->F);
    if (!rc) rc = to_float(h, c.sbcc, m.sbcc, h->nsbcc);
    if (!rc) rc = to_float(h, c.rpex, m.rpex, h->nwall);
    if (rc) return rc;
    // metric divergence and its line-end values, FP64, for the freestream part of the fluxes: the same closure and
    // sweeps as the flux derivatives (n45 = 0), applied to xim/etm/zem; flx is free scratch here
    strict::mpigo_ddd(c, h->st, tp(h, h->tl_mpigo), h->tl_mpigo.n, h->tl_mpigo.maxline, 0, 0, c.xim, c.etm, c.zem, N,
                      3);
    const double *mf[3] = {c.xim, c.etm, c.zem};
    for (int nn = 1; nn <= 3; nn++) {
      SweepIO<double, double> io{mf[nn - 1], N, c.flx + 3 * (nn - 1) * N, N, nullptr, 3, 1, true};
      strict::sweep_ddd(c, h->st, nn, false, io);
    }
    strict::metric_divergence(c, h->st, c.flx, const_cast<float *>(m.gm));
    CKL();
    rc = to_float(h, c.drva, const_cast<float *>(m.drvm), 10 * h->F);
    if (rc) return rc;
  }
  {
    int rc = setup_gust(h);
    if (rc) return rc;
  }
  // initial condition and time scalars (src/Main3D.f90:520-522)
  k_ic<<<256, 256, 0, h->st>>>(c);
  CKL();
  CK(cudaMemsetAsync(c.scal, 0, sizeof(Scalars) * h->ncase, h->st));
  strict::scalar(c, h->st, SC_INIT, 0);
  CKL();
  CK(cudaStreamSynchronize(h->st));
  if (h->tune)
    if (int rc = autotune(h)) return rc;
  h->n_host = 0;
  h->steps_done = 0;
  h->inited = true;
  return ATI_OK;
}

// ---- fused calls ----------------------------------------------------------------
// The stage engine, for both the FP64 (double intermediates) and the mixed
// (float intermediates) cases.  Same sequence as src/Main3D.f90:555-952 with
// the per-variable loops turned into multi-field launches.
template <typename R>
struct EngineCalls;

template <>
struct EngineCalls<double> {
  static void sweep(bool strict, const Eng<double> &e, cudaStream_t st, int nn, bool filt,
                    const SweepIO<double, double> &io) {
    if (strict) strict::sweep_ddd(e, st, nn, filt, io);
    else fast::sweep_ddd(e, st, nn, filt, io);
  }
  static void qsweep(bool strict, const Eng<double> &e, cudaStream_t st, int nn, const SweepIO<double, double> &io) {
    sweep(strict, e, st, nn, true, io);
  }
  static void mpigo(bool strict, const Eng<double> &e, cudaStream_t st, const FaceTask *t, int n, int ml, int nt,
                    const double *s1, const double *s2, const double *s3, int64_t fs, int nf) {
    if (strict) strict::mpigo_ddd(e, st, t, n, ml, nt, 0, s1, s2, s3, fs, nf);
    else fast::mpigo_ddd(e, st, t, n, ml, nt, 0, s1, s2, s3, fs, nf);
  }
  static void qmpigo(bool strict, const Eng<double> &e, cudaStream_t st, const FaceTask *t, int n, int ml,
                     const double *q, int64_t fs, const FieldOfs<double> &) {
    mpigo(strict, e, st, t, n, ml, 1, q, q, q, fs, 5);
  }
  static void pw(bool strict, const Eng<double> &e, cudaStream_t st, int which) {
    if (strict) strict::pointwise_d(e, st, which);
    else fast::pointwise_d(e, st, which);
  }
  static void face(bool strict, const Eng<double> &e, cudaStream_t st, int which, const FaceTask *t, int n, int ml) {
    if (strict) strict::face_d(e, st, which, t, n, ml);
    else fast::face_d(e, st, which, t, n, ml);
  }
};

template <>
struct EngineCalls<float> {
  static void sweep(bool, const Eng<float> &e, cudaStream_t st, int nn, bool filt, const SweepIO<float, float> &io) {
    fast::sweep_fff(e, st, nn, filt, io);
  }
  static void qsweep(bool, const Eng<float> &e, cudaStream_t st, int nn, const SweepIO<double, double> &io) {
    fast::sweep_ddf(e, st, nn, true, io);
  }
  static void mpigo(bool, const Eng<float> &e, cudaStream_t st, const FaceTask *t, int n, int ml, int nt,
                    const float *s1, const float *s2, const float *s3, int64_t fs, int nf) {
    fast::mpigo_fff(e, st, t, n, ml, nt, 0, s1, s2, s3, fs, nf);
  }
  static void qmpigo(bool, const Eng<float> &e, cudaStream_t st, const FaceTask *t, int n, int ml, const double *q,
                     int64_t fs, const FieldOfs<double> &fo) {
    fast::mpigo_ddf(e, st, t, n, ml, 1, 0, q, q, q, fs, 5, fo);
  }
  static void pw(bool, const Eng<float> &e, cudaStream_t st, int which) { fast::pointwise_f(e, st, which); }
  static void face(bool, const Eng<float> &e, cudaStream_t st, int which, const FaceTask *t, int n, int ml) {
    fast::face_f(e, st, which, t, n, ml);
  }
};

// Tile shapes timed on the handle's own grid: lines per CTA of the eta/zeta
// sweeps (a 5-field derivative sweep of each direction, into scratch planes)
// and points per pointwise tile (the flux kernel).  Every line and every point
// is computed the same way whatever the tiles, so the choice changes timings only.
template <typename R>
static int autotune_t(ati_handle *h, Eng<R> &e) {
  using C = EngineCalls<R>;
  const bool strict = h->cfg.precision == ATI_FP64_STRICT;
  const int64_t N = h->N;
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  // a buffer larger than L2, written before every timed run so that each candidate reads its inputs from DRAM
  // as it does inside a step (timed back to back on the same arrays, L2 would favour low occupancy)
  const size_t flush_bytes = 256u << 20;
  void *flush = nullptr;
  if (cudaMalloc(&flush, flush_bytes) != cudaSuccess) {
    cudaGetLastError();
    flush = nullptr;
  }
  auto time_it = [&](auto &&fn) {
    if (flush) cudaMemsetAsync(flush, 0, flush_bytes, h->st);
    cudaEventRecord(a, h->st);
    fn();
    cudaEventRecord(b, h->st);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
  };
  // candidates are timed in turn, five rounds, best of each; a candidate replaces
  // the default only when it is at least 3 % faster (timings of one launch are noisy)
  auto pick = [&](const std::vector<int> &cand, int dflt, auto &&setup, auto &&run) -> int {
    std::vector<float> best(cand.size(), 1e30f);
    for (int round = 0; round < 5; round++)
      for (size_t q = 0; q < cand.size(); q++) {
        setup(cand[q]);
        run();  // warm
        best[q] = std::min(best[q], time_it(run));
      }
    size_t qd = 0, qb = 0;
    for (size_t q = 0; q < cand.size(); q++) {
      if (cand[q] == dflt) qd = q;
      if (best[q] < best[qb]) qb = q;
    }
    return best[qb] < 0.97f * best[qd] ? cand[qb] : dflt;
  };
  auto set_tiles = [&](int sg2, int sg3, int pt) {
    make_tiles(h, sg2, sg3, pt);
    upload_tiles(h);
    e.npt = h->ed.npt;
    for (int nn = 0; nn < 4; nn++) e.sg_lines[nn] = h->sg_lines[nn];
    for (int nn = 1; nn <= 3; nn++) e.nlt[nn] = h->ed.nlt[nn];
  };
  // eta and zeta apart: the line length decides whether the forward values fit shared memory
  auto sweep_of = [&](int nn) {
    return [&, nn] {
      SweepIO<R, R> io{e.flx, 3 * N, e.dv, 3 * N, nullptr, 5, 1, false};
      C::sweep(strict, e, h->st, nn, false, io);
    };
  };
  // (the mixed path solves every line in segmented tiles of fixed shape: only its point tiles are timed)
  const std::vector<int> sgc{SG_MIN, 2 * SG_MIN, SG_DEFAULT, SG_MAX};
  int sg2 = SG_DEFAULT, sg3 = SG_DEFAULT;
  if (!h->mixed) {
    sg2 = pick(sgc, SG_DEFAULT, [&](int v) { set_tiles(v, SG_DEFAULT, PT_DEFAULT); }, sweep_of(2));
    sg3 = pick(sgc, SG_DEFAULT, [&](int v) { set_tiles(sg2, v, PT_DEFAULT); }, sweep_of(3));
  }
  set_tiles(sg2, sg3, PT_DEFAULT);
  // point tiles, per pointwise kernel: their best sizes differ (the tile's set-up is a chain of dependent loads
  // that small tiles repeat for every point; large tiles leave a partial last wave of CTAs)
  const int flux_kind = stress_at_point(h) ? PW_FLUX_STRESS : PW_FLUX;
  std::vector<int> kinds{PW_PRIM, flux_kind, PW_DIV, PW_RK};
  if (!stress_at_point(h) && h->cfg.nviscous == 1) kinds.push_back(PW_VISC);
  // the RK update rewrites qa from qo and de: qa is kept aside and put back (de and the stage planes written
  // here are recomputed before they are read)
  double *keep = h->ed.fw;
  CK(cudaMemcpyAsync(keep, h->ed.qa, sizeof(double) * 5 * N, cudaMemcpyDeviceToDevice, h->st));
  std::vector<int> cand(PT_CAND, PT_CAND + 3);
  for (int w : kinds) {
    const int v = pick(cand, PT_DEFAULT, [&](int c) { h->pw_pt[w] = c; apply_pw_tiles(h); },
                       [&] { C::pw(strict, e, h->st, w); });
    h->pw_pt[w] = v == PT_DEFAULT ? 0 : v;
    apply_pw_tiles(h);
  }
  h->pw_pt[PW_CFL] = h->pw_pt[PW_PRIM];  // (once every ten steps: it takes the tiles of the same loads)
  apply_pw_tiles(h);
  if (h->pw_pt[flux_kind]) h->pt_points = h->pw_pt[flux_kind];  // the size ati_tiles reports
  CK(cudaMemcpyAsync(h->ed.qa, keep, sizeof(double) * 5 * N, cudaMemcpyDeviceToDevice, h->st));
  if (flush) cudaFree(flush);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  CKL();
  return ATI_OK;
}

static int autotune(ati_handle *h) { return h->mixed ? autotune_t<float>(h, h->ef) : autotune_t<double>(h, h->ed); }

// The derivative sweeps of the three directions within a stage read and write
// disjoint planes and face buffers, so xi runs on the handle's stream and eta,
// zeta on two side streams forked from and joined back into it (inside the step
// graph too): each direction alone leaves the GPU under-occupied.  With
// profiling on they run one after another, so each launch is timed alone.
template <typename F>
static void three_directions(ati_handle *h, F &&sweep) {
  if (h->profiling) {
    for (int nn = 3; nn >= 1; nn--) sweep(nn, h->st);
    return;
  }
  cudaEventRecord(h->ev_fork, h->st);
  for (int q = 0; q < 2; q++) cudaStreamWaitEvent(h->side[q], h->ev_fork, 0);
  sweep(1, h->st);
  sweep(2, h->side[0]);
  sweep(3, h->side[1]);
  for (int q = 0; q < 2; q++) {
    cudaEventRecord(h->ev_join[q], h->side[q]);
    cudaStreamWaitEvent(h->st, h->ev_join[q], 0);
  }
}

template <typename R>
static int filter_step_t(ati_handle *h, const Eng<R> &e) {
  using C = EngineCalls<R>;
  const bool strict = h->cfg.precision == ATI_FP64_STRICT;
  const int64_t N = h->N;
  // per-step filter of the five variables in place on qa, then qo = qa
  // (src/Main3D.f90:555-561); the last sweep writes qo as well
  // the mixed path filters q - q_inf (rho_inf = 1, rhoE_inf = p_inf/(gamma-1)): the filter annihilates constants,
  // and removing them before the FP32 rounding keeps the rounding relative to the deviation
  FieldOfs<double> fo{};
  if (Freestream<R>::on) { fo.v[0] = h->sh.s.rhooo; fo.v[4] = h->sh.s.hamm1 * h->sh.s.poo; }
  PROF(h, ATI_K_MPIGO, C::qmpigo(strict, e, h->st, tp(h, h->tl_mpigo), h->tl_mpigo.n, h->tl_mpigo.maxline, h->ed.qa, N, fo));
  for (int nn = 1; nn <= 3; nn++) {
    SweepIO<double, double> io{h->ed.qa, N, h->ed.qa, N, nn == 3 ? h->ed.qo : nullptr, 5, 1, false};
    for (int f = 0; f < 5; f++) io.ofs[f] = fo.v[f];
    PROF(h, ATI_K_FILTER_XI + nn - 1, C::qsweep(strict, e, h->st, nn, io));
  }
  CKL();
  return ATI_OK;
}

template <typename R>
static cudaError_t face_pre(bool strict, const Eng<R> &e, cudaStream_t st, const FaceChain &c) {
  if constexpr (std::is_same<R, float>::value) return fast::face_pre_f(e, st, c);
  else return strict ? strict::face_pre_d(e, st, c) : fast::face_pre_d(e, st, c);
}

template <typename R>
static int rk_stage_t(ati_handle *h, const Eng<R> &e, int nk) {
  using C = EngineCalls<R>;
  const bool strict = h->cfg.precision == ATI_FP64_STRICT;
  cudaStream_t st = h->st;
  const int64_t N = h->N;
  const Eng<double> &ed = h->ed;
  const TaskRange &mpt = Freestream<R>::on ? h->tl_mpigo_x : h->tl_mpigo;  // (segmented sweeps: see tl_mpigo_x)
  auto sc = [&](int op) {
    if (strict) strict::scalar(ed, st, op, nk);
    else fast::scalar(ed, st, op, nk);
  };
  PROF(h, ATI_K_SCALAR, sc(SC_MOVEF_A));
  PROF(h, ATI_K_PRIM, C::pw(strict, e, st, PW_PRIM));
  if (nk == 1) {
    if (h->n_host % 10 == 1) {
      if (h->any_cfl) {
        PROF(h, ATI_K_SCALAR, sc(SC_CFL_RESET));
        PROF(h, ATI_K_CFL, C::pw(strict, e, st, PW_CFL));
      }
      PROF(h, ATI_K_SCALAR, sc(SC_DT_NEW));
    }
    PROF(h, ATI_K_SCALAR, sc(SC_DT));
  }
  if (h->cfg.nviscous == 1) {
    // d(u,v,w,T)/d(zeta,eta,xi) (src/Main3D.f90:629-651): four fields per launch
    PROF(h, ATI_K_MPIGO, C::mpigo(strict, e, st, tp(h, mpt), mpt.n, mpt.maxline, 0, e.prim,
                                  e.prim, e.prim, N, 4));
    three_directions(h, [&](int nn, cudaStream_t s) {
      SweepIO<R, R> io{e.prim, N, e.dv + (nn - 1) * N, 3 * N, nullptr, 4, 2, true};
      PROF(h, ATI_K_DERIV_XI + nn - 1, C::sweep(strict, e, s, nn, false, io));
    });
    if (!stress_at_point(h)) PROF(h, ATI_K_VISC, C::pw(strict, e, st, PW_VISC));
  }
  // fluxes and their derivatives (src/Main3D.f90:710-768): five fields per launch; the mixed path and the FP64
  // fast path take the stresses inside the flux kernel and leave the stress planes to stress_planes()
  const bool fused = stress_at_point(h);
  PROF(h, ATI_K_FLUX, C::pw(strict, e, st, fused ? PW_FLUX_STRESS : PW_FLUX));
  PROF(h, ATI_K_MPIGO, C::mpigo(strict, e, st, tp(h, mpt), mpt.n, mpt.maxline, 0, e.flx,
                                e.flx + N, e.flx + 2 * N, 3 * N, 5));
  three_directions(h, [&](int nn, cudaStream_t s) {
    SweepIO<R, R> io{e.flx + (nn - 1) * N, 3 * N, e.flx + (nn - 1) * N, 3 * N, nullptr, 5, 1, true};
    PROF(h, ATI_K_DERIV_XI + nn - 1, C::sweep(strict, e, s, nn, false, io));
  });
  PROF(h, ATI_K_DIV, C::pw(strict, e, st, PW_DIV));
  if (h->ngust) {
    // inflow turbulence: the gust targets of the inflow sponge, evaluated on the steps that take a new dt
    // (n % 10 == 1, and the first step) and held in between: 10 steps are a few thousandths of the eddies'
    // convective time L / U_inf, and the 2048-mode synthesis would otherwise cost more than the sponge it feeds
    // (the strict mode, the parity mode, sums the modes in FP64 in the CPU restatement's order; the others in FP32)
    const bool g64 = h->dgust64 != nullptr;
    const Scheme &S0 = h->sh.s;
    if (nk == 1 && (h->n_host % 10 == 1 || h->steps_done == 0)) {
      if (g64)
        PROF(h, ATI_K_DIV, gust_eval64(st, h->dgust, h->dgust64, h->ngust, h->dtc, h->dmodes, ed.scal, h->ddelta64,
                                       S0.gam, S0.gamm1, S0.hamm1, S0.ham));
      else PROF(h, ATI_K_DIV, gust_eval(st, h->dgust, h->ngust, h->dtc, h->dmodes, ed.scal, h->ddelta, S0.gam));
    }
    if constexpr (std::is_same<R, float>::value)
      PROF(h, ATI_K_DIV, gust_apply_f(st, h->dgust, h->ngust, h->ddelta, ed.asz, ed.bsz, e.de, N));
    else if (g64) PROF(h, ATI_K_DIV, gust_apply64(st, h->dgust, h->ngust, h->ddelta64, ed.asz, ed.bsz, e.de, N));
    else PROF(h, ATI_K_DIV, gust_apply_d(st, h->dgust, h->ngust, h->ddelta, ed.asz, ed.bsz, e.de, N));
  }
  if (h->fused) {
    // the face chains fused: one cooperative launch before the RK update (characteristic boundaries of every
    // direction, frame update) and one after it (wall, junctions, interface averaging), phases ordered by bounded
    // grid barriers (src/Main3D.f90:780-952)
    auto span = [&](const TaskRange &r) { return TaskSpan{tp(h, r), h->dcum + r.off, r.n, h->task_lines(r.off, r.n)}; };
    FaceChain pre{}, post{};
    pre.prep = span(h->tl_gcbc);
    for (int d = 1; d <= 3; d++) pre.dir[d] = span(h->tl_gcbc_dir[d]);
    pre.bar = h->dbar;
    pre.limit = h->spin_limit;
    pre.nk = nk;
    post.prep = span(h->tl_wall);
    post.pack = span(h->tl_pack);
    for (int d = 1; d <= 3; d++) post.dir[d] = span(h->tl_avg_dir[d]);
    post.jn = h->djn;
    post.njct = h->njct;
    post.jnk = h->jnk;
    post.bar = h->dbar + 1;
    post.limit = h->spin_limit;
    post.nk = nk;
    CK(cudaMemsetAsync(h->dbar, 0, sizeof(unsigned) * 2, st));
    cudaError_t ce = cudaSuccess;
    PROF(h, ATI_K_GCBC, ce = face_pre<R>(strict, e, st, pre));
    if (ce != cudaSuccess) return fail(h, ATI_ECUDA, std::string("fused face chain: ") + cudaGetErrorString(ce));
    PROF(h, ATI_K_RK, C::pw(strict, e, st, PW_RK));
    PROF(h, ATI_K_AVERAGE, ce = (strict ? strict::face_post : fast::face_post)(ed, st, post));
    if (ce != cudaSuccess) return fail(h, ATI_ECUDA, std::string("fused face chain: ") + cudaGetErrorString(ce));
    CKL();
    return ATI_OK;
  }
  // characteristic boundary conditions (src/Main3D.f90:780-869)
  if (h->tl_gcbc.n) PROF(h, ATI_K_GCBC, C::face(strict, e, st, FK_GCBC_PREP, tp(h, h->tl_gcbc), h->tl_gcbc.n, h->tl_gcbc.maxline));
  for (int d = 1; d <= 3; d++)
    if (h->tl_gcbc_dir[d].n)
      PROF(h, ATI_K_GCBC, C::face(strict, e, st, FK_GCBC_APPLY, tp(h, h->tl_gcbc_dir[d]), h->tl_gcbc_dir[d].n,
                                  h->tl_gcbc_dir[d].maxline));
  // RK update, wall, junction, interface averaging (src/Main3D.f90:873-952)
  PROF(h, ATI_K_SCALAR, sc(SC_MOVEF_B));
  PROF(h, ATI_K_RK, C::pw(strict, e, st, PW_RK));
  auto fd = [&](int which, const TaskRange &r) {
    if (!r.n) return;
    if (strict) strict::face_d(ed, st, which, tp(h, r), r.n, r.maxline);
    else fast::face_d(ed, st, which, tp(h, r), r.n, r.maxline);
  };
  PROF(h, ATI_K_WALL_JUNCTION, fd(FK_WALL, h->tl_wall));
  PROF(h, ATI_K_WALL_JUNCTION, (strict ? strict::junction : fast::junction)(ed, st, h->djn, h->njct, h->jnk));
  PROF(h, ATI_K_AVERAGE, fd(FK_PACK, h->tl_pack));
  for (int d = 1; d <= 3; d++) PROF(h, ATI_K_AVERAGE, fd(FK_AVG, h->tl_avg_dir[d]));
  CKL();
  return ATI_OK;
}

static int filter_step(ati_handle *h) { return h->mixed ? filter_step_t<float>(h, h->ef) : filter_step_t<double>(h, h->ed); }
static int rk_stage(ati_handle *h, int nk) { return h->mixed ? rk_stage_t<float>(h, h->ef, nk) : rk_stage_t<double>(h, h->ed, nk); }

static int one_step(ati_handle *h) {
  int rc = filter_step(h);
  for (int nk = 1; nk <= h->cfg.nkrk && !rc; nk++) rc = rk_stage(h, nk);
  if (rc) return rc;
  const bool strict = h->cfg.precision == ATI_FP64_STRICT;
  PROF(h, ATI_K_SCALAR, (strict ? strict::scalar : fast::scalar)(h->ed, h->st, SC_ADVANCE, 0));
  if (h->probe_cap > 0 && h->tl_force.n) {
    h->launches++;
    k_wall_probe<<<1, 256, 0, h->st>>>(h->ed, tp(h, h->tl_force), h->tl_force.n, h->probe_n0, h->probe_cap,
                                       h->probe_npts, h->probe_p, h->probe_t);
  }
  CKL();
  return ATI_OK;
}

// The failure flags of every case, after the handle's work in flight (a bounded wait when the handle has a wait
// limit: the copy is issued only once the stream is idle, so a timed-out wait leaves no copy behind).
static int read_flags(ati_handle *h, std::vector<Scalars> &sc) {
  if (int rc = wait_stream(h)) return rc;
  sc.resize(h->ncase);
  CK(cudaMemcpyAsync(sc.data(), h->ed.scal, sizeof(Scalars) * h->ncase, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  return ATI_OK;
}

// the status a case's device flag stands for
static int flag_status(ati_handle *h, int c, int flag) {
  if (flag & FLAG_TIMEOUT)
    return fail(h, ATI_ETIMEDOUT, "a bounded device wait of case " + std::to_string(c) + " gave up (flag " +
                                      std::to_string(flag) + ")");
  if (flag)
    return fail(h, ATI_ENONFINITE, "non-finite or non-positive density/pressure in the state of case " +
                                       std::to_string(c) + " (flag " + std::to_string(flag) + ")");
  return ATI_OK;
}

static int check_flag(ati_handle *h) {
  std::vector<Scalars> sc;
  if (int rc = read_flags(h, sc)) return rc;
  for (int c = 0; c < h->ncase; c++)
    if (sc[c].flag) return flag_status(h, c, sc[c].flag);
  return ATI_OK;
}

extern "C" int ati_case_check(ati_handle_t *h, int cs) {
  if (!h || cs < 0 || cs >= h->ncase) return fail(h, ATI_EINVAL, "ati_case_check: bad argument");
  if (!h->inited) return fail(h, ATI_ESTATE, "ati_init not called");
  std::vector<Scalars> sc;
  if (int rc = read_flags(h, sc)) return rc;
  return flag_status(h, cs, sc[cs].flag);
}

extern "C" int ati_filter_step(ati_handle_t *h) {
  if (!h) return fail(h, ATI_EINVAL, "null handle");
  if (!h->inited) return fail(h, ATI_ESTATE, "ati_init not called");
  return filter_step(h);
}

extern "C" int ati_rk_stage(ati_handle_t *h, int nk) {
  if (!h) return fail(h, ATI_EINVAL, "null handle");
  if (!h->inited) return fail(h, ATI_ESTATE, "ati_init not called");
  if (nk < 1 || nk > h->cfg.nkrk) return fail(h, ATI_EINVAL, "ati_rk_stage: nk out of range");
  return rk_stage(h, nk);
}

// A whole time step is captured once into a CUDA graph per variant (with and
// without the new-dt-target kernels of n % 10 == 1) and replayed; the first
// step of a case runs eagerly so every kernel attribute is set before capture.
static int step_graph(ati_handle *h) {
  const int v = (h->n_host % 10 == 1) ? 1 : 0;
  if (!h->gexec[v]) {
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
    const int64_t l0 = h->launches;
    int rc = one_step(h);
    cudaError_t e = cudaStreamEndCapture(h->st, &g);
    h->launches = l0;
    if (rc) return rc;
    if (e != cudaSuccess) return fail(h, ATI_ECUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    // the kernels the graph holds (launch sites that had nothing to do launched nothing)
    size_t nnode = 0;
    e = cudaGraphGetNodes(g, nullptr, &nnode);
    std::vector<cudaGraphNode_t> nodes(nnode);
    if (e == cudaSuccess && nnode) e = cudaGraphGetNodes(g, nodes.data(), &nnode);
    int64_t nk = 0;
    for (size_t q = 0; q < nnode && e == cudaSuccess; q++) {
      cudaGraphNodeType t;
      e = cudaGraphNodeGetType(nodes[q], &t);
      if (t == cudaGraphNodeTypeKernel) nk++;
    }
    if (e != cudaSuccess) {
      cudaGraphDestroy(g);
      return fail(h, ATI_ECUDA, std::string("graph nodes: ") + cudaGetErrorString(e));
    }
    h->glaunches[v] = nk;
    e = cudaGraphInstantiate(&h->gexec[v], g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(h, ATI_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  }
  h->launches += h->glaunches[v];  // the kernels the graph replays
  CK(cudaGraphLaunch(h->gexec[v], h->st));
  return ATI_OK;
}

static int issue_steps(ati_handle *h, int nsteps) {
  if (!h) return fail(h, ATI_EINVAL, "null handle");
  if (!h->inited) return fail(h, ATI_ESTATE, "ati_init not called");
  if (nsteps < 0) return fail(h, ATI_EINVAL, "nsteps < 0");
  for (int s = 0; s < nsteps; s++) {
    int rc;
    if (h->profiling || !h->graphs_ok || h->steps_done == 0) {
      rc = one_step(h);
    } else {
      rc = step_graph(h);
    }
    if (rc) return rc;
    h->n_host++;
    h->steps_done++;
  }
  return ATI_OK;
}

extern "C" int ati_step(ati_handle_t *h, int nsteps) {
  int rc = issue_steps(h, nsteps);
  return rc ? rc : check_flag(h);
}

extern "C" int ati_step_async(ati_handle_t *h, int nsteps) { return issue_steps(h, nsteps); }

extern "C" int ati_query(ati_handle_t *h, int *idle) {
  if (!h || !idle) return fail(h, ATI_EINVAL, "ati_query: bad argument");
  const cudaError_t e = cudaStreamQuery(h->st);
  if (e == cudaSuccess) *idle = 1;
  else if (e == cudaErrorNotReady) *idle = 0;
  else return fail(h, ATI_ECUDA, std::string("cudaStreamQuery: ") + cudaGetErrorString(e));
  return ATI_OK;
}

extern "C" int ati_check(ati_handle_t *h) {
  if (!h) return fail(h, ATI_EINVAL, "null handle");
  return check_flag(h);
}

extern "C" int ati_case_forces(ati_handle_t *h, int cs, double out[2]) {
  if (!h || !out || cs < 0 || cs >= h->ncase) return fail(h, ATI_EINVAL, "forces: bad argument");
  if (!h->inited) return fail(h, ATI_ESTATE, "ati_init not called");
  const TaskRange &r = h->tl_force_c[cs];
  const int q0 = r.off - h->tl_force.off;  // position in the wall-face list
  stress_planes(h);
  if (h->mixed) strict::forces_f(h->ef, h->st, tp(h, r), r.n, h->area, h->wnor, h->dwoff + q0, h->dforce + 2 * q0);
  else strict::forces_d(h->ed, h->st, tp(h, r), r.n, h->area, h->wnor, h->dwoff + q0, h->dforce + 2 * q0);
  CKL();
  std::vector<double> part((size_t)2 * r.n);
  CK(cudaMemcpyAsync(part.data(), h->dforce + 2 * q0, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  const Scheme &S = h->shc[cs].s;
  const double dynp = 2.0 / (S.amachoo * S.amachoo * h->cfgs[cs].span);
  out[0] = 0.0; out[1] = 0.0;
  for (int q = 0; q < r.n; q++) {  // blocks in rank order, as MPI_REDUCE over wcom
    out[0] = out[0] + part[2 * q] * dynp;
    out[1] = out[1] + part[2 * q + 1] * dynp;
  }
  return ATI_OK;
}

extern "C" int ati_forces(ati_handle_t *h, double out[2]) { return ati_case_forces(h, 0, out); }

extern "C" int ati_case_config(ati_handle_t *h, int cs, ati_config_t *cfg) {
  if (!h || !cfg || cs < 0 || cs >= h->ncase) return fail(h, ATI_EINVAL, "config: bad argument");
  *cfg = h->cfgs[cs];
  return ATI_OK;
}

extern "C" int ati_get_config(ati_handle_t *h, ati_config_t *cfg) { return ati_case_config(h, 0, cfg); }

extern "C" int ati_case_frame(ati_handle_t *h, int cs, double umf[3], double *aoa) {
  if (!h || !umf || !aoa || cs < 0 || cs >= h->ncase) return fail(h, ATI_EINVAL, "frame: bad argument");
  Scalars sc;
  CK(cudaMemcpyAsync(&sc, h->ed.scal + cs, sizeof(sc), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  for (int q = 0; q < 3; q++) umf[q] = sc.umf[q + 1];
  *aoa = sc.aoa;
  return ATI_OK;
}

extern "C" int ati_get_frame(ati_handle_t *h, double umf[3], double *aoa) { return ati_case_frame(h, 0, umf, aoa); }

// ---- surface-pressure recorder ----------------------------------------------------

extern "C" int ati_wall_probe_enable(ati_handle_t *h, int capacity) {
  if (!h || capacity < 0) return fail(h, ATI_EINVAL, "ati_wall_probe_enable: bad argument");
  if (!h->inited) return fail(h, ATI_ESTATE, "ati_init not called");
  if (h->ncase > 1) return fail(h, ATI_EINVAL, "ati_wall_probe_enable: single-case handles only");
  CK(cudaStreamSynchronize(h->st));
  probe_free(h);
  drop_graphs(h);  // the step graphs hold (or lack) the recording kernel
  if (capacity == 0) return ATI_OK;
  int64_t npts = 0;
  for (int q = 0; q < h->tl_force.n; q++) npts += h->blk[h->htasks[h->tl_force.off + q].b].lxi + 1;
  if (npts == 0) return fail(h, ATI_EINVAL, "ati_wall_probe_enable: the case has no wall face");
  if (cudaMalloc(&h->probe_p, sizeof(double) * npts * capacity) != cudaSuccess ||
      cudaMalloc(&h->probe_t, sizeof(double) * capacity) != cudaSuccess) {
    cudaGetLastError();
    probe_free(h);
    return fail(h, ATI_ENOMEM, "ati_wall_probe_enable: device allocation failed");
  }
  h->probe_cap = capacity;
  h->probe_npts = npts;
  h->probe_n0 = h->n_host;
  return ATI_OK;
}

extern "C" int ati_wall_probe_read(ati_handle_t *h, double *p, double *t, int64_t *nrec, int64_t *npts) {
  if (!h || !nrec || !npts) return fail(h, ATI_EINVAL, "ati_wall_probe_read: bad argument");
  if (h->probe_cap == 0) return fail(h, ATI_ESTATE, "ati_wall_probe_read: recorder not enabled");
  const int64_t done = h->n_host - h->probe_n0, cap = h->probe_cap;
  const int64_t nr = done < cap ? done : cap;
  *nrec = nr;
  *npts = h->probe_npts;
  if (!p) return ATI_OK;
  // oldest record kept sits at slot (done - nr) mod cap: at most two contiguous runs
  const int64_t s0 = (done - nr) % cap, run1 = nr < cap - s0 ? nr : cap - s0, np = h->probe_npts;
  CK(cudaMemcpyAsync(p, h->probe_p + s0 * np, sizeof(double) * np * run1, cudaMemcpyDeviceToHost, h->st));
  if (nr > run1)
    CK(cudaMemcpyAsync(p + run1 * np, h->probe_p, sizeof(double) * np * (nr - run1), cudaMemcpyDeviceToHost, h->st));
  if (t) {
    CK(cudaMemcpyAsync(t, h->probe_t + s0, sizeof(double) * run1, cudaMemcpyDeviceToHost, h->st));
    if (nr > run1) CK(cudaMemcpyAsync(t + run1, h->probe_t, sizeof(double) * (nr - run1), cudaMemcpyDeviceToHost, h->st));
  }
  CK(cudaStreamSynchronize(h->st));
  return ATI_OK;
}

// ---- instrumentation ------------------------------------------------------------
extern "C" int ati_profile_enable(ati_handle_t *h, int enable) {
  if (!h) return fail(h, ATI_EINVAL, "null handle");
  CK(cudaStreamSynchronize(h->st));
  prof_drain(h);
  h->profiling = enable != 0;
  for (int q = 0; q < ATI_K_NSLOTS; q++) { h->prof_ms[q] = 0.0; h->prof_n[q] = 0; }
  return ATI_OK;
}

extern "C" int ati_profile_read(ati_handle_t *h, int nslots, double *ms, int64_t *launches) {
  if (!h || nslots < 0 || (nslots > 0 && (!ms || !launches))) return fail(h, ATI_EINVAL, "ati_profile_read: bad argument");
  CK(cudaStreamSynchronize(h->st));
  prof_drain(h);
  for (int q = 0; q < nslots && q < ATI_K_NSLOTS; q++) { ms[q] = h->prof_ms[q]; launches[q] = h->prof_n[q]; }
  return ATI_OK;
}

extern "C" int ati_launch_count(ati_handle_t *h, int64_t *count) {
  if (!h || !count) return fail(h, ATI_EINVAL, "ati_launch_count: bad argument");
  *count = h->launches;
  return ATI_OK;
}

extern "C" void *ati_stream(ati_handle_t *h) { return h ? (void *)h->st : nullptr; }
