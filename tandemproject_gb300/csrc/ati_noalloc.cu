// ati_noalloc.cu — the allocation-free variant of the compact derivative.
//
// Some callers cannot allocate GPU memory at the point where they need a
// derivative: a host code that hands every byte of device memory to its own
// pool at start-up, or a time loop that must never allocate once running
// (a device allocation can synchronise the whole device and can fail late,
// when memory is fragmented).  ati_deriv_lines_noalloc serves them: the
// caller passes its own input and output arrays, and the only extra memory
// the kernel needs -- the LU factor table and the forward-elimination values
// -- lives in the file-scope device array below (about 16 MB on every GPU that
// uses it, held until the process exits).  No call allocates or frees anything.
//
// When the array is reserved: with CUDA's default lazy module loading this file's
// module, and the array with it, is loaded into a context the first time the
// module is used there, which is the first call's address look-up.  That first
// call on a device therefore reserves the 16 MB, and it fails with ATI_ECUDA if
// the device has no 16 MB left.  A caller whose own pool takes the device memory
// makes one call (nlines may be 1) before the pool does, and before any stream
// capture; with CUDA_MODULE_LOADING=EAGER in the environment the driver reserves
// the array when the context is created instead.
//
// Arithmetic: the same one-sided compact scheme as deriv on a line whose two
// ends are physical or interface boundaries (src/Subroutines3D.f90:84-141
// with ndf = 0 at both ends), with the LU factors of penta
// (src/Subroutineso.f90:15-67); this file is compiled without FMA
// contraction, so the results equal ati_deriv's bit for bit.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "../../include/ati.h"

namespace {

constexpr int64_t kMaxPoints = ATI_NOALLOC_MAX_POINTS;
constexpr int kMaxLen = ATI_NOALLOC_MAX_LEN;
constexpr int64_t kScratchDoubles = 5 * (int64_t)kMaxLen + kMaxPoints;

// factor table (5 per line position) followed by the forward-elimination plane
static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr double kAlpha = 0.5862704032801503, kBeta = 0.09549533555017055;
constexpr double kAa = 0.6431406736919156, kAb = 0.2586011023495066, kAc = 0.007140953479797375;

struct Rows {
  double abc[3][6];
  double albe[3][5];  // boundary rows of the left-hand side, offsets -2..2
};

// LU factors of the pentadiagonal left-hand side with one-sided boundary rows
// at both ends, one thread (the recurrence of penta is sequential).
__global__ void k_noalloc_factors(double *fac, int len, Rows R) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  const int is = 0, ie = len - 1;
  double *f = fac;
  for (int i = 0; i < len; i++)
    for (int q = 0; q < 5; q++) f[i * 5 + q] = 1.0;
  // f[i*5 + {0: xl1, 1: xl2, 2: xu1, 3: xu2, 4: xu3}] before the final scaling
  auto S = [&](int o, int r) { return R.albe[r][o + 2]; };
  int i = is;
  f[i * 5 + 2] = 1.0; f[i * 5 + 3] = S(1, 0); f[i * 5 + 4] = S(2, 0);
  i = is + 1;
  f[i * 5 + 1] = S(-1, 1) * f[(i - 1) * 5 + 2];
  f[i * 5 + 2] = 1.0 / (1.0 - f[(i - 1) * 5 + 3] * f[i * 5 + 1]);
  f[i * 5 + 3] = S(1, 1) - f[(i - 1) * 5 + 4] * f[i * 5 + 1];
  f[i * 5 + 4] = S(2, 1);
  i = is + 2;
  f[i * 5 + 0] = S(-2, 2) * f[(i - 2) * 5 + 2];
  f[i * 5 + 1] = (S(-1, 2) - f[(i - 2) * 5 + 3] * f[i * 5 + 0]) * f[(i - 1) * 5 + 2];
  f[i * 5 + 2] = 1.0 / (1.0 - f[(i - 2) * 5 + 4] * f[i * 5 + 0] - f[(i - 1) * 5 + 3] * f[i * 5 + 1]);
  f[i * 5 + 3] = S(1, 2) - f[(i - 1) * 5 + 4] * f[i * 5 + 1];
  f[i * 5 + 4] = S(2, 2);
  for (i = is + 3; i <= ie - 3; i++) {
    f[i * 5 + 0] = kBeta * f[(i - 2) * 5 + 2];
    f[i * 5 + 1] = (kAlpha - f[(i - 2) * 5 + 3] * f[i * 5 + 0]) * f[(i - 1) * 5 + 2];
    f[i * 5 + 2] = 1.0 / (1.0 - f[(i - 2) * 5 + 4] * f[i * 5 + 0] - f[(i - 1) * 5 + 3] * f[i * 5 + 1]);
    f[i * 5 + 3] = kAlpha - f[(i - 1) * 5 + 4] * f[i * 5 + 1];
    f[i * 5 + 4] = kBeta;
  }
  for (int r = 0; r < 3; r++) {  // rows ie-2, ie-1, ie mirror boundary rows 2, 1, 0
    const int k = 2 - r;
    i = ie - 2 + r;
    f[i * 5 + 0] = S(2, k) * f[(i - 2) * 5 + 2];
    f[i * 5 + 1] = (S(1, k) - f[(i - 2) * 5 + 3] * f[i * 5 + 0]) * f[(i - 1) * 5 + 2];
    f[i * 5 + 2] = 1.0 / (1.0 - f[(i - 2) * 5 + 4] * f[i * 5 + 0] - f[(i - 1) * 5 + 3] * f[i * 5 + 1]);
    if (r < 2) f[i * 5 + 3] = S(-1, k) - f[(i - 1) * 5 + 4] * f[i * 5 + 1];
    if (r == 0) f[i * 5 + 4] = S(-2, k);
  }
  for (i = 0; i < len; i++) {
    f[i * 5 + 3] = f[i * 5 + 3] * f[i * 5 + 2];
    f[i * 5 + 4] = f[i * 5 + 4] * f[i * 5 + 2];
  }
}

// one thread per contiguous line: RHS, forward elimination into the scratch
// plane, back substitution into the caller's output
__global__ void k_noalloc_deriv(const double *in, double *out, int64_t nlines, int len, const double *fac,
                                double *fw, Rows R) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nlines) return;
  const int L = len;
  const double *p = in + t * L;
  double *w = fw + t * L;
  double *o = out + t * L;
  const double *a;
  double sbs0, sbs1, sbs2, sbe0, sbe1, sbe2;
  {
    const double w0 = p[0], w1 = p[1], w2 = p[2], w3 = p[3], w4 = p[4], w5 = p[5], w6 = p[6];
    a = R.abc[0];
    sbs0 = a[0] * (w1 - w0) + a[1] * (w2 - w0) + a[2] * (w3 - w0) + a[3] * (w4 - w0) + a[4] * (w5 - w0) + a[5] * (w6 - w0);
    a = R.abc[1];
    sbs1 = a[0] * (w0 - w1) + a[1] * (w2 - w1) + a[2] * (w3 - w1) + a[3] * (w4 - w1) + a[4] * (w5 - w1) + a[5] * (w6 - w1);
    a = R.abc[2];
    sbs2 = a[0] * (w0 - w2) + a[1] * (w1 - w2) + a[2] * (w3 - w2) + a[3] * (w4 - w2) + a[4] * (w5 - w2) + a[5] * (w6 - w2);
  }
  {
    const double w0 = p[L - 1], w1 = p[L - 2], w2 = p[L - 3], w3 = p[L - 4], w4 = p[L - 5], w5 = p[L - 6], w6 = p[L - 7];
    a = R.abc[0];
    sbe0 = a[0] * (w0 - w1) + a[1] * (w0 - w2) + a[2] * (w0 - w3) + a[3] * (w0 - w4) + a[4] * (w0 - w5) + a[5] * (w0 - w6);
    a = R.abc[1];
    sbe1 = a[0] * (w1 - w0) + a[1] * (w1 - w2) + a[2] * (w1 - w3) + a[3] * (w1 - w4) + a[4] * (w1 - w5) + a[5] * (w1 - w6);
    a = R.abc[2];
    sbe2 = a[0] * (w2 - w0) + a[1] * (w2 - w1) + a[2] * (w2 - w3) + a[3] * (w2 - w4) + a[4] * (w2 - w5) + a[5] * (w2 - w6);
  }
  double f2 = sbs0, f1 = sbs1 - fac[1 * 5 + 1] * f2;
  w[0] = f2;
  w[1] = f1;
  {
    const double v = sbs2 - fac[2 * 5 + 0] * f2 - fac[2 * 5 + 1] * f1;
    w[2] = v;
    f2 = f1; f1 = v;
  }
  double a0 = p[0], a1 = p[1], a2 = p[2], a3 = p[3], a4 = p[4], a5 = p[5];
  for (int i = 3; i <= L - 4; i++) {
    const double a6 = p[i + 3];
    const double sb = kAa * (a4 - a2) + kAb * (a5 - a1) + kAc * (a6 - a0);
    const double v = sb - fac[i * 5 + 0] * f2 - fac[i * 5 + 1] * f1;
    w[i] = v;
    f2 = f1; f1 = v;
    a0 = a1; a1 = a2; a2 = a3; a3 = a4; a4 = a5; a5 = a6;
  }
  const double sbe[3] = {sbe2, sbe1, sbe0};
  for (int r = 0; r < 3; r++) {
    const int i = L - 3 + r;
    const double v = sbe[r] - fac[i * 5 + 0] * f2 - fac[i * 5 + 1] * f1;
    if (r < 2) w[i] = v;
    f2 = f1; f1 = v;
  }
  double b0 = fac[(L - 1) * 5 + 2] * f1;
  double b1 = fac[(L - 2) * 5 + 2] * f2 - fac[(L - 2) * 5 + 3] * b0;
  o[L - 1] = b0;
  o[L - 2] = b1;
  for (int i = L - 3; i >= 0; i--) {
    const double v = fac[i * 5 + 2] * w[i] - fac[i * 5 + 3] * b1 - fac[i * 5 + 4] * b0;
    o[i] = v;
    b0 = b1; b1 = v;
  }
}

std::mutex g_mu;
// per device: the scratch array's device address, the context it was looked up in, and the line length whose
// LU factors the array holds (-1: none)
void *g_ptr[64] = {nullptr};
void *g_ctx[64] = {nullptr};
int g_len[64];
bool g_len_init = false;

// cuCtxGetCurrent from the driver, fetched through the runtime (no link-time dependency on libcuda): a device
// reset or a new primary context reloads the module, and the array may then sit at another address
using CtxGetCurrent = int (*)(void **);
CtxGetCurrent ctx_get_current() {
  static CtxGetCurrent fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return (CtxGetCurrent) nullptr;
    return (CtxGetCurrent)p;
  }();
  return fn;
}
void *current_ctx() {
  void *c = nullptr;
  if (CtxGetCurrent f = ctx_get_current()) {
    if (f(&c) != 0) c = nullptr;
  }
  return c;
}

Rows make_rows() {
  // interior and one-sided boundary coefficients (src/MainVar3D.f90:34-68,
  // src/Main3D.f90:71-73, 295-297)
  Rows R{};
  const double r0[6] = {-3.456878182643609, 5.839043358834730, 1.015886726041007, -0.2246526470654333,
                        0.08564940889936562, -0.01836710059356763};
  const double r1[6] = {-0.3177447290722621, -0.02807631929593225, 1.593461635747659, 0.2533027046976367,
                        -0.03619652460174756, 0.004080281419108407};
  const double r2[6] = {-0.1219006056449124, -0.6301651351188667, 0.6521195063966084, 0.3938843551210350,
                        0.01904944407973912, -0.001027260523947668};
  for (int q = 0; q < 6; q++) { R.abc[0][q] = r0[q]; R.abc[1][q] = r1[q]; R.abc[2][q] = r2[q]; }
  const double b[3][5] = {{0, 0, 1, 5.912678614078549, 3.775623951744012},
                          {0, 0.08360703307833438, 1, 2.058102869495757, 0.9704052014790193},
                          {0.03250008295108466, 0.3998040493524358, 1, 0.7719261277615860, 0.1626635931256900}};
  for (int r = 0; r < 3; r++)
    for (int q = 0; q < 5; q++) R.albe[r][q] = b[r][q];
  return R;
}

}  // namespace

void ati_set_thread_error(const char *msg);  // ati_api.cu

extern "C" int ati_deriv_lines_noalloc(const double *in, double *out, int64_t nlines, int32_t len, void *stream) {
  if (!in || !out || nlines < 0) {
    ati_set_thread_error("ati_deriv_lines_noalloc: null pointer or negative line count");
    return ATI_EINVAL;
  }
  if (len < 7 || len > kMaxLen) {
    ati_set_thread_error("ati_deriv_lines_noalloc: line length must be 7..ATI_NOALLOC_MAX_LEN (4096)");
    return ATI_EINVAL;
  }
  if (nlines > kMaxPoints / len) {
    ati_set_thread_error("ati_deriv_lines_noalloc: nlines*len exceeds ATI_NOALLOC_MAX_POINTS (2,000,000)");
    return ATI_EINVAL;
  }
  if (nlines == 0) return ATI_OK;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    ati_set_thread_error("ati_deriv_lines_noalloc: no current CUDA device");
    return ATI_ECUDA;
  }
  // an error left pending by earlier, unrelated work is reported as such and left in place
  if (cudaError_t pe = cudaPeekAtLastError(); pe != cudaSuccess) {
    ati_set_thread_error((std::string("ati_deriv_lines_noalloc: a CUDA error from earlier work is pending "
                                      "(not cleared, nothing launched): ") + cudaGetErrorString(pe)).c_str());
    return ATI_ECUDA;
  }
  void *base = nullptr;
  bool refactor = false;
  {
    // set-up, once per device and context: look up the device address of the scratch array with that device
    // current (in host code the symbol itself is only a host-side stand-in, not a device address)
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_len_init) {
      for (int q = 0; q < 64; q++) g_len[q] = -1;
      g_len_init = true;
    }
    void *ctx = current_ctx();
    if (!g_ptr[dev] || !ctx || ctx != g_ctx[dev]) {
      void *p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) {
        ati_set_thread_error((std::string("ati_deriv_lines_noalloc: cudaGetSymbolAddress of the scratch array "
                                          "failed: ") + cudaGetErrorString(e)).c_str());
        return ATI_ECUDA;
      }
      if (p != g_ptr[dev]) g_len[dev] = -1;  // a new array: no factors yet
      g_ptr[dev] = p;
      g_ctx[dev] = current_ctx();
    }
    base = g_ptr[dev];
    refactor = g_len[dev] != len;
    g_len[dev] = len;
  }
  double *fac = (double *)base;
  double *fw = fac + 5 * (int64_t)kMaxLen;
  cudaStream_t st = (cudaStream_t)stream;
  const Rows R = make_rows();
  // the LU factors depend on the line length only: refactored when it changes (calls are ordered on the GPU, so
  // a call finds the factors of the previous call in the array)
  if (refactor) k_noalloc_factors<<<1, 1, 0, st>>>(fac, len, R);
  const int tpb = 128;
  k_noalloc_deriv<<<(unsigned)((nlines + tpb - 1) / tpb), tpb, 0, st>>>(in, out, nlines, len, fac, fw, R);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    std::lock_guard<std::mutex> lk(g_mu);
    g_len[dev] = -1;
    ati_set_thread_error(cudaGetErrorString(e));
    return ATI_ECUDA;
  }
  return ATI_OK;
}
