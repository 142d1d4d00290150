// ati_turb.cu — synthetic inflow turbulence for the sponge of the inflow zone.
//
// The reference has an inflow-eddy generator that is switched off
// (ltz = -1, src/SingleTurbulence3D.f90:260); its sponge (spongego,
// src/SingleTurbulence3D.f90:332-374) would drive the gust points towards an
// isentropic target built from a velocity v: rho_t = (1 - (gamma-1)/2 |v|^2)
// ^(1/(gamma-1)), momentum atz rho_t v, pressure rho_t^gamma / gamma.  Here v is
// a sum of Fourier modes of a von Karman spectrum (random-Fourier-mode
// synthesis), convected with the freestream, evaluated in FP32.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <vector>

#include "ati_turb.h"

namespace ati {

namespace {

// splitmix64 (Steele, Lea and Flood 2014): a 64-bit counter mixed by two
// xor-shift-multiply rounds; used here only to draw the mode parameters
struct SplitMix {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

}  // namespace

void build_modes(const ati_config_t &cfg, std::vector<float> &out) {
  out.clear();
  const int n = cfg.turb_modes;
  if (n <= 0 || cfg.turb_intensity <= 0.0) return;
  const double pi = std::acos(-1.0);
  const double uinf = std::sqrt(cfg.amach1 * cfg.amach1 + cfg.amach2 * cfg.amach2 + cfg.amach3 * cfg.amach3);
  const double urms = cfg.turb_intensity * uinf;  // per component
  const double L = cfg.turb_length > 0 ? cfg.turb_length : 0.1;
  const double ke = 0.747 / L;  // energy-spectrum peak of the von Karman form for integral length L
  const double kmin = 0.1 * ke, kmax = 20.0 * ke, lr = std::log(kmax / kmin);
  const double kz0 = 2.0 * pi / cfg.span;  // spanwise wavenumbers of a span-periodic field
  SplitMix rng{(uint64_t)(uint32_t)cfg.turb_seed * 0x2545F4914F6CDD1Dull + 1};
  std::vector<double> mk(3 * (size_t)n), ms(3 * (size_t)n), ma(n), mp(n);
  double e2 = 0.0;
  for (int m = 0; m < n; m++) {
    const double k = kmin * std::exp(lr * (m + 0.5) / n), dk = k * lr / n;
    const double r = k / ke;
    const double E = r * r * r * r / std::pow(1.0 + r * r, 17.0 / 6.0);
    const double ct = 1.0 - 2.0 * rng.uniform(), st = std::sqrt(std::fmax(0.0, 1.0 - ct * ct));
    const double ph = 2.0 * pi * rng.uniform(), al = 2.0 * pi * rng.uniform(), psi = 2.0 * pi * rng.uniform();
    double kv[3] = {k * st * std::cos(ph), k * st * std::sin(ph), k * ct};
    kv[2] = kz0 * std::nearbyint(kv[2] / kz0);  // keep the field periodic over the span
    const double kk = std::sqrt(kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2]);
    double kh[3] = {kv[0] / kk, kv[1] / kk, kv[2] / kk};
    // orthonormal pair normal to k: the polarisation s lies in that plane (divergence free)
    double e1[3];
    if (std::fabs(kh[2]) < 0.9) { e1[0] = -kh[1]; e1[1] = kh[0]; e1[2] = 0.0; }
    else { e1[0] = 0.0; e1[1] = -kh[2]; e1[2] = kh[1]; }
    const double n1 = std::sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
    for (double &v : e1) v /= n1;
    const double e2v[3] = {kh[1] * e1[2] - kh[2] * e1[1], kh[2] * e1[0] - kh[0] * e1[2], kh[0] * e1[1] - kh[1] * e1[0]};
    for (int q = 0; q < 3; q++) {
      mk[3 * m + q] = kv[q];
      ms[3 * m + q] = std::cos(al) * e1[q] + std::sin(al) * e2v[q];
    }
    ma[m] = std::sqrt(E * dk);
    mp[m] = psi;
    e2 += 2.0 * ma[m] * ma[m];
  }
  const double scale = std::sqrt(3.0 * urms * urms / e2);  // sum of 2 a^2 = 3 urms^2
  out.resize((size_t)8 * n);
  for (int m = 0; m < n; m++) {
    for (int q = 0; q < 3; q++) {
      out[8 * m + q] = (float)mk[3 * m + q];
      out[8 * m + 3 + q] = (float)ms[3 * m + q];
    }
    out[8 * m + 6] = (float)(ma[m] * scale);
    out[8 * m + 7] = (float)mp[m];
  }
}

namespace {

constexpr int GT = 256;  // gust points per CTA (the gust list is padded per case to this)
constexpr float TWO_PI_F = 6.28318530717958647692f;

// velocity of the modes [m0, m0 + nm) at (x, y, z): each CTA stages the modes
// in shared memory with their time phase folded into psi
__device__ __forceinline__ void accumulate(const float *sm, int nm, float x, float y, float z, float &vx, float &vy,
                                           float &vz) {
  for (int m = 0; m < nm; m++) {
    const float *md = sm + 8 * m;
    float ph = md[0] * x + md[1] * y + md[2] * z + md[7];
    ph = ph - TWO_PI_F * rintf(ph * (1.0f / TWO_PI_F));  // into [-pi, pi]
    const float c = 2.0f * md[6] * __cosf(ph);
    vx += c * md[3];
    vy += c * md[4];
    vz += c * md[5];
  }
}

// stage the modes [m0, m0 + nm) of one case: psi - (k . U_inf) t reduced mod 2 pi in FP64
__device__ __forceinline__ void stage_modes(float *sm, const float *modes, int m0, int nm, const double u[3], double t) {
  for (int q = threadIdx.x; q < nm; q += blockDim.x) {
    const float *md = modes + 8 * (m0 + q);
    for (int c = 0; c < 7; c++) sm[8 * q + c] = md[c];
    const double w = ((double)md[0] * u[0] + (double)md[1] * u[1] + (double)md[2] * u[2]) * t;
    const double r = w - 6.283185307179586 * floor(w / 6.283185307179586);
    sm[8 * q + 7] = (float)((double)md[7] - r);
  }
}

__global__ void __launch_bounds__(GT) k_gust_eval(const GustPt *pts, const TurbCase *tc, const float *modes,
                                                  const Scalars *scal, float *delta, double gam) {
  __shared__ float sm[8 * GT];
  const int64_t i = (int64_t)blockIdx.x * GT + threadIdx.x;
  const GustPt P = pts[i];
  const int cs = pts[(int64_t)blockIdx.x * GT].cs;  // one case per CTA (padded list)
  const TurbCase C = tc[cs];
  const double t = scal[cs].timo;
  float vx = 0.f, vy = 0.f, vz = 0.f;
  for (int m0 = 0; m0 < C.n; m0 += GT) {
    const int nm = min(GT, C.n - m0);
    __syncthreads();
    stage_modes(sm, modes + 8 * (int64_t)C.off, m0, nm, C.u, t);
    __syncthreads();
    accumulate(sm, nm, P.x, P.y, P.z, vx, vy, vz);
  }
  if (P.g < 0) return;
  // isentropic target of spongego (src/SingleTurbulence3D.f90:362-365)
  const float g = (float)gam, gm1 = g - 1.0f;
  const float rho = powf(1.0f - 0.5f * gm1 * (vx * vx + vy * vy + vz * vz), 1.0f / gm1);
  const float a = P.atz * rho;
  float *d = delta + 5 * i;
  d[0] = 1.0f - rho;                       // target rho 1 -> rho_t
  d[1] = -a * vx; d[2] = -a * vy; d[3] = -a * vz;  // target momentum 0 -> atz rho_t v
  d[4] = (1.0f / g) * (1.0f - powf(rho, g));       // target pressure 1/gamma -> rho_t^gamma / gamma
}

template <typename R>
__global__ void k_gust_apply(const GustPt *pts, int64_t npts, const float *delta, const double *asz, const double *bsz,
                             R *de, int64_t N) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npts) return;
  const int64_t g = pts[i].g;
  if (g < 0) return;
  const float *d = delta + 5 * i;
  const double as = asz[g], bs = bsz[g];
  de[g] = (R)((double)de[g] + as * d[0]);
  de[g + N] = (R)((double)de[g + N] + as * d[1]);
  de[g + 2 * N] = (R)((double)de[g + 2 * N] + as * d[2]);
  de[g + 3 * N] = (R)((double)de[g + 3 * N] + as * d[3]);
  de[g + 4 * N] = (R)((double)de[g + 4 * N] + bs * d[4]);
}

// The FP64 synthesis of the strict mode.  The mode sum and the target use explicitly rounded operations (no
// multiply-add contraction) in the order of the CPU restatement, so the two differ only through cos and pow.
__global__ void __launch_bounds__(GT) k_gust_eval64(const GustPt *pts, const GustPt64 *p64, const TurbCase *tc,
                                                    const float *modes, const Scalars *scal, double *delta,
                                                    double gam, double gamm1, double hamm1, double ham) {
  __shared__ double sm[8 * GT], sw[GT];
  const int64_t i = (int64_t)blockIdx.x * GT + threadIdx.x;
  const GustPt P = pts[i];
  const GustPt64 Q = p64[i];
  const int cs = pts[(int64_t)blockIdx.x * GT].cs;
  const TurbCase C = tc[cs];
  const double t = scal[cs].timo;
  double vx = 0.0, vy = 0.0, vz = 0.0;
  for (int m0 = 0; m0 < C.n; m0 += GT) {
    const int nm = min(GT, C.n - m0);
    __syncthreads();
    for (int q = threadIdx.x; q < nm; q += blockDim.x) {
      // k, s, 2 a, psi of the mode, and its time phase (k . U_inf) t
      const float *md = modes + 8 * ((int64_t)C.off + m0 + q);
      double *d = sm + 8 * q;
      for (int c = 0; c < 8; c++) d[c] = (double)md[c];
      d[6] = __dmul_rn(2.0, d[6]);
      sw[q] = __dmul_rn(__dadd_rn(__dadd_rn(__dmul_rn(d[0], C.u[0]), __dmul_rn(d[1], C.u[1])), __dmul_rn(d[2], C.u[2])),
                        t);
    }
    __syncthreads();
    for (int m = 0; m < nm; m++) {
      const double *d = sm + 8 * m;
      const double ph = __dsub_rn(__dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(d[0], Q.x), __dmul_rn(d[1], Q.y)),
                                                      __dmul_rn(d[2], Q.z)), d[7]), sw[m]);
      const double c = __dmul_rn(d[6], cos(ph));
      vx = __dadd_rn(vx, __dmul_rn(c, d[3]));
      vy = __dadd_rn(vy, __dmul_rn(c, d[4]));
      vz = __dadd_rn(vz, __dmul_rn(c, d[5]));
    }
  }
  if (P.g < 0) return;
  // isentropic target of spongego (src/SingleTurbulence3D.f90:362-372), as changes of the rest targets
  const double s2 = __dadd_rn(__dadd_rn(__dmul_rn(vx, vx), __dmul_rn(vy, vy)), __dmul_rn(vz, vz));
  const double rho = pow(__dsub_rn(1.0, __dmul_rn(__dmul_rn(0.5, gamm1), s2)), hamm1);
  const double a = __dmul_rn(Q.atz, rho);
  double *dl = delta + 5 * i;
  dl[0] = __dsub_rn(1.0, rho);
  dl[1] = -__dmul_rn(a, vx); dl[2] = -__dmul_rn(a, vy); dl[3] = -__dmul_rn(a, vz);
  dl[4] = __dsub_rn(ham, __dmul_rn(ham, pow(rho, gam)));
}

__global__ void k_gust_apply64(const GustPt *pts, int64_t npts, const double *delta, const double *asz,
                               const double *bsz, double *de, int64_t N) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npts) return;
  const int64_t g = pts[i].g;
  if (g < 0) return;
  const double *d = delta + 5 * i;
  const double as = asz[g], bs = bsz[g];
  de[g] = __dadd_rn(de[g], __dmul_rn(as, d[0]));
  de[g + N] = __dadd_rn(de[g + N], __dmul_rn(as, d[1]));
  de[g + 2 * N] = __dadd_rn(de[g + 2 * N], __dmul_rn(as, d[2]));
  de[g + 3 * N] = __dadd_rn(de[g + 3 * N], __dmul_rn(as, d[3]));
  de[g + 4 * N] = __dadd_rn(de[g + 4 * N], __dmul_rn(bs, d[4]));
}

__global__ void __launch_bounds__(GT) k_turb_sample(const TurbCase *tc, int cs, const float *modes, double t,
                                                    int64_t n, const double *xyz, double *v) {
  __shared__ float sm[8 * GT];
  const int64_t i = (int64_t)blockIdx.x * GT + threadIdx.x;
  const TurbCase C = tc[cs];
  const float x = i < n ? (float)xyz[i] : 0.f, y = i < n ? (float)xyz[n + i] : 0.f, z = i < n ? (float)xyz[2 * n + i] : 0.f;
  float vx = 0.f, vy = 0.f, vz = 0.f;
  for (int m0 = 0; m0 < C.n; m0 += GT) {
    const int nm = min(GT, C.n - m0);
    __syncthreads();
    stage_modes(sm, modes + 8 * (int64_t)C.off, m0, nm, C.u, t);
    __syncthreads();
    accumulate(sm, nm, x, y, z, vx, vy, vz);
  }
  if (i < n) {
    v[i] = vx;
    v[n + i] = vy;
    v[2 * n + i] = vz;
  }
}

}  // namespace

void gust_eval(cudaStream_t st, const GustPt *pts, int64_t npts, const TurbCase *tc, const float *modes,
               const Scalars *scal, float *delta, double gam) {
  if (npts == 0) return;
  k_gust_eval<<<(unsigned)(npts / GT), GT, 0, st>>>(pts, tc, modes, scal, delta, gam);
}
void gust_apply_d(cudaStream_t st, const GustPt *pts, int64_t npts, const float *delta, const double *asz,
                  const double *bsz, double *de, int64_t N) {
  if (npts == 0) return;
  k_gust_apply<double><<<(unsigned)((npts + 255) / 256), 256, 0, st>>>(pts, npts, delta, asz, bsz, de, N);
}
void gust_apply_f(cudaStream_t st, const GustPt *pts, int64_t npts, const float *delta, const double *asz,
                  const double *bsz, float *de, int64_t N) {
  if (npts == 0) return;
  k_gust_apply<float><<<(unsigned)((npts + 255) / 256), 256, 0, st>>>(pts, npts, delta, asz, bsz, de, N);
}
void gust_eval64(cudaStream_t st, const GustPt *pts, const GustPt64 *p64, int64_t npts, const TurbCase *tc,
                 const float *modes, const Scalars *scal, double *delta, double gam, double gamm1, double hamm1,
                 double ham) {
  if (npts == 0) return;
  k_gust_eval64<<<(unsigned)(npts / GT), GT, 0, st>>>(pts, p64, tc, modes, scal, delta, gam, gamm1, hamm1, ham);
}
void gust_apply64(cudaStream_t st, const GustPt *pts, int64_t npts, const double *delta, const double *asz,
                  const double *bsz, double *de, int64_t N) {
  if (npts == 0) return;
  k_gust_apply64<<<(unsigned)((npts + 255) / 256), 256, 0, st>>>(pts, npts, delta, asz, bsz, de, N);
}
void turb_sample(cudaStream_t st, const TurbCase *tc, int cs, const float *modes, double t, int64_t n,
                 const double *xyz, double *v) {
  if (n == 0) return;
  k_turb_sample<<<(unsigned)((n + GT - 1) / GT), GT, 0, st>>>(tc, cs, modes, t, n, xyz, v);
}

}  // namespace ati
