// ati_kernels.cu — sm_103a kernels of the ATI3D per-RK-stage hot path (FP64).
//
// Each kernel restates one loop nest of the reference (cited per kernel) over
// all blocks of the case at once.  This file is compiled twice: into
// namespace ati::fast with FMA contraction (the fused time step) and into
// ati::strict with -fmad=false, where every operation rounds as the
// reference's Fortran expressions do (set-up and the granular calls, which
// then agree with the CPU restatement bit for bit).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "ati_kernels.h"

#ifndef ATI_KNS
#error "compile with -DATI_KNS=fast or -DATI_KNS=strict"
#endif

namespace ati {
namespace ATI_KNS {

__device__ __forceinline__ int64_t idx3(int lxi, int let, int i, int j, int k, int nn) {
  // src/Subroutineso.f90:364-375
  if (nn == 1) return ((int64_t)k * (let + 1) + j) * (lxi + 1) + i;
  if (nn == 2) return ((int64_t)j * (let + 1) + i) * (lxi + 1) + k;
  return ((int64_t)i * (let + 1) + k) * (lxi + 1) + j;
}

__device__ __forceinline__ void ijk_of(const BlockDev &B, int nn, int &i1, int &i2, int &i3) {
  // src/Main3D.f90:203-205
  if (nn == 1) { i1 = B.lxi; i2 = B.let; i3 = B.lze; }
  else if (nn == 2) { i1 = B.let; i2 = B.lze; i3 = B.lxi; }
  else { i1 = B.lze; i2 = B.lxi; i3 = B.let; }
}

// ---------------------------------------------------------------------------
// Compact derivative / filter line sweeps: deriv (src/Subroutines3D.f90:84-141)
// and filte (src/Subroutines3D.f90:145-206).
//
// One thread owns one line.  For eta and zeta lines consecutive threads own
// consecutive xi positions, so every load and store of a warp is one
// contiguous 256-byte row; xi lines are contiguous per thread and are served
// from L1.  The six boundary right-hand sides are built first from the
// original values, so the sweep may run in place (deriv(1,1,m), filte).
// Forward-elimination values go to the scratch plane fw at the same point
// index; the back substitution reads them back.
// ---------------------------------------------------------------------------
template <int NN>
__device__ __forceinline__ bool line_geom(const BlockDev &B, int t, int64_t &base, int64_t &stride, int &jk, int &L) {
  const int nx = B.lxi + 1, ny = B.let + 1, nz = B.lze + 1;
  if (NN == 1) {
    if (t >= ny * nz) return false;
    base = B.off + (int64_t)t * nx; stride = 1; jk = t; L = nx;
  } else if (NN == 2) {
    if (t >= nx * nz) return false;
    const int xi = t % nx, ze = t / nx;
    base = B.off + (int64_t)ze * nx * ny + xi; stride = nx; jk = xi * nz + ze; L = ny;
  } else {
    if (t >= nx * ny) return false;
    base = B.off + t; stride = (int64_t)nx * ny; jk = t; L = nz;
  }
  return true;
}

template <int NN, bool FILT>
__global__ void __launch_bounds__(128) k_sweep(Ctx c, const double *in, double *out, int m) {
  const BlockDev &B = c.blk[blockIdx.y];
  int64_t base, stride;
  int jk, L;
  if (!line_geom<NN>(B, blockIdx.x * blockDim.x + threadIdx.x, base, stride, jk, L)) return;
  const Scheme &S = *c.sc;
  const int ns = B.ndf[0][NN], ne = B.ndf[1][NN];
  const int64_t nbs = B.nbsize[NN];
  const double *recv = c.recv + B.face_off[NN] * 6;
  const double *fac = (FILT ? c.facf : c.facd) + B.fac_off[NN] * 5;
  const double *pin = in + base;
  double *fw = c.fw + base;
#define LD(i) pin[(int64_t)(i) * stride]
  double sbs0, sbs1, sbs2, sbe0, sbe1, sbe2;
  if (!FILT) {
    const double aa = S.aa, ab = S.ab, ac = S.ac;
    if (ns == 0) {
      const double w0 = LD(0), w1 = LD(1), w2 = LD(2), w3 = LD(3), w4 = LD(4), w5 = LD(5), w6 = LD(6);
      const double *a = S.abc[0];
      sbs0 = a[0] * (w1 - w0) + a[1] * (w2 - w0) + a[2] * (w3 - w0) + a[3] * (w4 - w0) + a[4] * (w5 - w0) + a[5] * (w6 - w0);
      a = S.abc[1];
      sbs1 = a[0] * (w0 - w1) + a[1] * (w2 - w1) + a[2] * (w3 - w1) + a[3] * (w4 - w1) + a[4] * (w5 - w1) + a[5] * (w6 - w1);
      a = S.abc[2];
      sbs2 = a[0] * (w0 - w2) + a[1] * (w1 - w2) + a[2] * (w3 - w2) + a[3] * (w4 - w2) + a[4] * (w5 - w2) + a[5] * (w6 - w2);
    } else {
      double s0 = 0, s1 = 0;
#pragma unroll
      for (int q = 0; q <= LMD; q++) {
        const double v = LD(q);
        s0 += S.pbci[0][0][q] * v;
        s1 += S.pbci[0][1][q] * v;
      }
      sbs0 = s0 + recv[jk + nbs * 0];
      sbs1 = s1 + recv[jk + nbs * 1];
      sbs2 = aa * (LD(3) - LD(1)) + ab * (LD(4) - LD(0)) + ac * (LD(5) - recv[jk + nbs * 2]);
    }
    if (ne == 0) {
      const double w0 = LD(L - 1), w1 = LD(L - 2), w2 = LD(L - 3), w3 = LD(L - 4), w4 = LD(L - 5), w5 = LD(L - 6),
                   w6 = LD(L - 7);
      const double *a = S.abc[0];
      sbe0 = a[0] * (w0 - w1) + a[1] * (w0 - w2) + a[2] * (w0 - w3) + a[3] * (w0 - w4) + a[4] * (w0 - w5) + a[5] * (w0 - w6);
      a = S.abc[1];
      sbe1 = a[0] * (w1 - w0) + a[1] * (w1 - w2) + a[2] * (w1 - w3) + a[3] * (w1 - w4) + a[4] * (w1 - w5) + a[5] * (w1 - w6);
      a = S.abc[2];
      sbe2 = a[0] * (w2 - w0) + a[1] * (w2 - w1) + a[2] * (w2 - w3) + a[3] * (w2 - w4) + a[4] * (w2 - w5) + a[5] * (w2 - w6);
    } else {
      double s0 = 0, s1 = 0;
#pragma unroll
      for (int q = 0; q <= LMD; q++) {
        const double v = LD(L - 1 - q);
        s0 += S.pbci[0][0][q] * v;
        s1 += S.pbci[0][1][q] * v;
      }
      sbe0 = -s0 - recv[jk + nbs * 3];
      sbe1 = -s1 - recv[jk + nbs * 4];
      sbe2 = aa * (LD(L - 2) - LD(L - 4)) + ab * (LD(L - 1) - LD(L - 5)) + ac * (recv[jk + nbs * 5] - LD(L - 6));
    }
  } else {
    const double fa = S.fa, fb = S.fb, fc = S.fc;
    if (ns == 0) {
      const double w0 = LD(0), w1 = LD(1), w2 = LD(2), w3 = LD(3), w4 = LD(4), w5 = LD(5);
      const double ra0 = 2.0 * w0, ra1 = 2.0 * w1, ra2 = 2.0 * w2;
      const double res = S.fex[1] * (w1 - w0) + S.fex[2] * (w2 - w0) + S.fex[3] * (w3 - w0);
      const double rv1 = w0 - res * S.ffx[1], rv2 = w0 - res * S.ffx[2], rv3 = w0 - res * S.ffx[3];
      sbs0 = S.fam[0] * (rv1 + w1 - ra0) + S.fbm[0] * (rv2 + w2 - ra0) + S.fcm[0] * (rv3 + w3 - ra0);
      sbs1 = S.fam[1] * (w0 + w2 - ra1) + S.fbm[1] * (rv1 + w3 - ra1) + S.fcm[1] * (rv2 + w4 - ra1);
      sbs2 = S.fam[2] * (w1 + w3 - ra2) + S.fbm[2] * (w0 + w4 - ra2) + S.fcm[2] * (rv1 + w5 - ra2);
    } else {
      double s0 = 0, s1 = 0;
#pragma unroll
      for (int q = 0; q <= LMF; q++) {
        const double v = LD(q);
        s0 += S.pbci[1][0][q] * v;
        s1 += S.pbci[1][1][q] * v;
      }
      const double ra2 = 2.0 * LD(2);
      sbs0 = s0 + recv[jk + nbs * 0];
      sbs1 = s1 + recv[jk + nbs * 1];
      sbs2 = fa * (LD(1) + LD(3) - ra2) + fb * (LD(0) + LD(4) - ra2) + fc * (recv[jk + nbs * 2] + LD(5) - ra2);
    }
    if (ne == 0) {
      const double w0 = LD(L - 1), w1 = LD(L - 2), w2 = LD(L - 3), w3 = LD(L - 4), w4 = LD(L - 5), w5 = LD(L - 6);
      const double ra0 = 2.0 * w0, ra1 = 2.0 * w1, ra2 = 2.0 * w2;
      const double res = S.fex[1] * (w0 - w1) + S.fex[2] * (w0 - w2) + S.fex[3] * (w0 - w3);
      const double rv1 = w0 + res * S.ffx[1], rv2 = w0 + res * S.ffx[2], rv3 = w0 + res * S.ffx[3];
      sbe0 = S.fam[0] * (w1 + rv1 - ra0) + S.fbm[0] * (w2 + rv2 - ra0) + S.fcm[0] * (w3 + rv3 - ra0);
      sbe1 = S.fam[1] * (w2 + w0 - ra1) + S.fbm[1] * (w3 + rv1 - ra1) + S.fcm[1] * (w4 + rv2 - ra1);
      sbe2 = S.fam[2] * (w3 + w1 - ra2) + S.fbm[2] * (w4 + w0 - ra2) + S.fcm[2] * (w5 + rv1 - ra2);
    } else {
      double s0 = 0, s1 = 0;
#pragma unroll
      for (int q = 0; q <= LMF; q++) {
        const double v = LD(L - 1 - q);
        s0 += S.pbci[1][0][q] * v;
        s1 += S.pbci[1][1][q] * v;
      }
      const double ra2 = 2.0 * LD(L - 3);
      sbe0 = s0 + recv[jk + nbs * 3];
      sbe1 = s1 + recv[jk + nbs * 4];
      sbe2 = fa * (LD(L - 4) + LD(L - 2) - ra2) + fb * (LD(L - 5) + LD(L - 1) - ra2) +
             fc * (LD(L - 6) + recv[jk + nbs * 5] - ra2);
    }
  }
  // forward elimination (src/Subroutines3D.f90:124-128 / 190-194)
  double f2 = sbs0;
  double f1 = sbs1 - fac[1 * 5 + 1] * f2;
  fw[0] = f2;
  fw[stride] = f1;
  {
    const double v = sbs2 - fac[2 * 5 + 0] * f2 - fac[2 * 5 + 1] * f1;
    fw[2 * stride] = v;
    f2 = f1; f1 = v;
  }
  {
    double a0 = LD(0), a1 = LD(1), a2 = LD(2), a3 = LD(3), a4 = LD(4), a5 = LD(5);
    if (!FILT) {
      const double aa = S.aa, ab = S.ab, ac = S.ac;
      for (int i = 3; i <= L - 4; i++) {
        const double a6 = LD(i + 3);
        const double sb = aa * (a4 - a2) + ab * (a5 - a1) + ac * (a6 - a0);
        const double v = sb - fac[i * 5 + 0] * f2 - fac[i * 5 + 1] * f1;
        fw[(int64_t)i * stride] = v;
        f2 = f1; f1 = v;
        a0 = a1; a1 = a2; a2 = a3; a3 = a4; a4 = a5; a5 = a6;
      }
    } else {
      const double fa = S.fa, fb = S.fb, fc = S.fc;
      for (int i = 3; i <= L - 4; i++) {
        const double a6 = LD(i + 3);
        const double res = 2.0 * a3;
        const double sb = fa * (a2 + a4 - res) + fb * (a1 + a5 - res) + fc * (a0 + a6 - res);
        const double v = sb - fac[i * 5 + 0] * f2 - fac[i * 5 + 1] * f1;
        fw[(int64_t)i * stride] = v;
        f2 = f1; f1 = v;
        a0 = a1; a1 = a2; a2 = a3; a3 = a4; a4 = a5; a5 = a6;
      }
    }
  }
  {
    int i = L - 3;
    double v = sbe2 - fac[i * 5 + 0] * f2 - fac[i * 5 + 1] * f1;
    fw[(int64_t)i * stride] = v;
    f2 = f1; f1 = v;
    i = L - 2;
    v = sbe1 - fac[i * 5 + 0] * f2 - fac[i * 5 + 1] * f1;
    fw[(int64_t)i * stride] = v;
    f2 = f1; f1 = v;
    i = L - 1;
    v = sbe0 - fac[i * 5 + 0] * f2 - fac[i * 5 + 1] * f1;
    f2 = f1; f1 = v;  // f1 = fw(L-1), f2 = fw(L-2)
  }
  // back substitution (src/Subroutines3D.f90:129-136 / 195-202)
  double *po = out + base;
  double b0 = fac[(L - 1) * 5 + 2] * f1;
  double b1 = fac[(L - 2) * 5 + 2] * f2 - fac[(L - 2) * 5 + 3] * b0;
  const double last = b0;
  if (FILT) {
    po[(int64_t)(L - 1) * stride] = LD(L - 1) + b0;
    po[(int64_t)(L - 2) * stride] = LD(L - 2) + b1;
  } else {
    po[(int64_t)(L - 1) * stride] = b0;
    po[(int64_t)(L - 2) * stride] = b1;
  }
  for (int i = L - 3; i >= 0; i--) {
    const double v = fac[i * 5 + 2] * fw[(int64_t)i * stride] - fac[i * 5 + 3] * b1 - fac[i * 5 + 4] * b0;
    if (FILT) po[(int64_t)i * stride] = LD(i) + v;
    else po[(int64_t)i * stride] = v;
    b0 = b1; b1 = v;
  }
  if (!FILT) {
    double *drva = c.drva + B.face_off[NN] * 10;
    drva[jk + nbs * ((m - 1) + 5 * 0)] = b1;  // sb(is)
    drva[jk + nbs * ((m - 1) + 5 * 1)] = last;  // sb(ie)
  }
#undef LD
}

// ---------------------------------------------------------------------------
// mpigo (src/Subroutines3D.f90:16-80): closure values of every face with
// ndf = 1.  The thread of face (A, nn, ip), line jk, computes what the
// neighbour B sends from its face 1-ip (the reference's tag pairing) and
// writes it straight into A's recv buffer; with n45 = 1 it adds A's own
// boundary value times pbcot (periodic coordinate re-basing).
// ---------------------------------------------------------------------------
__global__ void k_mpigo(Ctx c, const FaceTask *tasks, int nt, int n45, const double *src1, const double *src2,
                        const double *src3) {
  const FaceTask T = tasks[blockIdx.y];
  const int jk = blockIdx.x * blockDim.x + threadIdx.x;
  if (jk >= T.nline) return;
  const Scheme &S = *c.sc;
  const BlockDev &A = c.blk[T.b];
  const BlockDev &Bn = c.blk[T.nb_b];
  const int nn = T.nn, ip = T.ip, ipp = 1 - ip;
  const double *src = nn == 1 ? src1 : (nn == 2 ? src2 : src3);
  int a1, a2, a3, b1, b2, b3;
  ijk_of(A, nn, a1, a2, a3);
  ijk_of(Bn, nn, b1, b2, b3);
  const int j = jk % (a2 + 1), k = jk / (a2 + 1);
  const int bcB = Bn.nbc[ipp][nn];
  const int ii = bcB == 40 ? 0 : 1;
  const double ra0 = bcB == 45 ? (double)n45 : 0.0;
  const int isB = ipp * b1, ieB = 1 - 2 * ipp;
  const int mp = nt == 0 ? LMD : LMF;
  const double res = ra0 * src[Bn.off + idx3(Bn.lxi, Bn.let, isB, j, k, nn)];
  double s0 = 0, s1 = 0, sap0 = 0;
  for (int i = 0; i <= mp; i++) {
    const double v = src[Bn.off + idx3(Bn.lxi, Bn.let, isB + ieB * (i + ii), j, k, nn)];
    if (i == 0) sap0 = v;
    s0 += S.pbco[nt][0][i] * v;
    s1 += S.pbco[nt][1][i] * v;
  }
  double r0 = s0 - res * S.pbcot[nt][0];
  double r1 = s1 - res * S.pbcot[nt][1];
  double r2 = sap0 - res;
  if (n45 == 1 && A.nbc[ip][nn] == 45) {
    const double v = src[A.off + idx3(A.lxi, A.let, ip * a1, j, k, nn)];
    r0 = r0 + v * S.pbcot[nt][0];
    r1 = r1 + v * S.pbcot[nt][1];
    r2 = r2 + v;
  }
  const int64_t nbs = A.nbsize[nn];
  double *recv = c.recv + A.face_off[nn] * 6;
  recv[jk + nbs * (0 + 3 * ip)] = r0;
  recv[jk + nbs * (1 + 3 * ip)] = r1;
  recv[jk + nbs * (2 + 3 * ip)] = r2;
}

// ---------------------------------------------------------------------------
// Pointwise stage kernels (grid-stride over all points of all blocks).
// ---------------------------------------------------------------------------
#define GRID_STRIDE(g, N) for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < (N); g += (int64_t)gridDim.x * blockDim.x)

// primitives, pressure, temperature, Sutherland viscosity (src/Main3D.f90:576-583);
// de(:,1) holds mu afterwards when viscous (src/Main3D.f90:627).
__global__ void k_prim(Ctx c) {
  const Scheme &S = *c.sc;
  const int64_t N = c.N;
  int bad = 0;
  GRID_STRIDE(g, N) {
    const double q1 = c.qa[g], q2 = c.qa[g + N], q3 = c.qa[g + 2 * N], q4 = c.qa[g + 3 * N], q5 = c.qa[g + 4 * N];
    const double d1 = 1.0 / q1, d2 = q2 * d1, d3 = q3 * d1, d4 = q4 * d1;
    const double pp = S.gamm1 * (q5 - 0.5 * (q2 * d2 + q3 * d3 + q4 * d4));
    const double d5 = S.gam * pp * d1;
    // T^1.5 as T*sqrt(T): same value as pow(T,1.5) to ~1 ulp, far fewer FP64 instructions
    const double mu = S.srefp1dre * (d5 * sqrt(d5)) / (d5 + S.srefoo);
    c.de[g] = S.nviscous == 1 ? mu : d1;
    c.de[g + N] = d2; c.de[g + 2 * N] = d3; c.de[g + 3 * N] = d4; c.de[g + 4 * N] = d5;
    c.p[g] = pp;
    c.ss[g] = mu;
    if (!(q1 > 0.0) || !(pp > 0.0) || !(fabs(q5) < 1e300)) bad = 1;
  }
  if (bad) atomicOr(&c.scal->flag, 1);
}

__device__ __forceinline__ void atomic_max_pos(unsigned long long *a, double v) {
  atomicMax(a, (unsigned long long)__double_as_longlong(v));
}

// CFL spectral radii, max over all points (src/Main3D.f90:590-602)
__global__ void k_cfl(Ctx c) {
  const int64_t N = c.N;
  const double u1 = c.scal->umf[1], u2 = c.scal->umf[2], u3 = c.scal->umf[3];
  double m1 = 0.0, m2 = 0.0;
  GRID_STRIDE(g, N) {
    const double x1 = c.xim[g], x2 = c.xim[g + N], x3 = c.xim[g + 2 * N];
    const double e1 = c.etm[g], e2 = c.etm[g + N], e3 = c.etm[g + 2 * N];
    const double z1 = c.zem[g], z2 = c.zem[g + N], z3 = c.zem[g + 2 * N];
    const double d2 = c.de[g + N] + u1, d3 = c.de[g + 2 * N] + u2, d4 = c.de[g + 3 * N] + u3;
    const double r1 = x1 * x1 + x2 * x2 + x3 * x3 + e1 * e1 + e2 * e2 + e3 * e3 + z1 * z1 + z2 * z2 + z3 * z3;
    const double r2 = fabs(x1 * d2 + x2 * d3 + x3 * d4) + fabs(e1 * d2 + e2 * d3 + e3 * d4) + fabs(z1 * d2 + z2 * d3 + z3 * d4);
    const double s2 = fabs(c.yaco[g]);
    const double v1 = (sqrt(c.de[g + 4 * N] * r1) + r2) * s2;
    const double d1 = 1.0 / c.qa[g];
    const double v2 = d1 * c.ss[g] * r1 * s2 * s2;
    m1 = fmax(m1, v1);
    m2 = fmax(m2, v2);
    if (v1 != v1 || v2 != v2) atomicOr(&c.scal->flag, 4);
  }
  for (int o = 16; o > 0; o >>= 1) {
    m1 = fmax(m1, __shfl_xor_sync(0xffffffffu, m1, o));
    m2 = fmax(m2, __shfl_xor_sync(0xffffffffu, m2, o));
  }
  __shared__ double s1[32], s2v[32];
  const int w = threadIdx.x >> 5, ln = threadIdx.x & 31;
  if (ln == 0) { s1[w] = m1; s2v[w] = m2; }
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    m1 = ln < nw ? s1[ln] : 0.0;
    m2 = ln < nw ? s2v[ln] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      m1 = fmax(m1, __shfl_xor_sync(0xffffffffu, m1, o));
      m2 = fmax(m2, __shfl_xor_sync(0xffffffffu, m2, o));
    }
    if (ln == 0) {
      atomic_max_pos(&c.scal->cflmax[0], m1);
      atomic_max_pos(&c.scal->cflmax[1], m2);
    }
  }
}

// physical gradients of one primitive (src/Main3D.f90:631-651):
// o1 = xim(:,1)*rr1 + etm(:,1)*rr2 + zem(:,1)*rr3, o2 with component 2, o3 with 3
__global__ void k_grad(Ctx c, double *o1, double *o2, double *o3) {
  const int64_t N = c.N;
  GRID_STRIDE(g, N) {
    const double r1 = c.rr[g], r2 = c.rr[g + N], r3 = c.rr[g + 2 * N];
    o1[g] = c.xim[g] * r1 + c.etm[g] * r2 + c.zem[g] * r3;
    o2[g] = c.xim[g + N] * r1 + c.etm[g + N] * r2 + c.zem[g + N] * r3;
    o3[g] = c.xim[g + 2 * N] * r1 + c.etm[g + 2 * N] * r2 + c.zem[g + 2 * N] * r3;
  }
}

// stresses and heat fluxes (src/Main3D.f90:653-692)
__global__ void k_stress(Ctx c) {
  const Scheme &S = *c.sc;
  const int64_t N = c.N;
  double *t = c.tau;
  GRID_STRIDE(g, N) {
    const double yac = c.yaco[g];
    double r1 = c.de[g] * yac;
    double r2 = S.gamm1prndtli * r1, r3 = 0.0, d5;
    double txx = t[g], tyy = t[g + N], tzz = t[g + 2 * N];
    const double txy = t[g + 3 * N], tyz = t[g + 4 * N], tzx = t[g + 5 * N];
    const double hxx = t[g + 6 * N], hyy = t[g + 7 * N], hzz = t[g + 8 * N];
    if (S.les == 1) {
      const double d1 = txx * txx + tyy * tyy + tzz * tzz + (hzz + txy) * (hzz + txy) + (hyy + tzx) * (hyy + tzx) +
                        (hxx + tyz) * (hxx + tyz);
      const double varr = pow(-1.0 / yac, 1.5);
      const double q1 = c.qa[g];
      r3 = q1 * (S.smago1 * S.smago1) * varr * sqrt(2.0 * d1);
      r1 = r1 + r3 * yac;
      r2 = r2 + S.tgamm1prndtli * r3 * yac;
      r3 = S.two_three * (q1 * S.smago2 * varr * d1);
      d5 = S.two_three * (txx + tyy + tzz);
      txx = r1 * (2.0 * txx - d5) - r3;
      tyy = r1 * (2.0 * tyy - d5) - r3;
      tzz = r1 * (2.0 * tzz - d5) - r3;
    } else {
      d5 = S.two_three * (txx + tyy + tzz);
      txx = r1 * (2.0 * txx - d5);
      tyy = r1 * (2.0 * tyy - d5);
      tzz = r1 * (2.0 * tzz - d5);
    }
    const double ntxy = r1 * (txy + hzz), ntyz = r1 * (tyz + hxx), ntzx = r1 * (tzx + hyy);
    const double d2 = c.de[g + N], d3 = c.de[g + 2 * N], d4 = c.de[g + 3 * N];
    t[g] = txx; t[g + N] = tyy; t[g + 2 * N] = tzz;
    t[g + 3 * N] = ntxy; t[g + 4 * N] = ntyz; t[g + 5 * N] = ntzx;
    t[g + 6 * N] = r2 * c.ss[g] + d2 * txx + d3 * ntxy + d4 * ntzx;
    t[g + 7 * N] = r2 * c.ss[g + N] + d2 * ntxy + d3 * tyy + d4 * ntyz;
    t[g + 8 * N] = r2 * c.ss[g + 2 * N] + d2 * ntzx + d3 * ntyz + d4 * tzz;
  }
}

// contravariant velocities (src/Main3D.f90:710-715)
__global__ void k_fluxprep(Ctx c) {
  const int64_t N = c.N;
  const double u1 = c.scal->umf[1], u2 = c.scal->umf[2], u3 = c.scal->umf[3];
  GRID_STRIDE(g, N) {
    const double r1 = c.de[g + N] + u1, r2 = c.de[g + 2 * N] + u2, r3 = c.de[g + 3 * N] + u3;
    c.ss[g] = c.xim[g] * r1 + c.xim[g + N] * r2 + c.xim[g + 2 * N] * r3;
    c.ss[g + N] = c.etm[g] * r1 + c.etm[g + N] * r2 + c.etm[g + 2 * N] * r3;
    c.ss[g + 2 * N] = c.zem[g] * r1 + c.zem[g + N] * r2 + c.zem[g + 2 * N] * r3;
  }
}

// flux components of variable m in the three directions (src/Main3D.f90:718-766)
__global__ void k_flux(Ctx c, int m) {
  const Scheme &S = *c.sc;
  const int64_t N = c.N;
  const double u1 = c.scal->umf[1], u2 = c.scal->umf[2], u3 = c.scal->umf[3];
  const bool visc = S.nviscous == 1;
  const double *t = c.tau;
  GRID_STRIDE(g, N) {
    const double s1 = c.ss[g], s2 = c.ss[g + N], s3 = c.ss[g + 2 * N];
    double r1, r2, r3;
    if (m == 1) {
      const double q = c.qa[g];
      r1 = q * s1; r2 = q * s2; r3 = q * s3;
    } else if (m <= 4) {
      const double q = c.qa[g + (m - 1) * N], pp = c.p[g];
      r1 = q * s1 + c.xim[g + (m - 2) * N] * pp;
      r2 = q * s2 + c.etm[g + (m - 2) * N] * pp;
      r3 = q * s3 + c.zem[g + (m - 2) * N] * pp;
      if (visc) {
        double ta, tb, tc;
        if (m == 2) { ta = t[g]; tb = t[g + 3 * N]; tc = t[g + 5 * N]; }
        else if (m == 3) { ta = t[g + 3 * N]; tb = t[g + N]; tc = t[g + 4 * N]; }
        else { ta = t[g + 5 * N]; tb = t[g + 4 * N]; tc = t[g + 2 * N]; }
        r1 = r1 - c.xim[g] * ta - c.xim[g + N] * tb - c.xim[g + 2 * N] * tc;
        r2 = r2 - c.etm[g] * ta - c.etm[g + N] * tb - c.etm[g + 2 * N] * tc;
        r3 = r3 - c.zem[g] * ta - c.zem[g + N] * tb - c.zem[g + 2 * N] * tc;
      }
    } else {
      const double pp = c.p[g];
      const double d5 = c.qa[g + 4 * N] + pp;
      const double x1 = c.xim[g], x2 = c.xim[g + N], x3 = c.xim[g + 2 * N];
      const double e1 = c.etm[g], e2 = c.etm[g + N], e3 = c.etm[g + 2 * N];
      const double z1 = c.zem[g], z2 = c.zem[g + N], z3 = c.zem[g + 2 * N];
      r1 = d5 * s1 - pp * (u1 * x1 + u2 * x2 + u3 * x3);
      r2 = d5 * s2 - pp * (u1 * e1 + u2 * e2 + u3 * e3);
      r3 = d5 * s3 - pp * (u1 * z1 + u2 * z2 + u3 * z3);
      if (visc) {
        const double ha = t[g + 6 * N], hb = t[g + 7 * N], hc = t[g + 8 * N];
        r1 = r1 - x1 * ha - x2 * hb - x3 * hc;
        r2 = r2 - e1 * ha - e2 * hb - e3 * hc;
        r3 = r3 - z1 * ha - z2 * hb - z3 * hc;
      }
    }
    c.rr[g] = r1; c.rr[g + N] = r2; c.rr[g + 2 * N] = r3;
  }
}

// divergence de(:,m) = rr1+rr2+rr3 (src/Main3D.f90:722...) plus the sponge
// term of spongego (src/SingleTurbulence3D.f90:368-372) on sponge points
__global__ void k_div(Ctx c, int m) {
  const Scheme &S = *c.sc;
  const int64_t N = c.N;
  GRID_STRIDE(g, N) {
    double d = c.rr[g] + c.rr[g + N] + c.rr[g + 2 * N];
    const double as = c.asz[g], bs = c.bsz[g];
    if (as != 0.0 || bs != 0.0) {
      if (m == 1) d = d + as * (c.qa[g] - 1.0);
      else if (m <= 4) d = d + as * (c.qa[g + (m - 1) * N] - 0.0);
      else d = d + bs * (c.p[g] - S.ham * 1.0);
    }
    c.de[g + (m - 1) * N] = d;
  }
}

// RK update (src/Main3D.f90:876-881)
__global__ void k_rk(Ctx c) {
  const int64_t N = c.N;
  const double dtk = c.scal->dtk;
  GRID_STRIDE(g, N) {
    const double r1 = dtk * c.yaco[g];
#pragma unroll
    for (int q = 0; q < 5; q++) c.qa[g + q * N] = c.qo[g + q * N] - r1 * c.de[g + q * N];
  }
}

// ---------------------------------------------------------------------------
// characteristic boundary treatment: eleme, xtq2r, xtr2q
// (src/Subroutines3D.f90:235-324) and the GCBC/GCIC loops of
// src/Main3D.f90:780-869.
// ---------------------------------------------------------------------------
struct Elem {
  double rhoi, ao, aoi, ve[3], hv2, vn, vs;
};

__device__ __forceinline__ void eleme(const Scheme &S, const Ctx &c, int64_t g, const double cm[3], const double umf[4],
                                      Elem &e) {
  const int64_t N = c.N;
  e.rhoi = 1.0 / c.qa[g];
  e.ao = sqrt(S.gam * e.rhoi * c.p[g]);
  e.aoi = 1.0 / e.ao;
  e.ve[0] = e.rhoi * c.qa[g + N];
  e.ve[1] = e.rhoi * c.qa[g + 2 * N];
  e.ve[2] = e.rhoi * c.qa[g + 3 * N];
  e.hv2 = 0.5 * (e.ve[0] * e.ve[0] + e.ve[1] * e.ve[1] + e.ve[2] * e.ve[2]);
  e.vn = cm[0] * e.ve[0] + cm[1] * e.ve[1] + cm[2] * e.ve[2];
  e.vs = cm[0] * umf[1] + cm[1] * umf[2] + cm[2] * umf[3];
}

__device__ __forceinline__ void xtq2r(const Scheme &S, const Elem &e, const double cm[3], double xt[5][5]) {
  const double ho = S.gamm1 * e.aoi * e.aoi, bo = 1.0 - ho * e.hv2, co = e.aoi * e.vn;
  const double dm0 = e.aoi * cm[0], dm1 = e.aoi * cm[1], dm2 = e.aoi * cm[2];
  const double rv0 = ho * e.ve[0], rv1 = ho * e.ve[1], rv2 = ho * e.ve[2];
  const double *ve = e.ve;
  xt[0][0] = bo * cm[0] + dm1 * ve[2] - dm2 * ve[1];
  xt[0][1] = cm[0] * rv0;
  xt[0][2] = cm[0] * rv1 + dm2;
  xt[0][3] = cm[0] * rv2 - dm1;
  xt[0][4] = -ho * cm[0];
  xt[1][0] = bo * cm[1] + dm2 * ve[0] - dm0 * ve[2];
  xt[1][1] = cm[1] * rv0 - dm2;
  xt[1][2] = cm[1] * rv1;
  xt[1][3] = cm[1] * rv2 + dm0;
  xt[1][4] = -ho * cm[1];
  xt[2][0] = bo * cm[2] + dm0 * ve[1] - dm1 * ve[0];
  xt[2][1] = cm[2] * rv0 + dm1;
  xt[2][2] = cm[2] * rv1 - dm0;
  xt[2][3] = cm[2] * rv2;
  xt[2][4] = -ho * cm[2];
  xt[3][0] = 1.0 - bo - co;
  xt[3][1] = dm0 - rv0;
  xt[3][2] = dm1 - rv1;
  xt[3][3] = dm2 - rv2;
  xt[3][4] = ho;
  xt[4][0] = 1.0 - bo + co;
  xt[4][1] = -dm0 - rv0;
  xt[4][2] = -dm1 - rv1;
  xt[4][3] = -dm2 - rv2;
  xt[4][4] = ho;
}

__device__ __forceinline__ void xtr2q(const Scheme &S, const Elem &e, const double cm[3], double xt[5][5]) {
  const double bo = e.hv2 + S.hamm1 * e.ao * e.ao, co = e.ao * e.vn;
  const double dm0 = e.ao * cm[0], dm1 = e.ao * cm[1], dm2 = e.ao * cm[2];
  const double *ve = e.ve;
  xt[0][0] = cm[0]; xt[0][1] = cm[1]; xt[0][2] = cm[2]; xt[0][3] = 0.5; xt[0][4] = 0.5;
  xt[1][0] = cm[0] * ve[0];
  xt[1][1] = cm[1] * ve[0] - dm2;
  xt[1][2] = cm[2] * ve[0] + dm1;
  xt[1][3] = 0.5 * (ve[0] + dm0);
  xt[1][4] = xt[1][3] - dm0;
  xt[2][0] = cm[0] * ve[1] + dm2;
  xt[2][1] = cm[1] * ve[1];
  xt[2][2] = cm[2] * ve[1] - dm0;
  xt[2][3] = 0.5 * (ve[1] + dm1);
  xt[2][4] = xt[2][3] - dm1;
  xt[3][0] = cm[0] * ve[2] - dm1;
  xt[3][1] = cm[1] * ve[2] + dm0;
  xt[3][2] = cm[2] * ve[2];
  xt[3][3] = 0.5 * (ve[2] + dm2);
  xt[3][4] = xt[3][3] - dm2;
  xt[4][0] = e.hv2 * cm[0] + dm2 * ve[1] - dm1 * ve[2];
  xt[4][1] = e.hv2 * cm[1] + dm0 * ve[2] - dm2 * ve[0];
  xt[4][2] = e.hv2 * cm[2] + dm1 * ve[0] - dm0 * ve[1];
  xt[4][3] = 0.5 * (bo + co);
  xt[4][4] = xt[4][3] - co;
}

__device__ __forceinline__ void face_point(const BlockDev &B, int nn, int ip, int jk, int &i, int &j, int &k, int &i1) {
  int a1, a2, a3;
  ijk_of(B, nn, a1, a2, a3);
  j = jk % (a2 + 1);
  k = jk / (a2 + 1);
  i = ip * a1;
  i1 = a1;
}

// GCBC/GCIC preparation: drva = X * (J * (ra0*drva + ra1*de)) (src/Main3D.f90:780-795)
__global__ void k_gcbc_prep(Ctx c, const FaceTask *tasks) {
  const FaceTask T = tasks[blockIdx.y];
  const int jk = blockIdx.x * blockDim.x + threadIdx.x;
  if (jk >= T.nline) return;
  const Scheme &S = *c.sc;
  const BlockDev &B = c.blk[T.b];
  const int nn = T.nn, ip = T.ip, np = T.bc;
  int i, j, k, i1;
  face_point(B, nn, ip, jk, i, j, k, i1);
  const int64_t g = B.off + idx3(B.lxi, B.let, i, j, k, nn), N = c.N, nbs = T.nline;
  const double ra0 = (double)((20 - np) * (25 - np) * (30 - np) / 3000), ra1 = 1.0 - ra0;
  double *drva = c.drva + B.face_off[nn] * 10;
  const double *cmv = c.cm + B.face_off[nn] * 6;
  const double cm[3] = {cmv[jk + nbs * (0 + 3 * ip)], cmv[jk + nbs * (1 + 3 * ip)], cmv[jk + nbs * (2 + 3 * ip)]};
  double umf[4] = {0, c.scal->umf[1], c.scal->umf[2], c.scal->umf[3]};
  Elem e;
  eleme(S, c, g, cm, umf, e);
  double xt[5][5];
  xtq2r(S, e, cm, xt);
  double v[5];
  const double yac = c.yaco[g];
#pragma unroll
  for (int q = 0; q < 5; q++) v[q] = yac * (ra0 * drva[jk + nbs * (q + 5 * ip)] + ra1 * c.de[g + q * N]);
#pragma unroll
  for (int r = 0; r < 5; r++) {
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < 5; q++) s += xt[r][q] * v[q];
    drva[jk + nbs * (r + 5 * ip)] = s;
  }
}

// GCBC/GCIC application for the faces of one direction (src/Main3D.f90:817-869).
// Launched once per direction in the reference's order so that edge points
// touched by faces of two directions accumulate in the same order.
__global__ void k_gcbc_apply(Ctx c, const FaceTask *tasks) {
  const FaceTask T = tasks[blockIdx.y];
  const int jk = blockIdx.x * blockDim.x + threadIdx.x;
  if (jk >= T.nline) return;
  const Scheme &S = *c.sc;
  const BlockDev &B = c.blk[T.b];
  const int nn = T.nn, ip = T.ip, np = T.bc, iq = 1 - 2 * ip;
  const double ra0 = (double)iq;
  int i, j, k, i1;
  face_point(B, nn, ip, jk, i, j, k, i1);
  const int64_t g = B.off + idx3(B.lxi, B.let, i, j, k, nn), N = c.N, nbs = T.nline;
  const double *drva = c.drva + B.face_off[nn] * 10;
  const double *cmv = c.cm + B.face_off[nn] * 6;
  const double cm[3] = {cmv[jk + nbs * (0 + 3 * ip)], cmv[jk + nbs * (1 + 3 * ip)], cmv[jk + nbs * (2 + 3 * ip)]};
  double umf[4] = {0, c.scal->umf[1], c.scal->umf[2], c.scal->umf[3]};
  Elem e;
  eleme(S, c, g, cm, umf, e);
  double cha[5], d0[5];
#pragma unroll
  for (int q = 0; q < 5; q++) { d0[q] = drva[jk + nbs * (q + 5 * ip)]; cha[q] = d0[q]; }
  if (np == 10) {
    if (ra0 * (e.vn + e.vs + e.ao) > 0.0) cha[3] = 0.0;
    if (ra0 * (e.vn + e.vs - e.ao) > 0.0) cha[4] = 0.0;
  } else if (np == 20 || np == 25) {
    if (c.rpex[T.wall_off + jk] == 0.0) {
      const double s = cm[0] * c.scal->dudtmf[1] + cm[1] * c.scal->dudtmf[2] + cm[2] * c.scal->dudtmf[3];
      cha[3 + ip] = cha[4 - ip] + 2.0 * ra0 * e.aoi * c.qa[g] * (s + 50.0 * (e.vn + e.vs));
    }
  } else {  // 30: characteristic interface, incoming waves from the neighbour
    const BlockDev &Bn = c.blk[T.nb_b];
    const double *nbr = c.drva + Bn.face_off[nn] * 10;
    double *drvb = c.drvb + B.face_off[nn] * 10;
    double dha[5];
#pragma unroll
    for (int q = 0; q < 5; q++) {
      dha[q] = nbr[jk + nbs * (q + 5 * (1 - ip))];
      drvb[jk + nbs * (q + 5 * ip)] = dha[q];
    }
    if (ra0 * (e.vn + e.vs) > 0.0) { cha[0] = dha[0]; cha[1] = dha[1]; cha[2] = dha[2]; }
    if (ra0 * (e.vn + e.vs + e.ao) > 0.0) cha[3] = dha[3];
    if (ra0 * (e.vn + e.vs - e.ao) > 0.0) cha[4] = dha[4];
  }
  double xt[5][5];
  xtr2q(S, e, cm, xt);
  double dif[5], dh[5];
#pragma unroll
  for (int q = 0; q < 5; q++) dif[q] = cha[q] - d0[q];
#pragma unroll
  for (int r = 0; r < 5; r++) {
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < 5; q++) s += xt[r][q] * dif[q];
    dh[r] = s;
  }
  const double *w = c.sbcc + T.sbcc_off + (int64_t)jk * (MBCI + 1);
  for (int ii = 0; ii <= MBCI; ii++) {
    const int64_t g2 = B.off + idx3(B.lxi, B.let, i + iq * ii, j, k, nn);
    const double wv = w[ii];
#pragma unroll
    for (int q = 0; q < 5; q++) c.de[g2 + q * N] = c.de[g2 + q * N] + wv * dh[q];
  }
}

// wall temperature and velocity (src/Main3D.f90:886-895)
__global__ void k_wall(Ctx c, const FaceTask *tasks) {
  const FaceTask T = tasks[blockIdx.y];
  const int jk = blockIdx.x * blockDim.x + threadIdx.x;
  if (jk >= T.nline) return;
  const Scheme &S = *c.sc;
  const BlockDev &B = c.blk[T.b];
  int i, j, k, i1;
  face_point(B, T.nn, T.ip, jk, i, j, k, i1);
  const int64_t g = B.off + idx3(B.lxi, B.let, i, j, k, T.nn), N = c.N;
  const double ra0 = S.ham * S.hamm1 * S.wtemp;
  const double ra1 = (double)((T.bc - 20) / 5);
  const double rp = c.rpex[T.wall_off + jk];
  const double ra2 = 1.0 - rp, ra3 = 1.0 - ra1 * ra2;
  const double fctr = (1.0 - ra3) * c.qa[g];
  const double q2 = ra3 * c.qa[g + N] - fctr * c.scal->umf[1];
  const double q3 = ra3 * c.qa[g + 2 * N] - fctr * c.scal->umf[2];
  const double q4 = ra3 * c.qa[g + 3 * N] - fctr * c.scal->umf[3];
  c.qa[g + N] = q2; c.qa[g + 2 * N] = q3; c.qa[g + 3 * N] = q4;
  const double q1 = c.qa[g];
  c.qa[g + 4 * N] = rp * c.qa[g + 4 * N] + ra2 * (ra0 * q1 + 0.5 * (q2 * q2 + q3 * q3 + q4 * q4) / q1);
}

// junction averaging of the corner lines shared by four blocks
// (src/SingleTurbulence3D.f90:378-443)
__global__ void k_junction(Ctx c, const JunctionDev *jn, int njct) {
  const int jx = blockIdx.y;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (jx >= njct) return;
  const JunctionDev J = jn[jx];
  if (k >= J.nk) return;
  const int64_t N = c.N;
  int64_t g[4];
#pragma unroll
  for (int q = 0; q < 4; q++) g[q] = J.base[q] + (int64_t)k * J.kstr[q];
  double avg[5];
#pragma unroll
  for (int m = 0; m < 5; m++) {
    const double d1 = c.qa[g[0] + m * N], d2 = c.qa[g[1] + m * N], d3 = c.qa[g[2] + m * N], d4 = c.qa[g[3] + m * N];
    if (m == 0 || m == 4) avg[m] = 0.25 * (d1 + d2 + d3 + d4);
    else avg[m] = 0.5 * (c.qa[g[J.pa - 1] + m * N] + c.qa[g[J.pb - 1] + m * N]);
  }
#pragma unroll
  for (int q = 0; q < 4; q++)
#pragma unroll
    for (int m = 0; m < 5; m++) c.qa[g[q] + m * N] = avg[m];
}

// interface averaging: pack qa of every BC 30/35/45 face (src/Main3D.f90:908-914)
__global__ void k_pack(Ctx c, const FaceTask *tasks) {
  const FaceTask T = tasks[blockIdx.y];
  const int jk = blockIdx.x * blockDim.x + threadIdx.x;
  if (jk >= T.nline) return;
  const BlockDev &B = c.blk[T.b];
  int i, j, k, i1;
  face_point(B, T.nn, T.ip, jk, i, j, k, i1);
  const int64_t g = B.off + idx3(B.lxi, B.let, i, j, k, T.nn), N = c.N, nbs = T.nline;
  double *drva = c.drva + B.face_off[T.nn] * 10;
#pragma unroll
  for (int q = 0; q < 5; q++) drva[jk + nbs * (q + 5 * T.ip)] = c.qa[g + q * N];
  c.rr[g] = 1.0;
}

// interface averaging of the faces of one direction (src/Main3D.f90:926-952)
__global__ void k_avg(Ctx c, const FaceTask *tasks) {
  const FaceTask T = tasks[blockIdx.y];
  const int jk = blockIdx.x * blockDim.x + threadIdx.x;
  if (jk >= T.nline) return;
  const BlockDev &B = c.blk[T.b];
  const BlockDev &Bn = c.blk[T.nb_b];
  int i, j, k, i1;
  face_point(B, T.nn, T.ip, jk, i, j, k, i1);
  const int64_t g = B.off + idx3(B.lxi, B.let, i, j, k, T.nn), N = c.N, nbs = T.nline;
  const double *nbr = c.drva + Bn.face_off[T.nn] * 10;
  double *drvb = c.drvb + B.face_off[T.nn] * 10;
  const double cnt = c.rr[g] + 1.0;
  c.rr[g] = cnt;
  const double w = 1.0 / cnt;
  c.rr[g + N] = w;
#pragma unroll
  for (int q = 0; q < 5; q++) {
    const double dv = nbr[jk + nbs * (q + 5 * (1 - T.ip))];
    drvb[jk + nbs * (q + 5 * T.ip)] = dv;
    c.qa[g + q * N] = w * ((cnt - 1.0) * c.qa[g + q * N] + dv);
  }
}

// ---------------------------------------------------------------------------
// time-marching scalars: movef/pitch (src/Subroutineso.f90:192-259) and the
// dt schedule (src/Main3D.f90:571-610, 873-874, 964-965), one thread.
// ---------------------------------------------------------------------------
__device__ void d_movef(const Scheme &S, Scalars &s, double dtko, double dtk) {
  if (S.nsmf == 0) {
    const double ra0 = S.pi / S.timf, ra1 = ra0 * fmin(s.timo, S.timf), ra2 = ra0 * fmin(s.timo + dtko, S.timf);
    double fctr = 1.0 - cos(ra1), dfdt = ra0 * sin(ra2);
    double progmf = 0.5 * (fctr + dtk * dfdt);
    for (int q = 1; q <= 3; q++) s.umf[q] = progmf * S.uoo[q];
    fctr = sin(ra1);
    dfdt = ra0 * cos(ra2);
    progmf = 0.5 * ra0 * (fctr + dtk * dfdt);
    for (int q = 1; q <= 3; q++) s.dudtmf[q] = progmf * S.uoo[q];
    if (S.tp > 0 && s.timo + dtk > S.tps) {
      const double pi = S.pi, am = S.amachoo;
      const double daoa = (S.aoa1 - S.aoa0) * pi / 180, raoa0 = S.aoa0 * pi / 180;
      const double ra3 = s.timo - S.tps, dtsdt = pi / S.tp;
      const double ts = fmin(dtsdt * ra3, pi), tsdt = fmin(dtsdt * (ra3 + dtko), pi);
      const double aoat = raoa0 + 0.5 * daoa * (1 - cos(ts));
      const double aoatdt = raoa0 + 0.5 * daoa * (1 - cos(tsdt));
      const double f = 0.5 * daoa * dtsdt;
      const double ut1 = am * cos(aoat), ut2 = am * sin(aoat);
      const double du1 = -(am * f * sin(aoatdt) * sin(tsdt)), du2 = am * f * cos(aoatdt) * sin(tsdt);
      s.umf[1] = ut1 + dtk * du1; s.umf[2] = ut2 + dtk * du2; s.umf[3] = 0.0 + dtk * 0.0;
      const double dv1 = -(am * f * sin(aoat) * sin(ts)), dv2 = am * f * cos(aoat) * sin(ts);
      const double st = sin(tsdt);
      const double dd1 = -(am * f * (cos(aoatdt) * f * (st * st) + dtsdt * sin(aoatdt) * cos(tsdt)));
      const double dd2 = -(am * f * (sin(aoatdt) * f * (st * st) - dtsdt * cos(aoatdt) * cos(tsdt)));
      s.dudtmf[1] = dv1 + dtk * dd1; s.dudtmf[2] = dv2 + dtk * dd2; s.dudtmf[3] = 0.0 + dtk * 0.0;
      s.aoa = atan(s.umf[2] / s.umf[1]) * 180 / pi;
    }
  } else {
    for (int q = 1; q <= 3; q++) { s.umf[q] = S.uoo[q]; s.dudtmf[q] = 0.0; }
  }
}

__global__ void k_scalar(Ctx c, int op, int nk) {
  const Scheme &S = *c.sc;
  Scalars &s = *c.scal;
  const int nkrk = S.nkrk;
  if (op == SC_MOVEF_A) {
    const double dtko = s.dt * min(max(nk - 2, 0), 1) / (nkrk - nk + 3);
    const double dtk = s.dt * min(nk - 1, 1) / (nkrk - nk + 2);
    d_movef(S, s, dtko, dtk);
  } else if (op == SC_CFL_RESET) {
    s.cflmax[0] = 0ull; s.cflmax[1] = 0ull;
  } else if (op == SC_DT_NEW) {  // n % 10 == 1: new dt target
    s.ndt = s.n; s.dts = s.dte;
    if (S.dto < 0.0) {
      const double m1 = __longlong_as_double((long long)s.cflmax[0]);
      const double m2 = __longlong_as_double((long long)s.cflmax[1]);
      const double ra0 = S.cfl / m1;
      double ra1 = ra0;
      if (S.nviscous == 1) ra1 = 0.5 / m2;
      s.dte = fmin(ra0, ra1);
    } else {
      s.dte = S.dto;
    }
  } else if (op == SC_DT) {
    const double sn = sin(0.05 * S.pi * (double)(s.n - s.ndt));
    s.dt = s.dts + (s.dte - s.dts) * (sn * sn);
  } else if (op == SC_MOVEF_B) {
    const double dtko = s.dt * min(nk - 1, 1) / (nkrk - nk + 2);
    const double dtk = s.dt / (nkrk - nk + 1);
    d_movef(S, s, dtko, dtk);
    s.dtk = dtk;
  } else if (op == SC_ADVANCE) {
    s.n = s.n + 1;
    s.timo = s.timo + s.dt;
    if (!(fabs(s.dt) < 1e300)) s.flag |= 2;
  } else if (op == SC_INIT) {
    d_movef(S, s, 0.0, 0.0);
  }
}

// ---------------------------------------------------------------------------
// metrics (src/Main3D.f90:378-413): non-conservative cross products and J
// from the coordinate derivatives held in qo(1:3) (x), qa(1:3) (y), de(1:3) (z)
// ---------------------------------------------------------------------------
__global__ void k_metrics(Ctx c) {
  const int64_t N = c.N;
  GRID_STRIDE(g, N) {
    const double qo1 = c.qo[g], qo2 = c.qo[g + N], qo3 = c.qo[g + 2 * N];
    const double qa1 = c.qa[g], qa2 = c.qa[g + N], qa3 = c.qa[g + 2 * N];
    const double de1 = c.de[g], de2 = c.de[g + N], de3 = c.de[g + 2 * N];
    const double x1 = qa2 * de3 - de2 * qa3, x2 = de2 * qo3 - qo2 * de3, x3 = qo2 * qa3 - qa2 * qo3;
    const double e1 = qa3 * de1 - de3 * qa1, e2 = de3 * qo1 - qo3 * de1, e3 = qo3 * qa1 - qa3 * qo1;
    const double z1 = qa1 * de2 - de1 * qa2, z2 = de1 * qo2 - qo1 * de2, z3 = qo1 * qa2 - qa1 * qo2;
    c.xim[g] = x1; c.xim[g + N] = x2; c.xim[g + 2 * N] = x3;
    c.etm[g] = e1; c.etm[g + N] = e2; c.etm[g + 2 * N] = e3;
    c.zem[g] = z1; c.zem[g + N] = z2; c.zem[g + 2 * N] = z3;
    c.yaco[g] = 3.0 / (qo1 * x1 + qo2 * e1 + qo3 * z1 + qa1 * x2 + qa2 * e2 + qa3 * z2 + de1 * x3 + de2 * e3 + de3 * z3);
  }
}

// clpost wall integrals (src/rpt.f90:1017-1056), one CTA per wall face,
// deterministic tree sum; out[face*2 + dir]
__global__ void k_forces(Ctx c, const FaceTask *tasks, const double *area, const double *wnor, const int64_t *woff,
                         double *out) {
  const FaceTask T = tasks[blockIdx.x];
  const BlockDev &B = c.blk[T.b];
  const int64_t N = c.N, nw = T.nline;
  const double *ar = area + woff[blockIdx.x], *wn = wnor + 3 * woff[blockIdx.x];
  double acc[2] = {0.0, 0.0};
  for (int64_t ll = threadIdx.x; ll < nw; ll += blockDim.x) {
    // wall list order of wallArea: k over lze, i over lxi (src/rpt.f90:802-803)
    const int kk = (int)(ll / (B.lxi + 1)), ii = (int)(ll % (B.lxi + 1));
    const int jw = T.ip * B.let;
    const int64_t g = B.off + ((int64_t)kk * (B.let + 1) + jw) * (B.lxi + 1) + ii;
    const double w1 = wn[ll], w2 = wn[ll + nw], w3 = wn[ll + 2 * nw];
    for (int dir = 0; dir < 2; dir++) {
      double v = c.p[g] * (dir == 0 ? w1 : w2) * ar[ll];
      if (c.sc->nviscous == 1) {
        const double *t = c.tau;
        double tw;
        if (dir == 0) tw = c.qa[g] * (t[g] * w1 + t[g + 3 * N] * w2 + t[g + 5 * N] * w3);
        else tw = c.qa[g] * (t[g + 3 * N] * w1 + t[g + N] * w2 + t[g + 4 * N] * w3);
        v += tw * ar[ll];
      }
      acc[dir] += v;
    }
  }
  __shared__ double sh[2][256];
  sh[0][threadIdx.x] = acc[0];
  sh[1][threadIdx.x] = acc[1];
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sh[0][threadIdx.x] += sh[0][threadIdx.x + s];
      sh[1][threadIdx.x] += sh[1][threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[blockIdx.x * 2 + 0] = sh[0][0];
    out[blockIdx.x * 2 + 1] = sh[1][0];
  }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
void launch_sweep(const Ctx &c, cudaStream_t st, int nn, bool filt, const double *in, double *out, int m, int nblocks,
                  int maxlines) {
  const int tpb = 128;
  dim3 grid((maxlines + tpb - 1) / tpb, nblocks);
  if (!filt) {
    if (nn == 1) k_sweep<1, false><<<grid, tpb, 0, st>>>(c, in, out, m);
    else if (nn == 2) k_sweep<2, false><<<grid, tpb, 0, st>>>(c, in, out, m);
    else k_sweep<3, false><<<grid, tpb, 0, st>>>(c, in, out, m);
  } else {
    if (nn == 1) k_sweep<1, true><<<grid, tpb, 0, st>>>(c, in, out, m);
    else if (nn == 2) k_sweep<2, true><<<grid, tpb, 0, st>>>(c, in, out, m);
    else k_sweep<3, true><<<grid, tpb, 0, st>>>(c, in, out, m);
  }
}

void launch_mpigo(const Ctx &c, cudaStream_t st, const FaceTask *tasks, int ntask, int maxline, int nt, int n45,
                  const double *s1, const double *s2, const double *s3) {
  if (ntask == 0) return;
  const int tpb = 128;
  k_mpigo<<<dim3((maxline + tpb - 1) / tpb, ntask), tpb, 0, st>>>(c, tasks, nt, n45, s1, s2, s3);
}

static int pw_grid(int64_t N) {
  int64_t b = (N + 255) / 256;
  const int64_t cap = 152 * 16;
  return (int)(b < cap ? (b < 1 ? 1 : b) : cap);
}

void launch_pointwise(const Ctx &c, cudaStream_t st, int which, int m, double *o1, double *o2, double *o3) {
  const int g = pw_grid(c.N), t = 256;
  switch (which) {
    case PW_PRIM: k_prim<<<g, t, 0, st>>>(c); break;
    case PW_CFL: k_cfl<<<g, t, 0, st>>>(c); break;
    case PW_GRAD: k_grad<<<g, t, 0, st>>>(c, o1, o2, o3); break;
    case PW_STRESS: k_stress<<<g, t, 0, st>>>(c); break;
    case PW_FLUXPREP: k_fluxprep<<<g, t, 0, st>>>(c); break;
    case PW_FLUX: k_flux<<<g, t, 0, st>>>(c, m); break;
    case PW_DIV: k_div<<<g, t, 0, st>>>(c, m); break;
    case PW_RK: k_rk<<<g, t, 0, st>>>(c); break;
    case PW_METRICS: k_metrics<<<g, t, 0, st>>>(c); break;
  }
}

void launch_face(const Ctx &c, cudaStream_t st, int which, const FaceTask *tasks, int ntask, int maxline) {
  if (ntask == 0) return;
  const int tpb = 128;
  dim3 grid((maxline + tpb - 1) / tpb, ntask);
  switch (which) {
    case FK_GCBC_PREP: k_gcbc_prep<<<grid, tpb, 0, st>>>(c, tasks); break;
    case FK_GCBC_APPLY: k_gcbc_apply<<<grid, tpb, 0, st>>>(c, tasks); break;
    case FK_WALL: k_wall<<<grid, tpb, 0, st>>>(c, tasks); break;
    case FK_PACK: k_pack<<<grid, tpb, 0, st>>>(c, tasks); break;
    case FK_AVG: k_avg<<<grid, tpb, 0, st>>>(c, tasks); break;
  }
}

void launch_junction(const Ctx &c, cudaStream_t st, const JunctionDev *jn, int njct, int nk) {
  if (njct == 0) return;
  const int tpb = 64;
  k_junction<<<dim3((nk + tpb - 1) / tpb, njct), tpb, 0, st>>>(c, jn, njct);
}

void launch_scalar(const Ctx &c, cudaStream_t st, int op, int nk) { k_scalar<<<1, 1, 0, st>>>(c, op, nk); }

void launch_forces(const Ctx &c, cudaStream_t st, const FaceTask *tasks, int ntask, const double *area,
                   const double *wnor, const int64_t *woff, double *out) {
  if (ntask == 0) return;
  k_forces<<<ntask, 256, 0, st>>>(c, tasks, area, wnor, woff, out);
}

}  // namespace ATI_KNS
}  // namespace ati
