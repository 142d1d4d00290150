// ati_kernels.cu — sm_103a kernels of the ATI3D per-RK-stage hot path.
//
// Each kernel restates one loop nest of the reference (cited per kernel) over
// all blocks of the case at once.  The kernels are templated on the type of
// the stage intermediates (double: the FP64 path, float: the mixed path; the
// state qa/qo stays double) and keep the reference's operation order.  This
// file is compiled twice: into namespace ati::fast with FMA contraction and
// into ati::strict with -fmad=false, where every operation rounds as the
// reference's Fortran expressions do (set-up and the granular calls, which
// then agree with the CPU restatement bit for bit).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <map>
#include <mutex>
#include <type_traits>
#include <utility>

#include "ati_convert.h"
#include "ati_kernels.h"
#include "ati_tma.h"

#ifndef ATI_KNS
#error "compile with -DATI_KNS=fast or -DATI_KNS=strict"
#endif
#ifndef ATI_KFAST
#error "compile with -DATI_KFAST=1 (fast) or -DATI_KFAST=0 (strict)"
#endif

namespace ati {
namespace ATI_KNS {

// the fast build may reorder the FP64 line solves (scaled-factor tables);
// the strict build keeps the reference's operation order
constexpr bool kFast = ATI_KFAST != 0;

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

// asynchronous global-to-shared copies (cp.async, sm_80 and later): the copy
// holds no register while in flight, so a thread can have a whole line's
// loads outstanding at once.  A thread's own copies are complete after
// cp_async_wait; other threads see them after a barrier that follows the wait.
template <int BYTES>
__device__ __forceinline__ void cp_async(void *smem, const void *gmem) {
  static_assert(BYTES == 4 || BYTES == 8 || BYTES == 16, "cp.async.ca copies 4, 8 or 16 bytes");
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(s), "l"(gmem), "n"(BYTES) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int PENDING>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(PENDING) : "memory");
}

// ---------------------------------------------------------------------------
// Compact derivative / filter of one line: deriv (src/Subroutines3D.f90:84-141)
// and filte (src/Subroutines3D.f90:145-206).  ld(i) gives the original value at
// position i, fw holds the forward-elimination values, put(i, v) receives the
// derivative (or the filter correction) at i.  The six boundary rows and the
// first window are read before anything is stored, so fw may alias the input
// (in-place solve in shared memory).
// ---------------------------------------------------------------------------
template <bool FILT, typename TC, class Src>
__device__ __forceinline__ void line_ends(const Coef<TC> &C, int L, int ns, int ne, const TC *rcv, int64_t nbs, int jk,
                                          const Src &ld, TC &sbs0, TC &sbs1, TC &sbs2, TC &sbe0, TC &sbe1,
                                          TC &sbe2) {
  const TC two = (TC)2;
  if (!FILT) {
    const TC aa = C.aa, ab = C.ab, ac = C.ac;
    if (ns == 0) {
      const TC w0 = ld(0), w1 = ld(1), w2 = ld(2), w3 = ld(3), w4 = ld(4), w5 = ld(5), w6 = ld(6);
      const TC *a = C.abc[0];
      sbs0 = a[0] * (w1 - w0) + a[1] * (w2 - w0) + a[2] * (w3 - w0) + a[3] * (w4 - w0) + a[4] * (w5 - w0) + a[5] * (w6 - w0);
      a = C.abc[1];
      sbs1 = a[0] * (w0 - w1) + a[1] * (w2 - w1) + a[2] * (w3 - w1) + a[3] * (w4 - w1) + a[4] * (w5 - w1) + a[5] * (w6 - w1);
      a = C.abc[2];
      sbs2 = a[0] * (w0 - w2) + a[1] * (w1 - w2) + a[2] * (w3 - w2) + a[3] * (w4 - w2) + a[4] * (w5 - w2) + a[5] * (w6 - w2);
    } else {
      TC s0 = 0, s1 = 0;
#pragma unroll
      for (int q = 0; q <= LMD; q++) {
        const TC v = ld(q);
        s0 += C.pbci[0][0][q] * v;
        s1 += C.pbci[0][1][q] * v;
      }
      sbs0 = s0 + rcv[jk + nbs * 0];
      sbs1 = s1 + rcv[jk + nbs * 1];
      sbs2 = aa * (ld(3) - ld(1)) + ab * (ld(4) - ld(0)) + ac * (ld(5) - rcv[jk + nbs * 2]);
    }
    if (ne == 0) {
      const TC w0 = ld(L - 1), w1 = ld(L - 2), w2 = ld(L - 3), w3 = ld(L - 4), w4 = ld(L - 5), w5 = ld(L - 6),
               w6 = ld(L - 7);
      const TC *a = C.abc[0];
      sbe0 = a[0] * (w0 - w1) + a[1] * (w0 - w2) + a[2] * (w0 - w3) + a[3] * (w0 - w4) + a[4] * (w0 - w5) + a[5] * (w0 - w6);
      a = C.abc[1];
      sbe1 = a[0] * (w1 - w0) + a[1] * (w1 - w2) + a[2] * (w1 - w3) + a[3] * (w1 - w4) + a[4] * (w1 - w5) + a[5] * (w1 - w6);
      a = C.abc[2];
      sbe2 = a[0] * (w2 - w0) + a[1] * (w2 - w1) + a[2] * (w2 - w3) + a[3] * (w2 - w4) + a[4] * (w2 - w5) + a[5] * (w2 - w6);
    } else {
      TC s0 = 0, s1 = 0;
#pragma unroll
      for (int q = 0; q <= LMD; q++) {
        const TC v = ld(L - 1 - q);
        s0 += C.pbci[0][0][q] * v;
        s1 += C.pbci[0][1][q] * v;
      }
      sbe0 = -s0 - rcv[jk + nbs * 3];
      sbe1 = -s1 - rcv[jk + nbs * 4];
      sbe2 = aa * (ld(L - 2) - ld(L - 4)) + ab * (ld(L - 1) - ld(L - 5)) + ac * (rcv[jk + nbs * 5] - ld(L - 6));
    }
  } else {
    const TC fa = C.fa, fb = C.fb, fc = C.fc;
    if (ns == 0) {
      const TC w0 = ld(0), w1 = ld(1), w2 = ld(2), w3 = ld(3), w4 = ld(4), w5 = ld(5);
      const TC ra0 = two * w0, ra1 = two * w1, ra2 = two * w2;
      const TC res = C.fex[1] * (w1 - w0) + C.fex[2] * (w2 - w0) + C.fex[3] * (w3 - w0);
      const TC rv1 = w0 - res * C.ffx[1], rv2 = w0 - res * C.ffx[2], rv3 = w0 - res * C.ffx[3];
      sbs0 = C.fam[0] * (rv1 + w1 - ra0) + C.fbm[0] * (rv2 + w2 - ra0) + C.fcm[0] * (rv3 + w3 - ra0);
      sbs1 = C.fam[1] * (w0 + w2 - ra1) + C.fbm[1] * (rv1 + w3 - ra1) + C.fcm[1] * (rv2 + w4 - ra1);
      sbs2 = C.fam[2] * (w1 + w3 - ra2) + C.fbm[2] * (w0 + w4 - ra2) + C.fcm[2] * (rv1 + w5 - ra2);
    } else {
      TC s0 = 0, s1 = 0;
#pragma unroll
      for (int q = 0; q <= LMF; q++) {
        const TC v = ld(q);
        s0 += C.pbci[1][0][q] * v;
        s1 += C.pbci[1][1][q] * v;
      }
      const TC ra2 = two * ld(2);
      sbs0 = s0 + rcv[jk + nbs * 0];
      sbs1 = s1 + rcv[jk + nbs * 1];
      sbs2 = fa * (ld(1) + ld(3) - ra2) + fb * (ld(0) + ld(4) - ra2) + fc * (rcv[jk + nbs * 2] + ld(5) - ra2);
    }
    if (ne == 0) {
      const TC w0 = ld(L - 1), w1 = ld(L - 2), w2 = ld(L - 3), w3 = ld(L - 4), w4 = ld(L - 5), w5 = ld(L - 6);
      const TC ra0 = two * w0, ra1 = two * w1, ra2 = two * w2;
      const TC res = C.fex[1] * (w0 - w1) + C.fex[2] * (w0 - w2) + C.fex[3] * (w0 - w3);
      const TC rv1 = w0 + res * C.ffx[1], rv2 = w0 + res * C.ffx[2], rv3 = w0 + res * C.ffx[3];
      sbe0 = C.fam[0] * (w1 + rv1 - ra0) + C.fbm[0] * (w2 + rv2 - ra0) + C.fcm[0] * (w3 + rv3 - ra0);
      sbe1 = C.fam[1] * (w2 + w0 - ra1) + C.fbm[1] * (w3 + rv1 - ra1) + C.fcm[1] * (w4 + rv2 - ra1);
      sbe2 = C.fam[2] * (w3 + w1 - ra2) + C.fbm[2] * (w4 + w0 - ra2) + C.fcm[2] * (w5 + rv1 - ra2);
    } else {
      TC s0 = 0, s1 = 0;
#pragma unroll
      for (int q = 0; q <= LMF; q++) {
        const TC v = ld(L - 1 - q);
        s0 += C.pbci[1][0][q] * v;
        s1 += C.pbci[1][1][q] * v;
      }
      const TC ra2 = two * ld(L - 3);
      sbe0 = s0 + rcv[jk + nbs * 3];
      sbe1 = s1 + rcv[jk + nbs * 4];
      sbe2 = fa * (ld(L - 4) + ld(L - 2) - ra2) + fb * (ld(L - 5) + ld(L - 1) - ra2) +
             fc * (ld(L - 6) + rcv[jk + nbs * 5] - ra2);
    }
  }
}

// right-hand side of interior row i from the window a0..a6 = ld(i-3..i+3)
template <bool FILT, typename TC>
__device__ __forceinline__ TC interior_rhs(const Coef<TC> &C, TC a0, TC a1, TC a2, TC a3, TC a4, TC a5, TC a6) {
  if (!FILT) return C.aa * (a4 - a2) + C.ab * (a5 - a1) + C.ac * (a6 - a0);
  const TC res = (TC)2 * a3;
  return C.fa * (a2 + a4 - res) + C.fb * (a1 + a5 - res) + C.fc * (a0 + a6 - res);
}

template <bool FILT, typename TC, class Src, class Fw, class Sink>
__device__ __forceinline__ void solve_line(const Coef<TC> &C, const TC *fac, int L, int ns, int ne, const TC *rcv,
                                           int64_t nbs, int jk, const Src &ld, Fw &fw, Sink &put, TC &first,
                                           TC &last) {
  TC sbs0, sbs1, sbs2, sbe0, sbe1, sbe2;
  line_ends<FILT, TC>(C, L, ns, ne, rcv, nbs, jk, ld, sbs0, sbs1, sbs2, sbe0, sbe1, sbe2);
  // the first window is read before any forward value is stored
  TC a0 = ld(0), a1 = ld(1), a2 = ld(2), a3 = ld(3), a4 = ld(4), a5 = ld(5);
  // forward elimination (src/Subroutines3D.f90:124-128 / 190-194)
  TC f2 = sbs0;
  TC f1 = sbs1 - __ldg(fac + (1 * 5 + 1)) * f2;
  fw.st(0, f2);
  fw.st(1, f1);
  {
    const TC v = sbs2 - __ldg(fac + (2 * 5 + 0)) * f2 - __ldg(fac + (2 * 5 + 1)) * f1;
    fw.st(2, v);
    f2 = f1; f1 = v;
  }
  // interior rows in blocks of four, software-pipelined: the next block's
  // inputs are read before this block's forward values are stored, so the
  // loads are in flight during the recurrence even where the compiler cannot
  // tell the forward store from the input (both in one shared-memory column)
  auto fstep = [&](int i, TC a6) {
    const TC sb = interior_rhs<FILT, TC>(C, a0, a1, a2, a3, a4, a5, a6);
    const TC v = sb - __ldg(fac + (i * 5 + 0)) * f2 - __ldg(fac + (i * 5 + 1)) * f1;
    fw.st(i, v);
    f2 = f1; f1 = v;
    a0 = a1; a1 = a2; a2 = a3; a3 = a4; a4 = a5; a5 = a6;
  };
  const int iend = L - 4;  // last interior row
  int i = 3;
  if (i + 3 <= iend) {
    TC n0 = ld(i + 3), n1 = ld(i + 4), n2 = ld(i + 5), n3 = ld(i + 6);
    for (; i + 3 <= iend; i += 4) {
      const TC c0 = n0, c1 = n1, c2 = n2, c3 = n3;
      if (i + 7 <= iend) { n0 = ld(i + 7); n1 = ld(i + 8); n2 = ld(i + 9); n3 = ld(i + 10); }
      fstep(i, c0);
      fstep(i + 1, c1);
      fstep(i + 2, c2);
      fstep(i + 3, c3);
    }
  }
  for (; i <= iend; i++) fstep(i, ld(i + 3));
  {
    int i = L - 3;
    TC v = sbe2 - __ldg(fac + (i * 5 + 0)) * f2 - __ldg(fac + (i * 5 + 1)) * f1;
    fw.st(i, v);
    f2 = f1; f1 = v;
    i = L - 2;
    v = sbe1 - __ldg(fac + (i * 5 + 0)) * f2 - __ldg(fac + (i * 5 + 1)) * f1;
    fw.st(i, v);
    f2 = f1; f1 = v;
    i = L - 1;
    v = sbe0 - __ldg(fac + (i * 5 + 0)) * f2 - __ldg(fac + (i * 5 + 1)) * f1;
    f2 = f1; f1 = v;  // f1 = fw(L-1), f2 = fw(L-2)
  }
  // back substitution (src/Subroutines3D.f90:129-136 / 195-202)
  TC b0 = __ldg(fac + ((L - 1) * 5 + 2)) * f1;
  TC b1 = __ldg(fac + ((L - 2) * 5 + 2)) * f2 - __ldg(fac + ((L - 2) * 5 + 3)) * b0;
  last = b0;
  put(L - 1, b0);
  put(L - 2, b1);
  // blocks of four rows, the next block's forward values read before this block's results are stored
  auto bstep = [&](int i, TC w) {
    const TC v = __ldg(fac + (i * 5 + 2)) * w - __ldg(fac + (i * 5 + 3)) * b1 - __ldg(fac + (i * 5 + 4)) * b0;
    put(i, v);
    b0 = b1; b1 = v;
  };
  int k = L - 3;
  if (k >= 3) {
    TC m0 = fw.ld(k), m1 = fw.ld(k - 1), m2 = fw.ld(k - 2), m3 = fw.ld(k - 3);
    for (; k >= 3; k -= 4) {
      const TC c0 = m0, c1 = m1, c2 = m2, c3 = m3;
      if (k >= 7) { m0 = fw.ld(k - 4); m1 = fw.ld(k - 5); m2 = fw.ld(k - 6); m3 = fw.ld(k - 7); }
      bstep(k, c0);
      bstep(k - 1, c1);
      bstep(k - 2, c2);
      bstep(k - 3, c3);
    }
  }
  for (; k >= 0; k--) bstep(k, fw.ld(k));
  first = b1;
}

// The FP64 fast path's line solve: the same elimination with the forward
// values carried as u = c2 v (scaled-factor rows, FU_RT per row), 10 FP64
// operations per point of a derivative instead of 11.  Pipelined like solve_line.
template <bool FILT, class Src, class Fw, class Sink>
__device__ __forceinline__ void solve_line_u(const Coef<double> &C, const double *fu, int L, int ns, int ne,
                                             const double *rcv, int64_t nbs, int jk, const Src &ld, Fw &fw, Sink &put,
                                             double &first, double &last) {
  double sbs0, sbs1, sbs2, sbe0, sbe1, sbe2;
  line_ends<FILT, double>(C, L, ns, ne, rcv, nbs, jk, ld, sbs0, sbs1, sbs2, sbe0, sbe1, sbe2);
  double a0 = ld(0), a1 = ld(1), a2 = ld(2), a3 = ld(3), a4 = ld(4), a5 = ld(5);
  auto F = [&](int i, int k) { return __ldg(fu + i * FU_RT + k); };
  double u2 = F(0, 7) * sbs0;
  double u1 = F(1, 7) * sbs1 - F(1, 1) * u2;
  fw.st(0, u2);
  fw.st(1, u1);
  {
    const double v = F(2, 7) * sbs2 - F(2, 0) * u2 - F(2, 1) * u1;
    fw.st(2, v);
    u2 = u1; u1 = v;
  }
  auto fstep = [&](int i, double a6) {
    double r;
    if (!FILT) {
      r = F(i, 2) * (a4 - a2) + F(i, 3) * (a5 - a1) + F(i, 4) * (a6 - a0);
    } else {
      r = F(i, 2) * (a2 + a4) + F(i, 3) * (a1 + a5) + F(i, 4) * (a0 + a6) - F(i, 8) * a3;
    }
    const double v = r - F(i, 0) * u2 - F(i, 1) * u1;
    fw.st(i, v);
    u2 = u1; u1 = v;
    a0 = a1; a1 = a2; a2 = a3; a3 = a4; a4 = a5; a5 = a6;
  };
  const int iend = L - 4;
  int i = 3;
  if (i + 3 <= iend) {
    double n0 = ld(i + 3), n1 = ld(i + 4), n2 = ld(i + 5), n3 = ld(i + 6);
    for (; i + 3 <= iend; i += 4) {
      const double c0 = n0, c1 = n1, c2 = n2, c3 = n3;
      if (i + 7 <= iend) { n0 = ld(i + 7); n1 = ld(i + 8); n2 = ld(i + 9); n3 = ld(i + 10); }
      fstep(i, c0);
      fstep(i + 1, c1);
      fstep(i + 2, c2);
      fstep(i + 3, c3);
    }
  }
  for (; i <= iend; i++) fstep(i, ld(i + 3));
  {
    int k = L - 3;
    double v = F(k, 7) * sbe2 - F(k, 0) * u2 - F(k, 1) * u1;
    fw.st(k, v);
    u2 = u1; u1 = v;
    k = L - 2;
    v = F(k, 7) * sbe1 - F(k, 0) * u2 - F(k, 1) * u1;
    fw.st(k, v);
    u2 = u1; u1 = v;
    k = L - 1;
    v = F(k, 7) * sbe0 - F(k, 0) * u2 - F(k, 1) * u1;
    u2 = u1; u1 = v;  // u1 = u(L-1), u2 = u(L-2)
  }
  double b0 = u1;
  double b1 = u2 - F(L - 2, 5) * b0;
  last = b0;
  put(L - 1, b0);
  put(L - 2, b1);
  auto bstep = [&](int k, double w) {
    const double v = w - F(k, 5) * b1 - F(k, 6) * b0;
    put(k, v);
    b0 = b1; b1 = v;
  };
  int k = L - 3;
  if (k >= 3) {
    double m0 = fw.ld(k), m1 = fw.ld(k - 1), m2 = fw.ld(k - 2), m3 = fw.ld(k - 3);
    for (; k >= 3; k -= 4) {
      const double c0 = m0, c1 = m1, c2 = m2, c3 = m3;
      if (k >= 7) { m0 = fw.ld(k - 4); m1 = fw.ld(k - 5); m2 = fw.ld(k - 6); m3 = fw.ld(k - 7); }
      bstep(k, c0);
      bstep(k - 1, c1);
      bstep(k - 2, c2);
      bstep(k - 3, c3);
    }
  }
  for (; k >= 0; k--) bstep(k, fw.ld(k));
  first = b1;
}

// line geometry of direction NN: base point, stride, face index, length
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

// input conversion: a wider input loses its constant offset before rounding
template <typename TI, typename TC>
__device__ __forceinline__ TC cvt_in(TI v, TI ofs) {
  if constexpr (std::is_same<TI, TC>::value) return v;
  else return cvt<TC>(ofs == (TI)0 ? v : v - ofs);  // x - 0 is x: no subtraction for offset-free fields
}

template <typename TI, typename TC>
struct GlobalSrc {
  const TI *p;
  int64_t s;
  TI ofs;
  // read-only-path loads: every element of a line is read before the line's first result is
  // stored, so the loads may be scheduled ahead of the forward-value stores
  __device__ __forceinline__ TC operator()(int i) const { return cvt_in<TI, TC>(__ldg(p + (int64_t)i * s), ofs); }
};
template <typename TC>
struct GlobalFw {
  TC *p;
  int64_t s;
  __device__ __forceinline__ void st(int i, TC v) { p[(int64_t)i * s] = v; }
  __device__ __forceinline__ TC ld(int i) const { return p[(int64_t)i * s]; }
};
// forward values of one line in shared memory, column threadIdx.x of a [i][line] tile
template <typename TC>
struct SmemFw {
  TC *p;
  int s;
  __device__ __forceinline__ void st(int i, TC v) { p[i * s] = v; }
  __device__ __forceinline__ TC ld(int i) const { return p[i * s]; }
};
template <bool FILT, typename TI, typename TO, typename TC>
struct GlobalSink {
  const TI *in;
  TO *out, *out2;
  int64_t s;
  __device__ __forceinline__ void operator()(int i, TC v) {
    const int64_t o = (int64_t)i * s;
    TO r;
    if (FILT) r = (TO)(in[o] + cvt<TI>(v));  // rr = rr + sb (src/Subroutines3D.f90:200-202)
    else r = (TO)v;
    out[o] = r;
    if (out2) out2[o] = r;
  }
};

template <typename TI, typename TO, typename TC>
struct SweepArgs {
  const BlockDev *blk;
  const LTile *lt;  // work queue: tile blockIdx.x = lines [t0, t0 + CTA lines) of block b
  const Coef<TC> *cf;
  const TC *fac;
  SweepIO<TI, TO> io;
  TC *fw;
  int64_t fw_fs;
  const TC *recv;
  int64_t recv_fs;
  TC *drva;
  const double *facu;  // FP64 fast path: scaled-factor rows (FU_RT per row)
  const TmaMap *tmap;  // TMA staging (segmented eta/zeta sweeps): this array's tensor map of block b at tmap[b]
  Scalars *scal;       // per-case flags (a bounded wait that gave up sets FLAG_TIMEOUT)
  bool rowtiles;       // segmented eta tiles end with their grid row
};

// eta and zeta lines: one thread per line; consecutive threads own
// consecutive xi positions, so each warp access of an eta or zeta sweep is one
// contiguous row.  A CTA takes the lines of one work-queue tile of one block
// (sg_lines[NN] of them, one per thread).
// SFW: lines short enough that a CTA's lines fit 48 KB are staged whole in
// shared memory (one column per thread) and solved there: all loads of a line
// are in flight at once, and the forward values skip their round trip through DRAM
template <int NN, bool FILT, bool SFW, typename TI, typename TO, typename TC>
__global__ void __launch_bounds__(SG_MAX) k_sweep_g(SweepArgs<TI, TO, TC> a) {
  extern __shared__ __align__(16) unsigned char sg_smem[];
  const LTile LT = a.lt[blockIdx.x];
  const BlockDev &B = a.blk[LT.b];
  const int f = blockIdx.y;
  int64_t base, stride;
  int jk, L;
  if (!line_geom<NN>(B, LT.t0 + threadIdx.x, base, stride, jk, L)) return;
  const Coef<TC> &C = *a.cf;
  const int ns = B.ndf[0][NN], ne = B.ndf[1][NN];
  const int64_t nbs = B.nbsize[NN];
  const TC *rcv = a.recv + f * a.recv_fs + B.face_off[NN] * 6;
  const TC *fac = a.fac + B.fac_off[NN] * 5;
  constexpr bool UF = kFast && std::is_same<TC, double>::value;  // scaled-factor rows
  const double *fu = UF ? a.facu + B.fac_off[NN] * FU_RT : nullptr;
  const TI *pin = a.io.in + f * a.io.in_fs + base;
  GlobalSrc<TI, TC> ld{pin, stride, a.io.ofs[f]};
  TO *o2 = a.io.out2 ? a.io.out2 + f * a.io.out_fs + base : nullptr;
  GlobalSink<FILT, TI, TO, TC> put{pin, a.io.out + f * a.io.out_fs + base, o2, stride};
  TC first, last;
  if constexpr (SFW) {
    // the whole line first, every load issued back to back, then the recurrences on shared memory
    // (the forward values overwrite inputs already consumed, as solve_line allows)
    TC *col = reinterpret_cast<TC *>(sg_smem) + threadIdx.x;
    const int P = (int)blockDim.x;
    if constexpr (std::is_same<TI, TC>::value) {
      // same type in and out: asynchronous copies, the whole line outstanding at once
#pragma unroll 8
      for (int i = 0; i < L; i++) cp_async<sizeof(TC)>(col + i * P, pin + (int64_t)i * stride);
      cp_async_commit();
      cp_async_wait<0>();
    } else {
#pragma unroll 8
      for (int i = 0; i < L; i++) col[i * P] = ld(i);
    }
    SmemFw<TC> fw{col, P};
    const SmemFw<TC> lds{col, P};
    auto sld = [&](int i) { return lds.ld(i); };
    if constexpr (UF) solve_line_u<FILT>(C, fu, L, ns, ne, rcv, nbs, jk, sld, fw, put, first, last);
    else solve_line<FILT, TC>(C, fac, L, ns, ne, rcv, nbs, jk, sld, fw, put, first, last);
  } else {
    GlobalFw<TC> fw{a.fw + f * a.fw_fs + base, stride};
    if constexpr (UF) solve_line_u<FILT>(C, fu, L, ns, ne, rcv, nbs, jk, ld, fw, put, first, last);
    else solve_line<FILT, TC>(C, fac, L, ns, ne, rcv, nbs, jk, ld, fw, put, first, last);
  }
  if (!FILT && a.io.drva) {
    TC *d = a.drva + B.face_off[NN] * 10;
    const int m = a.io.m0 + f;
    d[jk + nbs * ((m - 1) + 5 * 0)] = first;  // drva(jk,m,0) = sb(is)
    d[jk + nbs * ((m - 1) + 5 * 1)] = last;   // drva(jk,m,1) = sb(ie)
  }
}

// xi lines, chunked through shared memory.  A CTA owns XC_NL consecutive xi
// lines of one block and one field (one thread per line) and streams them in
// chunks of XC_C points: each chunk is loaded with coalesced reads into a
// transposed tile [point][line], every thread advances its own recurrence
// through the chunk, and the tile goes back to global memory coalesced.  The
// forward pass writes fw(i) at position i+3 of the scratch plane (the point
// whose load completed row i); the backward pass reads those chunks in reverse
// and writes the result of row i at position i.  The six boundary rows use
// direct loads of the line ends, and the last three forward values stay in
// registers.  The tile is small (XC_C x XC_NL words), so many CTAs share an SM.
constexpr int XC_C = 32;

template <bool FILT, typename TI, typename TO, typename TC>
__global__ void __launch_bounds__(XC_NL) k_sweep_xc(SweepArgs<TI, TO, TC> a) {
  // FP32 lines of one type in and out: two tiles, the next chunk's asynchronous
  // copies in flight while the recurrences run through the current one
  constexpr bool AS = std::is_same<TI, TC>::value && sizeof(TC) == 4;
  constexpr int NBUF = AS ? 2 : 1;
  __shared__ TC tile[NBUF][XC_C][XC_NL + 1];
  const LTile LT = a.lt[blockIdx.x];
  const BlockDev &B = a.blk[LT.b];
  const int f = blockIdx.y;
  const int L = B.lxi + 1, nline = (B.let + 1) * (B.lze + 1);
  const int t0 = LT.t0;
  const int nl = min(XC_NL, nline - t0);
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  constexpr int NW = XC_NL / 32;
  const bool act = t < nl;
  const int64_t off = B.off + (int64_t)t0 * L;
  const TI *in = a.io.in + f * a.io.in_fs + off;
  TC *fwg = a.fw + f * a.fw_fs + off;
  TO *out = a.io.out + f * a.io.out_fs + off;
  TO *out2 = a.io.out2 ? a.io.out2 + f * a.io.out_fs + off : nullptr;
  const Coef<TC> &C = *a.cf;
  const TC *fac = a.fac + B.fac_off[1] * 5;
  constexpr bool UF = kFast && std::is_same<TC, double>::value;  // scaled-factor rows (see solve_line_u)
  const double *fu = UF ? a.facu + B.fac_off[1] * FU_RT : nullptr;
  const int jk = t0 + t;
  const int64_t nbs = B.nbsize[1];
  // forward row i from a closure right-hand side sb (rows 0-2 and the last three)
  auto end_row = [&](int i, TC sb, TC g2, TC g1) -> TC {
    if constexpr (UF) return fu[i * FU_RT + 7] * sb - fu[i * FU_RT + 0] * g2 - fu[i * FU_RT + 1] * g1;
    else return sb - fac[i * 5 + 0] * g2 - fac[i * 5 + 1] * g1;
  };

  // boundary rows and the first window from the line itself
  TC sbs0 = 0, sbs1 = 0, sbs2 = 0, sbe0 = 0, sbe1 = 0, sbe2 = 0;
  TC a0 = 0, a1 = 0, a2 = 0, a3 = 0, a4 = 0, a5 = 0, f1 = 0, f2 = 0, w0 = 0, w1 = 0, w2 = 0;
  if (act) {
    const TC *rcv = a.recv + f * a.recv_fs + B.face_off[1] * 6;
    GlobalSrc<TI, TC> ld{in + (int64_t)t * L, 1, a.io.ofs[f]};
    line_ends<FILT, TC>(C, L, B.ndf[0][1], B.ndf[1][1], rcv, nbs, jk, ld, sbs0, sbs1, sbs2, sbe0, sbe1, sbe2);
    a0 = ld(0); a1 = ld(1); a2 = ld(2); a3 = ld(3); a4 = ld(4); a5 = ld(5);
    if constexpr (UF) {
      f2 = fu[7] * sbs0;
      f1 = fu[FU_RT + 7] * sbs1 - fu[FU_RT + 1] * f2;
    } else {
      f2 = sbs0;
      f1 = sbs1 - fac[1 * 5 + 1] * f2;
    }
    w0 = f2; w1 = f1;
    const TC v = end_row(2, sbs2, f2, f1);
    w2 = v;
    f2 = f1; f1 = v;
  }
  // forward elimination, chunk by chunk
  const TI ofs = a.io.ofs[f];
  const int nch = (L + XC_C - 1) / XC_C;
  // asynchronous copies of chunk c of the CTA's lines of src into tile bf, one group
  auto issue = [&](const TC *src, int c, int bf) {
    const int c0 = c * XC_C, cl = min(XC_C, L - c0);
    if (lane < cl)
      for (int ln = warp; ln < nl; ln += NW)
        cp_async<sizeof(TC)>(&tile[bf][lane][ln], src + (int64_t)ln * L + c0 + lane);
    cp_async_commit();
  };
  if constexpr (AS) issue(reinterpret_cast<const TC *>(in), 0, 0);
  for (int c = 0; c < nch; c++) {
    const int c0 = c * XC_C, cl = min(XC_C, L - c0), bf = AS ? (c & 1) : 0;
    __syncthreads();  // the previous chunk's write-back has read the tile about to be refilled
    if constexpr (AS) {
      if (c + 1 < nch) {
        issue(reinterpret_cast<const TC *>(in), c + 1, (c + 1) & 1);
        cp_async_wait<1>();
      } else {
        cp_async_wait<0>();
      }
    } else if (lane < cl) {
      for (int ln = warp; ln < nl; ln += NW) tile[0][lane][ln] = cvt_in<TI, TC>(in[(int64_t)ln * L + c0 + lane], ofs);
    }
    __syncthreads();
    if (act) {
      int s0 = 0;
      if (c0 == 0) {  // fw(0..2) go to positions 3..5
        tile[bf][3][t] = w0; tile[bf][4][t] = w1; tile[bf][5][t] = w2;
        s0 = 6;
      }
      for (int s = s0; s < cl; s++) {
        const int i = c0 + s - 3;
        const TC a6 = tile[bf][s][t];
        TC v;
        if constexpr (UF) {
          const double *r = fu + i * FU_RT;
          TC sb;
          if (!FILT) {
            sb = r[2] * (a4 - a2) + r[3] * (a5 - a1) + r[4] * (a6 - a0);
          } else {
            sb = r[2] * (a2 + a4) + r[3] * (a1 + a5) + r[4] * (a0 + a6) - r[8] * a3;
          }
          v = sb - r[0] * f2 - r[1] * f1;
        } else {
          const TC sb = interior_rhs<FILT, TC>(C, a0, a1, a2, a3, a4, a5, a6);
          v = sb - fac[i * 5 + 0] * f2 - fac[i * 5 + 1] * f1;
        }
        tile[bf][s][t] = v;
        f2 = f1; f1 = v;
        a0 = a1; a1 = a2; a2 = a3; a3 = a4; a4 = a5; a5 = a6;
      }
    }
    __syncthreads();
    if (lane < cl)
      for (int ln = warp; ln < nl; ln += NW) fwg[(int64_t)ln * L + c0 + lane] = tile[bf][lane][ln];
  }
  // the last three rows and the first three results, in registers
  TC b0 = 0, b1 = 0;
  if (act) {
    TC v = end_row(L - 3, sbe2, f2, f1);
    const TC fwl3 = v;
    f2 = f1; f1 = v;
    v = end_row(L - 2, sbe1, f2, f1);
    f2 = f1; f1 = v;
    v = end_row(L - 1, sbe0, f2, f1);
    f2 = f1; f1 = v;
    TC r3;
    if constexpr (UF) {
      b0 = f1;
      b1 = f2 - fu[(L - 2) * FU_RT + 5] * b0;
      r3 = fwl3 - fu[(L - 3) * FU_RT + 5] * b1 - fu[(L - 3) * FU_RT + 6] * b0;
    } else {
      b0 = fac[(L - 1) * 5 + 2] * f1;
      b1 = fac[(L - 2) * 5 + 2] * f2 - fac[(L - 2) * 5 + 3] * b0;
      r3 = fac[(L - 3) * 5 + 2] * fwl3 - fac[(L - 3) * 5 + 3] * b1 - fac[(L - 3) * 5 + 4] * b0;
    }
    if (!FILT && a.io.drva) {
      TC *d = a.drva + B.face_off[1] * 10;
      d[jk + nbs * ((a.io.m0 + f - 1) + 5 * 1)] = b0;  // drva(jk,m,1) = sb(ie)
    }
    const int64_t o = (int64_t)t * L;
    const TC rv[3] = {r3, b1, b0};
#pragma unroll
    for (int q = 0; q < 3; q++) {
      const int64_t p = o + L - 3 + q;
      TO r;
      if (FILT) r = (TO)(in[p] + cvt<TI>(rv[q]));  // rr = rr + sb (src/Subroutines3D.f90:200-202)
      else r = (TO)rv[q];
      out[p] = r;
      if (out2) out2[p] = r;
    }
    b0 = b1; b1 = r3;
  }
  // back substitution, chunks in reverse: position j holds fw(j-3)
  __syncthreads();  // the forward pass's last write-back is complete and has read its tile
  if constexpr (AS) issue(fwg, nch - 1, 0);
  for (int r = 0; r < nch; r++) {
    const int c = nch - 1 - r, c0 = c * XC_C, cl = min(XC_C, L - c0), bf = AS ? (r & 1) : 0;
    __syncthreads();
    if constexpr (AS) {
      if (r + 1 < nch) {
        issue(fwg, c - 1, (r + 1) & 1);
        cp_async_wait<1>();
      } else {
        cp_async_wait<0>();
      }
    } else if (lane < cl) {
      for (int ln = warp; ln < nl; ln += NW) tile[0][lane][ln] = fwg[(int64_t)ln * L + c0 + lane];
    }
    __syncthreads();
    if (act) {
      const int se = c0 == 0 ? 3 : 0;
      for (int s = cl - 1; s >= se; s--) {
        const int i = c0 + s - 3;
        TC v;
        if constexpr (UF) v = tile[bf][s][t] - fu[i * FU_RT + 5] * b1 - fu[i * FU_RT + 6] * b0;
        else v = fac[i * 5 + 2] * tile[bf][s][t] - fac[i * 5 + 3] * b1 - fac[i * 5 + 4] * b0;
        tile[bf][s][t] = v;
        b0 = b1; b1 = v;
      }
    }
    __syncthreads();
    const int sw = c0 == 0 ? 3 : 0;
    if (lane < cl && lane >= sw) {
      auto wr = [&](int ln, TI qin) {
        const int64_t p = (int64_t)ln * L + c0 + lane - 3;
        const TC v = tile[bf][lane][ln];
        TO r;
        if (FILT) r = (TO)(qin + cvt<TI>(v));
        else r = (TO)v;
        out[p] = r;
        if (out2) out2[p] = r;
      };
      auto qin = [&](int ln) -> TI { return FILT ? in[(int64_t)ln * L + c0 + lane - 3] : (TI)0; };
      int ln = warp;
      // four lines a pass, their inputs read before any of them is stored (the filter runs in place)
      for (; ln + 3 * NW < nl; ln += 4 * NW) {
        const TI q0 = qin(ln), q1 = qin(ln + NW), q2 = qin(ln + 2 * NW), q3 = qin(ln + 3 * NW);
        wr(ln, q0);
        wr(ln + NW, q1);
        wr(ln + 2 * NW, q2);
        wr(ln + 3 * NW, q3);
      }
      for (; ln < nl; ln += NW) wr(ln, qin(ln));
    }
  }
  if (act && !FILT && a.io.drva) {
    TC *d = a.drva + B.face_off[1] * 10;
    d[jk + nbs * ((a.io.m0 + f - 1) + 5 * 0)] = b1;  // drva(jk,m,0) = sb(is)
  }
}

// ---------------------------------------------------------------------------
// Segmented line solves (mixed path, FP32 arithmetic).  A CTA takes SEG_LINES
// consecutive lines of one block and one field and stages them whole in
// shared memory as a [point][line] tile.  Each line is cut into S =
// seg_count(L) segments: warp w solves segment w, lane l line l.  The LU
// solve (src/Subroutines3D.f90:124-136) is linear, so a segment's forward
// values are its particular solution (zero incoming values) plus
// g(i) v(s0-2) + h(i) v(s0-1), where g and h, the responses to the incoming
// values, depend only on the LU factors that every line of the block shares.
// They come precomputed per row (FP64 on the host, rounded once; G and H are
// the same for the back substitution), packed with the row's LU factors.  One warp carries the incoming values
// from segment to segment (a 2x2 update per segment), then every segment adds
// its correction and back-substitutes the same way.  A thread's serial chain
// is L/S rows instead of L, and every line is read from and written to DRAM
// once, with no forward-value scratch.  The results differ from the
// sequential solve by rounding only, and depend on the line length alone.
// ---------------------------------------------------------------------------
// TMA (eta and zeta derivative sweeps over FP32 inputs, blocks whose geometry a tensor map can describe): the
// tile of each line group comes in as one tensor copy, [point][line] rows of SEG_LINES floats; eta tiles then
// hold lines of one grid row only (the work queue's eta tiles start at row starts and multiples of 32 points)
template <int NN, bool FILT, bool TMA, typename TI, typename TO>
__global__ void __launch_bounds__(SEG_LINES *SEG_MAX) k_sweep_seg(SweepArgs<TI, TO, float> a, const float *rtab,
                                                                  int groups) {
  static_assert(!TMA || (NN != 1 && std::is_same<TI, float>::value), "TMA staging: eta/zeta lines of FP32 inputs");
  extern __shared__ __align__(16) unsigned char seg_smem[];
  // tile row stride in words: with per-thread copies a warp writes a column (xi) or a row, so one word of padding
  // keeps both conflict-free; a TMA tile is dense (lanes read rows of 32 consecutive words, conflict-free)
  constexpr int RS = TMA ? SEG_LINES : SEG_LINES + 1;
  constexpr bool ASYNC = std::is_same<TI, float>::value;
  __shared__ uint64_t tbar[SEG_GROUPS];  // TMA completion, one barrier per line group
  const int nwarp = (int)(blockDim.x >> 5);
  const LTile LT = a.lt[blockIdx.x];
  const BlockDev &B = a.blk[LT.b];
  const int f = blockIdx.y;
  const int lane = (int)(threadIdx.x & 31), w = (int)(threadIdx.x >> 5);
  const int L = NN == 1 ? B.lxi + 1 : (NN == 2 ? B.let + 1 : B.lze + 1);
  // groups > 1 (every line of the launch one segment long): warp w solves its own group of SEG_LINES lines with
  // its own tile; otherwise the CTA is one group and warp w solves segment w of its lines
  const int gsz = groups > 1 ? 1 : nwarp, grp = w / gsz, wl = w - grp * gsz;
  const int t0 = LT.t0 + grp * SEG_LINES;
  // lines of the group (none: the group idles, as on a padding tile past the block's lines); an eta tile built
  // for TMA ends with its grid row
  const int nx = B.lxi + 1;
  const int nl = LT.t0 >= B.nbsize[NN] ? 0
                 : (NN == 2 && a.rowtiles) ? min(SEG_LINES, nx - LT.t0 % nx - grp * SEG_LINES)
                                           : min(SEG_LINES, (int)B.nbsize[NN] - t0);
  // shared memory: the groups' tiles (TMA: first, 128-byte aligned), then the segment carries
  float *tiles;
  if constexpr (TMA) {
    const uint32_t pad = (128u - (smem_u32(seg_smem) & 127u)) & 127u;
    tiles = reinterpret_cast<float *>(seg_smem + pad);
  } else {
    tiles = reinterpret_cast<float *>(seg_smem + (size_t)nwarp * SEG_LINES * 2 * sizeof(float2));
  }
  const int ngrp = groups > 1 ? groups : 1;
  float2 *cf = TMA ? reinterpret_cast<float2 *>(tiles + (int64_t)ngrp * L * RS)
                   : reinterpret_cast<float2 *>(seg_smem);  // [segment][line] values a segment passes on
  float2 *cx = cf + nwarp * SEG_LINES;                       // [segment][line] values a segment receives
  float *tile = tiles + (int64_t)grp * L * RS;
  int64_t base = 0, stride = 1;
  int jk = 0, Lg = 0;
  line_geom<NN>(B, t0 + lane, base, stride, jk, Lg);
  const TI *in = a.io.in + f * a.io.in_fs;
  const TI ofs = a.io.ofs[f];

  // 1. stage the lines (inputs wider than FP32 lose their offset and are rounded on the way in);
  // source and destination pointers walk by constant steps
  bool tma_ok = true;
  if constexpr (TMA) {
    if (threadIdx.x == 0) {
      for (int q = 0; q < ngrp; q++) mbar_init(&tbar[q], 1);
      fence_mbar_init();
    }
    __syncthreads();
    if (nl > 0) {
      if (wl == 0 && lane == 0) {
        const TmaMap *tm = a.tmap + LT.b;
        tmap_acquire(tm);
        mbar_expect_tx(&tbar[grp], (uint32_t)(L * SEG_LINES * sizeof(float)));
        if constexpr (NN == 2) tma_load_4d(tile, tm, LT.t0 % nx + grp * SEG_LINES, 0, LT.t0 / nx, f, &tbar[grp]);
        else tma_load_3d(tile, tm, t0, 0, f, &tbar[grp]);
      }
      tma_ok = mbar_wait_bounded(&tbar[grp], 0);
      if (!tma_ok && lane == 0) atomicOr(&a.scal[B.cs].flag, FLAG_TIMEOUT);
    }
  }
  auto stage = [&](float *dst, const TI *src) {
    if constexpr (ASYNC) cp_async<4>(dst, src);
    else *dst = cvt_in<TI, float>(__ldg(src), ofs);
  };
  if constexpr (TMA) {
    // (staged by the tensor copy above)
  } else if constexpr (NN == 1) {
    // xi lines are contiguous: a warp copies one line at a time, lanes along the line
    const TI *src0 = in + B.off + (int64_t)t0 * L;
    for (int ln = wl; ln < nl; ln += gsz) {
      const TI *src = src0 + (int64_t)ln * L + lane;
      float *dst = tile + lane * RS + ln;
#pragma unroll 4
      for (int i = lane; i < L; i += 32, src += 32, dst += 32 * RS) stage(dst, src);
    }
  } else {
    // consecutive eta/zeta lines are consecutive points of a row: a warp copies one row at a time
    if (lane < nl) {
      const TI *src = in + base + (int64_t)wl * stride;
      const int64_t step = (int64_t)gsz * stride;
      float *dst = tile + wl * RS + lane;
#pragma unroll 4
      for (int i = wl; i < L; i += gsz, src += step, dst += gsz * RS) stage(dst, src);
    }
  }
  if constexpr (ASYNC) {
    cp_async_commit();
    cp_async_wait<0>();
  }
  __syncthreads();

  const int S = seg_count(L);
  const bool act = wl < S && lane < nl && tma_ok;  // (a group whose tile never landed computes nothing)
  const int s0 = seg_start(wl, L, S), s1 = seg_start(wl + 1, L, S);
  float *col = tile + lane;
  // the block's row table, SEG_RT floats per row (layout at SEG_RT)
  const float *rt = rtab + (int64_t)B.fac_off[NN] * SEG_RT;
  auto row = [&](int i) { return rt + i * SEG_RT; };
  // interior stencil weights in registers (loads from the coefficient struct could not move past the stores)
  const Coef<float> &C = *a.cf;
  const float k1 = FILT ? C.fa : C.aa, k2 = FILT ? C.fb : C.ab, k3 = FILT ? C.fc : C.ac;
  auto rhs = [&](float x0, float x1, float x2, float x3, float x4, float x5, float x6) {
    if (!FILT) return k1 * (x4 - x2) + k2 * (x5 - x1) + k3 * (x6 - x0);
    const float r = 2.f * x3;
    return k1 * (x2 + x4 - r) + k2 * (x1 + x5 - r) + k3 * (x0 + x6 - r);
  };
  const int ilo = max(s0, 3), ihi = min(s1, L - 3);  // interior rows [ilo, ihi) of the segment
  // 2. what a segment reads outside its own rows, before any row is overwritten:
  // the boundary-closure rows, the first window and the three rows after it
  float sbs0 = 0, sbs1 = 0, sbs2 = 0, sbe0 = 0, sbe1 = 0, sbe2 = 0;
  float a0 = 0, a1 = 0, a2 = 0, a3 = 0, a4 = 0, a5 = 0, h0 = 0, h1 = 0, h2 = 0;
  if (act) {
    auto sld = [&](int i) { return col[i * RS]; };
    if (wl == 0 || wl == S - 1) {
      // the closure values of the line ends (what mpigo leaves in recv).  In a derivative, a face periodic onto
      // its own block (BC 45 with the block as neighbour) takes them from the other end of the same line, which
      // is staged: the sums of k_mpigo (src/Subroutines3D.f90:16-80) in its operation order, skipping the shared
      // point.  (The filter's closures come from the state before its first direction, src/Main3D.f90:555-561,
      // so a filter sweep, which sees the state after the earlier directions, reads them from recv.)
      const float *rcv = a.recv + f * a.recv_fs + B.face_off[NN] * 6;
      const int64_t nbs = B.nbsize[NN];
      constexpr int nt = FILT ? 1 : 0, mp = FILT ? LMF : LMD;
      auto closure = [&](int r0, int dir, float *o) {
        float c0 = 0, c1 = 0, sap0 = 0;
        for (int i = 0; i <= mp; i++) {
          const float v = sld(r0 + i * dir);
          if (i == 0) sap0 = v;
          c0 += C.pbco[nt][0][i] * v;
          c1 += C.pbco[nt][1][i] * v;
        }
        o[0] = c0; o[1] = c1; o[2] = sap0;
      };
      float rl[6];
      for (int ip = 0; ip <= 1; ip++) {
        if (B.ndf[ip][NN] != 1) continue;
        if (!FILT && B.nbc[ip][NN] == 45 && B.ncd[ip][NN] == LT.b) closure(ip == 0 ? L - 2 : 1, ip == 0 ? -1 : 1, rl + 3 * ip);
        else for (int q = 0; q < 3; q++) rl[3 * ip + q] = rcv[jk + nbs * (3 * ip + q)];
      }
      line_ends<FILT, float>(C, L, B.ndf[0][NN], B.ndf[1][NN], rl, 1, 0, sld, sbs0, sbs1, sbs2, sbe0, sbe1, sbe2);
    }
    if (ilo < ihi) {
      a0 = sld(ilo - 3); a1 = sld(ilo - 2); a2 = sld(ilo - 1); a3 = sld(ilo); a4 = sld(ilo + 1); a5 = sld(ilo + 2);
    }
    if (wl < S - 1) { h0 = sld(s1); h1 = sld(s1 + 1); h2 = sld(s1 + 2); }
  }
  __syncthreads();

  // 3. forward elimination of the segment from zero incoming values (the particular solution), in place
  float pm2 = 0, pm1 = 0;
  if (act) {
    auto fwd = [&](int i, float r) {
      const float2 l = __ldg(reinterpret_cast<const float2 *>(row(i)));  // masked l0, l1
      const float p = r - l.x * pm2 - l.y * pm1;
      col[i * RS] = p;
      pm2 = pm1; pm1 = p;
    };
    int i = s0;
    for (; i < min(s1, 3); i++) fwd(i, i == 0 ? sbs0 : (i == 1 ? sbs1 : sbs2));
    const int iown = min(ihi, s1 - 3);  // windows inside the segment
    {
      // four rows per pass, walking a shared and a table pointer: the loop body is
      // the arithmetic itself (the loads of a pass come before its stores)
      float *pc = col + i * RS;
      const float *tr = row(i);
      auto l2 = [](const float *t) { return __ldg(reinterpret_cast<const float2 *>(t)); };
      // each pass loads the next pass's factors first (rows past the block read the table's padding)
      float2 m0 = l2(tr), m1 = l2(tr + SEG_RT), m2 = l2(tr + 2 * SEG_RT), m3 = l2(tr + 3 * SEG_RT);
      for (; i + 3 < iown; i += 4, pc += 4 * RS, tr += 4 * SEG_RT) {
        const float b0 = pc[3 * RS], b1 = pc[4 * RS], b2 = pc[5 * RS], b3 = pc[6 * RS];
        const float2 n0 = l2(tr + 4 * SEG_RT), n1 = l2(tr + 5 * SEG_RT), n2 = l2(tr + 6 * SEG_RT);
        const float2 n3 = l2(tr + 7 * SEG_RT);
        float p;
        p = rhs(a0, a1, a2, a3, a4, a5, b0) - m0.x * pm2 - m0.y * pm1; pc[0] = p; pm2 = pm1; pm1 = p;
        p = rhs(a1, a2, a3, a4, a5, b0, b1) - m1.x * pm2 - m1.y * pm1; pc[RS] = p; pm2 = pm1; pm1 = p;
        p = rhs(a2, a3, a4, a5, b0, b1, b2) - m2.x * pm2 - m2.y * pm1; pc[2 * RS] = p; pm2 = pm1; pm1 = p;
        p = rhs(a3, a4, a5, b0, b1, b2, b3) - m3.x * pm2 - m3.y * pm1; pc[3 * RS] = p; pm2 = pm1; pm1 = p;
        a0 = a4; a1 = a5; a2 = b0; a3 = b1; a4 = b2; a5 = b3;
        m0 = n0; m1 = n1; m2 = n2; m3 = n3;
      }
    }
    for (; i < iown; i++) {
      const float a6 = col[(i + 3) * RS];
      fwd(i, rhs(a0, a1, a2, a3, a4, a5, a6));
      a0 = a1; a1 = a2; a2 = a3; a3 = a4; a4 = a5; a5 = a6;
    }
    for (; i < ihi; i++) {  // windows reaching into the next segment: its first rows, read before the barrier
      const int d = i + 3 - s1;
      const float a6 = d == 0 ? h0 : (d == 1 ? h1 : h2);
      fwd(i, rhs(a0, a1, a2, a3, a4, a5, a6));
      a0 = a1; a1 = a2; a2 = a3; a3 = a4; a4 = a5; a5 = a6;
    }
    for (; i < s1; i++) fwd(i, i == L - 1 ? sbe0 : (i == L - 2 ? sbe1 : sbe2));
    cf[w * SEG_LINES + lane] = make_float2(pm2, pm1);  // rows s1-2, s1-1
  }
  // lines of one segment (S = 1, the same for the whole CTA) need neither carries nor corrections
  const bool multi = S > 1;
  if (multi) {
    __syncthreads();
    // 4. incoming values of every segment, carried by warp 0 (segment 0 receives zeros)
    if (w == 0 && lane < nl) {
      float2 x = make_float2(0.f, 0.f);
      cx[lane] = x;
      for (int k = 1; k < S; k++) {
        const int e = seg_start(k, L, S);
        const float2 c = cf[(k - 1) * SEG_LINES + lane];
        const float2 t2 = __ldg(reinterpret_cast<const float2 *>(row(e - 2) + 4));  // g, h
        const float2 t1 = __ldg(reinterpret_cast<const float2 *>(row(e - 1) + 4));
        x = make_float2(c.x + t2.x * x.x + t2.y * x.y, c.y + t1.x * x.x + t1.y * x.y);
        cx[k * SEG_LINES + lane] = x;
      }
    }
    __syncthreads();
  }
  TO *out = a.io.out + f * a.io.out_fs;
  TO *out2 = FILT && a.io.out2 ? a.io.out2 + f * a.io.out_fs : nullptr;  // (a derivative has one output)
  float *drv = (!FILT && a.io.drva) ? a.drva + B.face_off[NN] * 10 : nullptr;
  const int64_t nbs = B.nbsize[NN];
  const int m = a.io.m0 + f;
  // 5. the segment's forward values, then its back substitution from zero values beyond its end; with one
  // segment that gives the results, which eta/zeta lines write straight to DRAM (a warp writes a row)
  if (act) {
    const float2 x = multi ? cx[w * SEG_LINES + lane] : make_float2(0.f, 0.f);
    float q1 = 0, q2 = 0;  // rows i+1, i+2
    int i = s1 - 1;
    float *pc = col + i * RS;
    const float *tr = row(i);
    const int64_t o = base + (int64_t)i * stride;
    TO *po = out + o;
    TO *po2 = out2 ? out2 + o : nullptr;
    const TI *pi = in + o;
    auto sweep = [&](auto direct) {
      constexpr bool D = decltype(direct)::value;
      // one row: g = (g, h, c2, masked c3) and the masked c4 of the row, loaded a pass ahead
      auto l4 = [](const float *t) { return __ldg(reinterpret_cast<const float4 *>(t + 4)); };
      auto l1 = [](const float *t) { return __ldg(t + 10); };
      auto bwd = [&](float *c, const float4 g, const float c4) {
        const float v = *c + g.x * x.x + g.y * x.y;
        const float q = g.z * v - g.w * q1 - c4 * q2;
        if constexpr (D) {
          TO r;
          if (FILT) r = (TO)(*pi + cvt<TI>(q));  // rr = rr + sb (src/Subroutines3D.f90:200-202)
          else r = (TO)q;
          *po = r;
          po -= stride;
          if (out2) { *po2 = r; po2 -= stride; }
          if (FILT) pi -= stride;
        } else {
          *c = q;
        }
        q2 = q1; q1 = q;
      };
      float4 g0 = l4(tr), g1 = l4(tr - SEG_RT), g2 = l4(tr - 2 * SEG_RT), g3 = l4(tr - 3 * SEG_RT);
      float k0 = l1(tr), k1 = l1(tr - SEG_RT), k2 = l1(tr - 2 * SEG_RT), k3 = l1(tr - 3 * SEG_RT);
      for (; i - 3 >= s0; i -= 4, pc -= 4 * RS, tr -= 4 * SEG_RT) {
        // the next pass's rows (rows before the block read the table's padding)
        const float4 h0 = l4(tr - 4 * SEG_RT), h1 = l4(tr - 5 * SEG_RT), h2 = l4(tr - 6 * SEG_RT);
        const float4 h3 = l4(tr - 7 * SEG_RT);
        const float j0 = l1(tr - 4 * SEG_RT), j1 = l1(tr - 5 * SEG_RT), j2 = l1(tr - 6 * SEG_RT);
        const float j3 = l1(tr - 7 * SEG_RT);
        bwd(pc, g0, k0);
        bwd(pc - RS, g1, k1);
        bwd(pc - 2 * RS, g2, k2);
        bwd(pc - 3 * RS, g3, k3);
        g0 = h0; g1 = h1; g2 = h2; g3 = h3;
        k0 = j0; k1 = j1; k2 = j2; k3 = j3;
      }
      for (; i >= s0; i--, pc -= RS, tr -= SEG_RT) bwd(pc, l4(tr), l1(tr));
    };
    if (!multi && NN != 1) {
      sweep(std::true_type{});
      if (drv) {
        drv[jk + nbs * ((m - 1) + 5 * 0)] = q1;  // drva(jk,m,0) = sb(is): row 0, the last one solved
        drv[jk + nbs * ((m - 1) + 5 * 1)] = (float)out[base + (int64_t)(L - 1) * stride];  // drva(jk,m,1) = sb(ie)
      }
    } else {
      sweep(std::false_type{});
      if (multi) cf[w * SEG_LINES + lane] = make_float2(q1, q2);  // rows s0, s0+1
      else if (drv) {
        drv[jk + nbs * ((m - 1) + 5 * 0)] = col[0];
        drv[jk + nbs * ((m - 1) + 5 * 1)] = col[(L - 1) * RS];
      }
    }
  }
  if (multi) {
    __syncthreads();
    // 6. values beyond every segment's end, carried backwards by warp 0 (the last segment receives zeros)
    if (w == 0 && lane < nl) {
      float2 y = make_float2(0.f, 0.f);
      cx[(S - 1) * SEG_LINES + lane] = y;
      for (int k = S - 2; k >= 0; k--) {
        const int e = seg_start(k + 1, L, S);
        const float2 c = cf[(k + 1) * SEG_LINES + lane];
        const float2 t0 = __ldg(reinterpret_cast<const float2 *>(row(e) + 8));  // G, H
        const float2 t1 = __ldg(reinterpret_cast<const float2 *>(row(e + 1) + 8));
        y = make_float2(c.x + t0.x * y.x + t0.y * y.y, c.y + t1.x * y.x + t1.y * y.y);
        cx[k * SEG_LINES + lane] = y;
      }
    }
    __syncthreads();
    // 7. results: eta/zeta rows go straight to DRAM (a warp writes a contiguous row), xi lines through the tile
    if (act) {
      const float2 y = cx[w * SEG_LINES + lane];
      auto fv = [&](const float *c, const float *t) {
        const float2 g = __ldg(reinterpret_cast<const float2 *>(t));
        return *c + g.x * y.x + g.y * y.y;
      };
      auto fg = [&](const float *c, const float2 g) { return *c + g.x * y.x + g.y * y.y; };
      auto l2 = [](const float *t) { return __ldg(reinterpret_cast<const float2 *>(t)); };
      if (drv) {
        if (wl == 0) drv[jk + nbs * ((m - 1) + 5 * 0)] = fv(col, row(0) + 8);  // drva(jk,m,0) = sb(is)
        if (wl == S - 1) drv[jk + nbs * ((m - 1) + 5 * 1)] = fv(col + (L - 1) * RS, row(L - 1) + 8);
      }
      int i = s0;
      float *pc = col + i * RS;
      const float *tr = row(i) + 8;
      float2 e0 = l2(tr), e1 = l2(tr + SEG_RT), e2 = l2(tr + 2 * SEG_RT), e3 = l2(tr + 3 * SEG_RT);
      if constexpr (NN == 1) {
        for (; i + 3 < s1; i += 4, pc += 4 * RS, tr += 4 * SEG_RT) {
          const float2 f0 = l2(tr + 4 * SEG_RT), f1 = l2(tr + 5 * SEG_RT), f2 = l2(tr + 6 * SEG_RT);
          const float2 f3 = l2(tr + 7 * SEG_RT);
          const float r0 = fg(pc, e0), r1 = fg(pc + RS, e1), r2 = fg(pc + 2 * RS, e2), r3 = fg(pc + 3 * RS, e3);
          pc[0] = r0; pc[RS] = r1; pc[2 * RS] = r2; pc[3 * RS] = r3;
          e0 = f0; e1 = f1; e2 = f2; e3 = f3;
        }
        for (; i < s1; i++, pc += RS, tr += SEG_RT) *pc = fv(pc, tr);
      } else {
        // a walking output pointer: one 64-bit add per row
        const int64_t o = base + (int64_t)i * stride;
        TO *po = out + o;
        TO *po2 = out2 ? out2 + o : nullptr;
        const TI *pi = in + o;
        auto put = [&](float v) {
          TO r;
          if (FILT) r = (TO)(*pi + cvt<TI>(v));  // rr = rr + sb (src/Subroutines3D.f90:200-202)
          else r = (TO)v;
          *po = r;
          po += stride;
          if (out2) { *po2 = r; po2 += stride; }
          if (FILT) pi += stride;
        };
        for (; i + 3 < s1; i += 4, pc += 4 * RS, tr += 4 * SEG_RT) {
          const float2 f0 = l2(tr + 4 * SEG_RT), f1 = l2(tr + 5 * SEG_RT), f2 = l2(tr + 6 * SEG_RT);
          const float2 f3 = l2(tr + 7 * SEG_RT);
          const float r0 = fg(pc, e0), r1 = fg(pc + RS, e1), r2 = fg(pc + 2 * RS, e2), r3 = fg(pc + 3 * RS, e3);
          put(r0); put(r1); put(r2); put(r3);
          e0 = f0; e1 = f1; e2 = f2; e3 = f3;
        }
        for (; i < s1; i++, pc += RS, tr += SEG_RT) put(fv(pc, tr));
      }
    }
  }
  if constexpr (NN == 1) {
    __syncthreads();
    const int64_t o0 = B.off + (int64_t)t0 * L;
    auto wr = [&](int64_t p, float v, TI qin) {
      TO r;
      if (FILT) r = (TO)(qin + cvt<TI>(v));  // rr = rr + sb (src/Subroutines3D.f90:200-202)
      else r = (TO)v;
      out[p] = r;
      if (out2) out2[p] = r;
    };
    for (int ln = wl; ln < nl; ln += gsz) {
      const int64_t lb = o0 + (int64_t)ln * L;
      int i = lane;
      // four points a pass, their inputs read before any of them is stored (the filter runs in place)
      for (; i + 96 < L; i += 128) {
        TI q0 = 0, q1 = 0, q2 = 0, q3 = 0;
        if (FILT) { q0 = in[lb + i]; q1 = in[lb + i + 32]; q2 = in[lb + i + 64]; q3 = in[lb + i + 96]; }
        wr(lb + i, tile[i * RS + ln], q0);
        wr(lb + i + 32, tile[(i + 32) * RS + ln], q1);
        wr(lb + i + 64, tile[(i + 64) * RS + ln], q2);
        wr(lb + i + 96, tile[(i + 96) * RS + ln], q3);
      }
      for (; i < L; i += 32) wr(lb + i, tile[i * RS + ln], FILT ? in[lb + i] : (TI)0);
    }
  }
  if constexpr (TMA) {
    // a tile copy that did not land in time: wait once more (bounded) so that no copy into this CTA's shared
    // memory is left in flight when it exits
    if (!tma_ok) (void)mbar_wait_bounded(&tbar[grp], 0);
  }
}

// ---------------------------------------------------------------------------
// Paired segmented derivative solves (mixed path, FP32 inputs and outputs).  A
// CTA takes two consecutive groups of SEG_LINES lines (two halves) of one block,
// and lane l solves line l of both: the row-table loads, the loop and address
// arithmetic and the segment carries' control flow are spent once for two
// lines.  Each line's arithmetic is that of k_sweep_seg, expression for
// expression, so both kernels give the same results.
//   single != 0: the lines are one segment long; the CTA (one warp) takes the
//     tile of 2 SEG_LINES lines at lt[blockIdx.x].
//   single == 0: the CTA (one warp per segment) takes the tiles at
//     lt[2 blockIdx.x] and the one after it: the host pads every block's run of
//     tiles (every grid row's, for eta row tiles) to an even count, so the two
//     are consecutive lines and the padding tile lies past the run's lines.
// The halves' tiles lie one after the other in shared memory ([point][line]
// rows, as in k_sweep_seg); with TMA each half comes in as one tensor copy, both
// counted on one mbarrier.
// ---------------------------------------------------------------------------
// ADJ: the second half's line l lies SEG_LINES points after the first half's (zeta lines, and eta lines in row
// tiles): its results are stored at a fixed offset from the first half's, through one walking pointer.
template <int NN, bool TMA, bool ADJ>
__global__ void __launch_bounds__(SEG_LINES *SEG_MAX) k_sweep_pair(SweepArgs<float, float, float> a, const float *rtab,
                                                                   int single) {
  static_assert(!ADJ || NN != 1, "adjacent halves: eta/zeta lines");
  extern __shared__ __align__(16) unsigned char seg_smem[];
  constexpr int RS = TMA ? SEG_LINES : SEG_LINES + 1;
  __shared__ uint64_t tbar;
  const int nwarp = (int)(blockDim.x >> 5);
  const LTile LT = a.lt[single ? blockIdx.x : 2 * blockIdx.x];
  const BlockDev &B = a.blk[LT.b];
  const int f = blockIdx.y;
  const int lane = (int)(threadIdx.x & 31), w = (int)(threadIdx.x >> 5);
  const int nx = B.lxi + 1, ny = B.let + 1;
  const int L = NN == 1 ? nx : (NN == 2 ? ny : B.lze + 1);
  const int T0 = LT.t0;
  const int64_t nbs = B.nbsize[NN];
  // lines of each half (none past the block's lines or, for eta row tiles, past the grid row)
  const int lim = T0 >= nbs ? 0 : ((NN == 2 && a.rowtiles) ? nx - T0 % nx : (int)(nbs - T0));
  const int nl0 = max(0, min(SEG_LINES, lim)), nl1 = max(0, min(SEG_LINES, lim - SEG_LINES));
  const int HS = L * RS;  // offset of the second half's tile
  float *tiles;
  if constexpr (TMA) {
    const uint32_t pad = (128u - (smem_u32(seg_smem) & 127u)) & 127u;
    tiles = reinterpret_cast<float *>(seg_smem + pad);
  } else {
    tiles = reinterpret_cast<float *>(seg_smem + (size_t)nwarp * SEG_LINES * 2 * sizeof(float4));
  }
  // [segment][lane] values a segment passes on / receives, both halves' lines in one float4
  float4 *cf = TMA ? reinterpret_cast<float4 *>(tiles + 2 * (int64_t)HS) : reinterpret_cast<float4 *>(seg_smem);
  float4 *cx = cf + nwarp * SEG_LINES;
  const int64_t stride = NN == 1 ? 1 : (NN == 2 ? (int64_t)nx : (int64_t)nx * ny);
  int64_t base0 = 0, base1 = 0, sdum = 0;
  int jk0 = 0, jk1 = 0, Lg = 0;
  line_geom<NN>(B, T0 + lane, base0, sdum, jk0, Lg);
  line_geom<NN>(B, T0 + SEG_LINES + lane, base1, sdum, jk1, Lg);
  const float *in = a.io.in + f * a.io.in_fs;

  // 1. stage both halves
  bool tma_ok = true;
  if constexpr (TMA) {
    if (threadIdx.x == 0) {
      mbar_init(&tbar, 1);
      fence_mbar_init();
    }
    __syncthreads();
    if (nl0 > 0) {
      if (threadIdx.x == 0) {
        const TmaMap *tm = a.tmap + LT.b;
        tmap_acquire(tm);
        mbar_expect_tx(&tbar, (uint32_t)(L * SEG_LINES * sizeof(float)) * (nl1 > 0 ? 2u : 1u));
        for (int hh = 0; hh < 2; hh++) {
          if (hh == 1 && nl1 == 0) break;
          const int t0 = T0 + hh * SEG_LINES;
          if constexpr (NN == 2) tma_load_4d(tiles + hh * HS, tm, t0 % nx, 0, t0 / nx, f, &tbar);
          else tma_load_3d(tiles + hh * HS, tm, t0, 0, f, &tbar);
        }
      }
      tma_ok = mbar_wait_bounded(&tbar, 0);
      if (!tma_ok && lane == 0) atomicOr(&a.scal[B.cs].flag, FLAG_TIMEOUT);
    }
  } else {
#pragma unroll
    for (int hh = 0; hh < 2; hh++) {
      const int nl = hh ? nl1 : nl0;
      float *tile = tiles + hh * HS;
      if constexpr (NN == 1) {
        // xi lines are contiguous: a warp copies one line at a time, lanes along the line
        const float *src0 = in + B.off + (int64_t)(T0 + hh * SEG_LINES) * L;
        for (int ln = w; ln < nl; ln += nwarp) {
          const float *src = src0 + (int64_t)ln * L + lane;
          float *dst = tile + lane * RS + ln;
#pragma unroll 4
          for (int i = lane; i < L; i += 32, src += 32, dst += 32 * RS) cp_async<4>(dst, src);
        }
      } else if (lane < nl) {
        // consecutive eta/zeta lines are consecutive points of a row: a warp copies one row at a time
        const float *src = in + (hh ? base1 : base0) + (int64_t)w * stride;
        float *dst = tile + w * RS + lane;
#pragma unroll 4
        for (int i = w; i < L; i += nwarp, src += nwarp * stride, dst += nwarp * RS) cp_async<4>(dst, src);
      }
    }
    cp_async_commit();
    cp_async_wait<0>();
  }
  __syncthreads();

  const int S = seg_count(L);
  // (half 1's lines of a lane are a subset of half 0's: lane < nl1 implies lane < nl0)
  const bool act0 = w < S && lane < nl0 && tma_ok, act1 = w < S && lane < nl1 && tma_ok;
  const bool act = act0;
  const int s0 = seg_start(w, L, S), s1 = seg_start(w + 1, L, S);
  float *col = tiles + lane;  // half 0; half 1 at col + HS
  const float *rt = rtab + (int64_t)B.fac_off[NN] * SEG_RT;
  auto row = [&](int i) { return rt + i * SEG_RT; };
  const Coef<float> &C = *a.cf;
  const float k1 = C.aa, k2 = C.ab, k3 = C.ac;
  auto rhs = [&](float x0, float x1, float x2, float x3, float x4, float x5, float x6) {
    return k1 * (x4 - x2) + k2 * (x5 - x1) + k3 * (x6 - x0);
  };
  const int ilo = max(s0, 3), ihi = min(s1, L - 3);
  // 2. what a segment reads outside its own rows, before any row is overwritten (per half, as in k_sweep_seg)
  float sbs0[2] = {0, 0}, sbs1[2] = {0, 0}, sbs2[2] = {0, 0}, sbe0[2] = {0, 0}, sbe1[2] = {0, 0}, sbe2[2] = {0, 0};
  float a0[2] = {0, 0}, a1[2] = {0, 0}, a2[2] = {0, 0}, a3[2] = {0, 0}, a4[2] = {0, 0}, a5[2] = {0, 0};
  float h0[2] = {0, 0}, h1[2] = {0, 0}, h2[2] = {0, 0};
  if (act) {
#pragma unroll
    for (int hh = 0; hh < 2; hh++) {
      const float *ch = col + hh * HS;
      auto sld = [&](int i) { return ch[i * RS]; };
      if ((hh == 0 || act1) && (w == 0 || w == S - 1)) {
        const int jk = hh ? jk1 : jk0;
        const float *rcv = a.recv + f * a.recv_fs + B.face_off[NN] * 6;
        auto closure = [&](int r0, int dir, float *o) {
          float c0 = 0, c1 = 0, sap0 = 0;
          for (int i = 0; i <= LMD; i++) {
            const float v = sld(r0 + i * dir);
            if (i == 0) sap0 = v;
            c0 += C.pbco[0][0][i] * v;
            c1 += C.pbco[0][1][i] * v;
          }
          o[0] = c0; o[1] = c1; o[2] = sap0;
        };
        float rl[6];
        for (int ip = 0; ip <= 1; ip++) {
          if (B.ndf[ip][NN] != 1) continue;
          if (B.nbc[ip][NN] == 45 && B.ncd[ip][NN] == LT.b) closure(ip == 0 ? L - 2 : 1, ip == 0 ? -1 : 1, rl + 3 * ip);
          else for (int q = 0; q < 3; q++) rl[3 * ip + q] = rcv[jk + nbs * (3 * ip + q)];
        }
        line_ends<false, float>(C, L, B.ndf[0][NN], B.ndf[1][NN], rl, 1, 0, sld, sbs0[hh], sbs1[hh], sbs2[hh],
                                sbe0[hh], sbe1[hh], sbe2[hh]);
      }
      if (ilo < ihi) {
        a0[hh] = sld(ilo - 3); a1[hh] = sld(ilo - 2); a2[hh] = sld(ilo - 1);
        a3[hh] = sld(ilo); a4[hh] = sld(ilo + 1); a5[hh] = sld(ilo + 2);
      }
      if (w < S - 1) { h0[hh] = sld(s1); h1[hh] = sld(s1 + 1); h2[hh] = sld(s1 + 2); }
    }
  }
  __syncthreads();

  // 3. forward elimination of the segment from zero incoming values, in place, both halves
  float pm2[2] = {0, 0}, pm1[2] = {0, 0};
  if (act) {
    auto fwd = [&](int i, float r0, float r1) {
      const float2 l = __ldg(reinterpret_cast<const float2 *>(row(i)));  // masked l0, l1
      const float p0 = r0 - l.x * pm2[0] - l.y * pm1[0];
      const float p1 = r1 - l.x * pm2[1] - l.y * pm1[1];
      col[i * RS] = p0;
      col[HS + i * RS] = p1;
      pm2[0] = pm1[0]; pm1[0] = p0;
      pm2[1] = pm1[1]; pm1[1] = p1;
    };
    int i = s0;
    for (; i < min(s1, 3); i++) {
      const float r0 = i == 0 ? sbs0[0] : (i == 1 ? sbs1[0] : sbs2[0]);
      const float r1 = i == 0 ? sbs0[1] : (i == 1 ? sbs1[1] : sbs2[1]);
      fwd(i, r0, r1);
    }
    const int iown = min(ihi, s1 - 3);
    {
      float *pc = col + i * RS;
      const float *tr = row(i);
      auto l2 = [](const float *t) { return __ldg(reinterpret_cast<const float2 *>(t)); };
      float2 m0 = l2(tr), m1 = l2(tr + SEG_RT), m2 = l2(tr + 2 * SEG_RT), m3 = l2(tr + 3 * SEG_RT);
      for (; i + 3 < iown; i += 4, pc += 4 * RS, tr += 4 * SEG_RT) {
        float b0[2], b1[2], b2[2], b3[2];
#pragma unroll
        for (int hh = 0; hh < 2; hh++) {
          const float *q = pc + hh * HS;
          b0[hh] = q[3 * RS]; b1[hh] = q[4 * RS]; b2[hh] = q[5 * RS]; b3[hh] = q[6 * RS];
        }
        const float2 n0 = l2(tr + 4 * SEG_RT), n1 = l2(tr + 5 * SEG_RT), n2 = l2(tr + 6 * SEG_RT);
        const float2 n3 = l2(tr + 7 * SEG_RT);
#pragma unroll
        for (int hh = 0; hh < 2; hh++) {
          float *q = pc + hh * HS;
          float p, &pa = pm2[hh], &pb = pm1[hh];
          p = rhs(a0[hh], a1[hh], a2[hh], a3[hh], a4[hh], a5[hh], b0[hh]) - m0.x * pa - m0.y * pb; q[0] = p; pa = pb; pb = p;
          p = rhs(a1[hh], a2[hh], a3[hh], a4[hh], a5[hh], b0[hh], b1[hh]) - m1.x * pa - m1.y * pb; q[RS] = p; pa = pb; pb = p;
          p = rhs(a2[hh], a3[hh], a4[hh], a5[hh], b0[hh], b1[hh], b2[hh]) - m2.x * pa - m2.y * pb; q[2 * RS] = p; pa = pb; pb = p;
          p = rhs(a3[hh], a4[hh], a5[hh], b0[hh], b1[hh], b2[hh], b3[hh]) - m3.x * pa - m3.y * pb; q[3 * RS] = p; pa = pb; pb = p;
          a0[hh] = a4[hh]; a1[hh] = a5[hh]; a2[hh] = b0[hh]; a3[hh] = b1[hh]; a4[hh] = b2[hh]; a5[hh] = b3[hh];
        }
        m0 = n0; m1 = n1; m2 = n2; m3 = n3;
      }
    }
    auto shift = [&](const float *a6) {
#pragma unroll
      for (int hh = 0; hh < 2; hh++) {
        a0[hh] = a1[hh]; a1[hh] = a2[hh]; a2[hh] = a3[hh]; a3[hh] = a4[hh]; a4[hh] = a5[hh]; a5[hh] = a6[hh];
      }
    };
    for (; i < iown; i++) {
      const float a6[2] = {col[(i + 3) * RS], col[HS + (i + 3) * RS]};
      fwd(i, rhs(a0[0], a1[0], a2[0], a3[0], a4[0], a5[0], a6[0]), rhs(a0[1], a1[1], a2[1], a3[1], a4[1], a5[1], a6[1]));
      shift(a6);
    }
    for (; i < ihi; i++) {  // windows reaching into the next segment: its first rows, read before the barrier
      const int d = i + 3 - s1;
      const float a6[2] = {d == 0 ? h0[0] : (d == 1 ? h1[0] : h2[0]), d == 0 ? h0[1] : (d == 1 ? h1[1] : h2[1])};
      fwd(i, rhs(a0[0], a1[0], a2[0], a3[0], a4[0], a5[0], a6[0]), rhs(a0[1], a1[1], a2[1], a3[1], a4[1], a5[1], a6[1]));
      shift(a6);
    }
    for (; i < s1; i++) {
      const float r0 = i == L - 1 ? sbe0[0] : (i == L - 2 ? sbe1[0] : sbe2[0]);
      const float r1 = i == L - 1 ? sbe0[1] : (i == L - 2 ? sbe1[1] : sbe2[1]);
      fwd(i, r0, r1);
    }
    cf[w * SEG_LINES + lane] = make_float4(pm2[0], pm1[0], pm2[1], pm1[1]);  // rows s1-2, s1-1
  }
  const bool multi = S > 1;
  if (multi) {
    __syncthreads();
    // 4. incoming values of every segment, carried by warp 0 (segment 0 receives zeros)
    if (w == 0 && lane < nl0) {
      float2 x = make_float2(0.f, 0.f), y = make_float2(0.f, 0.f);
      cx[lane] = make_float4(0.f, 0.f, 0.f, 0.f);
      for (int k = 1; k < S; k++) {
        const int e = seg_start(k, L, S);
        const float4 c = cf[(k - 1) * SEG_LINES + lane];
        const float2 t2 = __ldg(reinterpret_cast<const float2 *>(row(e - 2) + 4));  // g, h
        const float2 t1 = __ldg(reinterpret_cast<const float2 *>(row(e - 1) + 4));
        x = make_float2(c.x + t2.x * x.x + t2.y * x.y, c.y + t1.x * x.x + t1.y * x.y);
        y = make_float2(c.z + t2.x * y.x + t2.y * y.y, c.w + t1.x * y.x + t1.y * y.y);
        cx[k * SEG_LINES + lane] = make_float4(x.x, x.y, y.x, y.y);
      }
    }
    __syncthreads();
  }
  float *out = a.io.out + f * a.io.out_fs;
  float *drv = a.io.drva ? a.drva + B.face_off[NN] * 10 : nullptr;
  const int m = a.io.m0 + f;
  // 5. the segment's forward values, then its back substitution from zero values beyond its end; with one
  // segment that gives the results, which eta/zeta lines write straight to DRAM (a warp writes a row)
  if (act) {
    const float4 xx = multi ? cx[w * SEG_LINES + lane] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float2 x[2] = {make_float2(xx.x, xx.y), make_float2(xx.z, xx.w)};
    float q1[2] = {0, 0}, q2[2] = {0, 0};  // rows i+1, i+2
    int i = s1 - 1;
    float *pc = col + i * RS;
    const float *tr = row(i);
    float *po0 = out + base0 + (int64_t)i * stride, *po1 = out + base1 + (int64_t)i * stride;
    auto sweep = [&](auto direct) {
      constexpr bool D = decltype(direct)::value;
      auto l4 = [](const float *t) { return __ldg(reinterpret_cast<const float4 *>(t + 4)); };
      auto l1 = [](const float *t) { return __ldg(t + 10); };
      auto bwd = [&](float *c, const float4 g, const float c4) {
        float q[2];
#pragma unroll
        for (int hh = 0; hh < 2; hh++) {
          const float v = c[hh * HS] + g.x * x[hh].x + g.y * x[hh].y;
          q[hh] = g.z * v - g.w * q1[hh] - c4 * q2[hh];
        }
        if constexpr (D) {
          *po0 = q[0];
          if constexpr (ADJ) {
            if (act1) po0[SEG_LINES] = q[1];
          } else {
            if (act1) *po1 = q[1];
            po1 -= stride;
          }
          po0 -= stride;
        } else {
          c[0] = q[0];
          c[HS] = q[1];
        }
#pragma unroll
        for (int hh = 0; hh < 2; hh++) { q2[hh] = q1[hh]; q1[hh] = q[hh]; }
      };
      float4 g0 = l4(tr), g1 = l4(tr - SEG_RT), g2 = l4(tr - 2 * SEG_RT), g3 = l4(tr - 3 * SEG_RT);
      float c0 = l1(tr), c1 = l1(tr - SEG_RT), c2 = l1(tr - 2 * SEG_RT), c3 = l1(tr - 3 * SEG_RT);
      for (; i - 3 >= s0; i -= 4, pc -= 4 * RS, tr -= 4 * SEG_RT) {
        const float4 n0 = l4(tr - 4 * SEG_RT), n1 = l4(tr - 5 * SEG_RT), n2 = l4(tr - 6 * SEG_RT);
        const float4 n3 = l4(tr - 7 * SEG_RT);
        const float j0 = l1(tr - 4 * SEG_RT), j1 = l1(tr - 5 * SEG_RT), j2 = l1(tr - 6 * SEG_RT);
        const float j3 = l1(tr - 7 * SEG_RT);
        bwd(pc, g0, c0);
        bwd(pc - RS, g1, c1);
        bwd(pc - 2 * RS, g2, c2);
        bwd(pc - 3 * RS, g3, c3);
        g0 = n0; g1 = n1; g2 = n2; g3 = n3;
        c0 = j0; c1 = j1; c2 = j2; c3 = j3;
      }
      for (; i >= s0; i--, pc -= RS, tr -= SEG_RT) bwd(pc, l4(tr), l1(tr));
    };
    if (!multi && NN != 1) {
      sweep(std::true_type{});
      if (drv) {
        drv[jk0 + nbs * ((m - 1) + 5 * 0)] = q1[0];  // drva(jk,m,0) = sb(is): row 0, the last one solved
        drv[jk0 + nbs * ((m - 1) + 5 * 1)] = out[base0 + (int64_t)(L - 1) * stride];  // drva(jk,m,1) = sb(ie)
        if (act1) {
          drv[jk1 + nbs * ((m - 1) + 5 * 0)] = q1[1];
          drv[jk1 + nbs * ((m - 1) + 5 * 1)] = out[base1 + (int64_t)(L - 1) * stride];
        }
      }
    } else {
      sweep(std::false_type{});
      if (multi) {
        cf[w * SEG_LINES + lane] = make_float4(q1[0], q2[0], q1[1], q2[1]);  // rows s0, s0+1
      } else if (drv) {
        drv[jk0 + nbs * ((m - 1) + 5 * 0)] = col[0];
        drv[jk0 + nbs * ((m - 1) + 5 * 1)] = col[(L - 1) * RS];
        if (act1) {
          drv[jk1 + nbs * ((m - 1) + 5 * 0)] = col[HS];
          drv[jk1 + nbs * ((m - 1) + 5 * 1)] = col[HS + (L - 1) * RS];
        }
      }
    }
  }
  if (multi) {
    __syncthreads();
    // 6. values beyond every segment's end, carried backwards by warp 0 (the last segment receives zeros)
    if (w == 0 && lane < nl0) {
      float2 x = make_float2(0.f, 0.f), y = make_float2(0.f, 0.f);
      cx[(S - 1) * SEG_LINES + lane] = make_float4(0.f, 0.f, 0.f, 0.f);
      for (int k = S - 2; k >= 0; k--) {
        const int e = seg_start(k + 1, L, S);
        const float4 c = cf[(k + 1) * SEG_LINES + lane];
        const float2 t0 = __ldg(reinterpret_cast<const float2 *>(row(e) + 8));  // G, H
        const float2 t1 = __ldg(reinterpret_cast<const float2 *>(row(e + 1) + 8));
        x = make_float2(c.x + t0.x * x.x + t0.y * x.y, c.y + t1.x * x.x + t1.y * x.y);
        y = make_float2(c.z + t0.x * y.x + t0.y * y.y, c.w + t1.x * y.x + t1.y * y.y);
        cx[k * SEG_LINES + lane] = make_float4(x.x, x.y, y.x, y.y);
      }
    }
    __syncthreads();
    // 7. results: eta/zeta rows go straight to DRAM (a warp writes a contiguous row), xi lines through the tile
    if (act) {
      const float4 yy = cx[w * SEG_LINES + lane];
      const float2 y[2] = {make_float2(yy.x, yy.y), make_float2(yy.z, yy.w)};
      auto fv = [&](const float *c, const float *t, int hh) {
        const float2 g = __ldg(reinterpret_cast<const float2 *>(t));
        return *c + g.x * y[hh].x + g.y * y[hh].y;
      };
      auto l2 = [](const float *t) { return __ldg(reinterpret_cast<const float2 *>(t)); };
      if (drv) {
        if (w == 0) {
          drv[jk0 + nbs * ((m - 1) + 5 * 0)] = fv(col, row(0) + 8, 0);  // drva(jk,m,0) = sb(is)
          if (act1) drv[jk1 + nbs * ((m - 1) + 5 * 0)] = fv(col + HS, row(0) + 8, 1);
        }
        if (w == S - 1) {
          drv[jk0 + nbs * ((m - 1) + 5 * 1)] = fv(col + (L - 1) * RS, row(L - 1) + 8, 0);
          if (act1) drv[jk1 + nbs * ((m - 1) + 5 * 1)] = fv(col + HS + (L - 1) * RS, row(L - 1) + 8, 1);
        }
      }
      int i = s0;
      float *pc = col + i * RS;
      const float *tr = row(i) + 8;
      float2 e0 = l2(tr), e1 = l2(tr + SEG_RT), e2 = l2(tr + 2 * SEG_RT), e3 = l2(tr + 3 * SEG_RT);
      // one row of both halves: r[hh] = the row's value plus the carried correction
      auto fg2 = [&](const float *c, const float2 g, float r[2]) {
#pragma unroll
        for (int hh = 0; hh < 2; hh++) r[hh] = c[hh * HS] + g.x * y[hh].x + g.y * y[hh].y;
      };
      if constexpr (NN == 1) {
        for (; i + 3 < s1; i += 4, pc += 4 * RS, tr += 4 * SEG_RT) {
          const float2 n0 = l2(tr + 4 * SEG_RT), n1 = l2(tr + 5 * SEG_RT), n2 = l2(tr + 6 * SEG_RT);
          const float2 n3 = l2(tr + 7 * SEG_RT);
          float r0[2], r1[2], r2[2], r3[2];
          fg2(pc, e0, r0); fg2(pc + RS, e1, r1); fg2(pc + 2 * RS, e2, r2); fg2(pc + 3 * RS, e3, r3);
#pragma unroll
          for (int hh = 0; hh < 2; hh++) {
            float *q = pc + hh * HS;
            q[0] = r0[hh]; q[RS] = r1[hh]; q[2 * RS] = r2[hh]; q[3 * RS] = r3[hh];
          }
          e0 = n0; e1 = n1; e2 = n2; e3 = n3;
        }
        for (; i < s1; i++, pc += RS, tr += SEG_RT) {
          float r[2];
          fg2(pc, l2(tr), r);
          pc[0] = r[0];
          pc[HS] = r[1];
        }
      } else {
        // walking output pointers: one 64-bit add per row and half
        float *po0 = out + base0 + (int64_t)i * stride, *po1 = out + base1 + (int64_t)i * stride;
        auto put = [&](const float r[2]) {
          *po0 = r[0];
          if constexpr (ADJ) {
            if (act1) po0[SEG_LINES] = r[1];
          } else {
            if (act1) *po1 = r[1];
            po1 += stride;
          }
          po0 += stride;
        };
        for (; i + 3 < s1; i += 4, pc += 4 * RS, tr += 4 * SEG_RT) {
          const float2 n0 = l2(tr + 4 * SEG_RT), n1 = l2(tr + 5 * SEG_RT), n2 = l2(tr + 6 * SEG_RT);
          const float2 n3 = l2(tr + 7 * SEG_RT);
          float r0[2], r1[2], r2[2], r3[2];
          fg2(pc, e0, r0); fg2(pc + RS, e1, r1); fg2(pc + 2 * RS, e2, r2); fg2(pc + 3 * RS, e3, r3);
          put(r0); put(r1); put(r2); put(r3);
          e0 = n0; e1 = n1; e2 = n2; e3 = n3;
        }
        for (; i < s1; i++, pc += RS, tr += SEG_RT) {
          float r[2];
          fg2(pc, l2(tr), r);
          put(r);
        }
      }
    }
  }
  if constexpr (NN == 1) {
    __syncthreads();
    // both halves' lines back to DRAM through the tiles, a warp along one line at a time
#pragma unroll
    for (int hh = 0; hh < 2; hh++) {
      const int nl = hh ? nl1 : nl0;
      const float *tile = tiles + hh * HS;
      const int64_t o0 = B.off + (int64_t)(T0 + hh * SEG_LINES) * L;
      for (int ln = w; ln < nl; ln += nwarp) {
        const int64_t lb = o0 + (int64_t)ln * L;
        int i = lane;
        for (; i + 96 < L; i += 128) {
          out[lb + i] = tile[i * RS + ln];
          out[lb + i + 32] = tile[(i + 32) * RS + ln];
          out[lb + i + 64] = tile[(i + 64) * RS + ln];
          out[lb + i + 96] = tile[(i + 96) * RS + ln];
        }
        for (; i < L; i += 32) out[lb + i] = tile[i * RS + ln];
      }
    }
  }
  if constexpr (TMA) {
    // a tile copy that did not land in time: wait once more (bounded) before the CTA exits
    if (!tma_ok) (void)mbar_wait_bounded(&tbar, 0);
  }
}

// ---------------------------------------------------------------------------
// Dense zeta derivative (mixed path, FP32 inputs and outputs; blocks whose zeta faces are periodic onto the
// block): d = M f for every zeta line, M the block's L x L operator built on the host from the line algorithm
// itself (the periodic faces' closures, the end rows, the interior right-hand side and the LU solve, in FP64,
// rounded once).  A CTA takes one tile of lines through every field, the operator staged in shared memory once; a
// thread takes one line into registers less the line's first value (M's rows sum to zero, the derivative of a
// constant being zero: a spanwise-uniform line keeps an exactly zero derivative, and the differences of a nearly
// uniform one are exact), then forms four rows at a time, the matrix rows read from shared memory four entries a
// load and broadcast to the warp: LM / 4 loads and LM / 2 packed FMAs (fma.rn.f32x2) a row and line, with no serial
// chain across rows.  Lines of up to 32 points load the next field's line before the products of this one.  The
// kernel comes in widths LM of 16, 24, 32, 48 and 64 points, the narrowest that holds the longest line taken;
// shorter lines read zeros past their end.
// ---------------------------------------------------------------------------
template <int LM>
__global__ void __launch_bounds__(256) k_sweep_dense(SweepArgs<float, float, float> a, const float *dzm) {
  extern __shared__ __align__(16) float dmat[];  // LM rows of LM floats (rows past L uninitialised, never stored)
  constexpr bool PF = LM <= 32;                   // the next field's line loaded during this one's products
  const LTile LT = a.lt[blockIdx.x];
  const BlockDev &B = a.blk[LT.b];
  const int L = B.lze + 1;
  const int64_t plane = (int64_t)(B.lxi + 1) * (B.let + 1);
  const int64_t t = (int64_t)LT.t0 + threadIdx.x;
  const bool live = t < plane;
  const int nf = a.io.nf;
  float g[LM], h[PF ? LM : 1];
  auto load = [&](int f, float *v) {
    const float *in = a.io.in + f * a.io.in_fs + B.off + t;
#pragma unroll
    for (int j = 0; j < LM; j++) v[j] = j < L ? in[(int64_t)j * plane] : 0.f;
  };
  if (live) load(0, g);  // the first field's loads in flight while the operator is staged
  const float4 *src = reinterpret_cast<const float4 *>(dzm + (size_t)LT.b * DENSE_MAX * DENSE_MAX);
  for (int q = threadIdx.x; q < L * (LM / 4); q += blockDim.x) {
    const int i = q / (LM / 4), j4 = q - i * (LM / 4);
    reinterpret_cast<float4 *>(dmat)[q] = src[i * (DENSE_MAX / 4) + j4];
  }
  __syncthreads();
  if (!live) return;  // (no barrier below)
  float *drv = a.io.drva ? a.drva + B.face_off[3] * 10 : nullptr;
  const int64_t nbs = B.nbsize[3];
  for (int f = 0; f < nf; f++) {
    if (f > 0) {
      if constexpr (PF) {
#pragma unroll
        for (int j = 0; j < LM; j++) g[j] = h[j];
      } else {
        load(f, g);
      }
    }
    if constexpr (PF) {
      if (f + 1 < nf) load(f + 1, h);
    }
    const float f0 = g[0];
    float2 gp[LM / 2];
#pragma unroll
    for (int j = 0; j < LM; j++) g[j] = j < L ? g[j] - f0 : 0.f;
#pragma unroll
    for (int k = 0; k < LM / 2; k++) gp[k] = make_float2(g[2 * k], g[2 * k + 1]);
    float *out = a.io.out + f * a.io.out_fs + B.off + t, *o = out;
    for (int i = 0; i < L; i += 4, o += 4 * plane) {
      const float4 *row = reinterpret_cast<const float4 *>(dmat + i * LM);
      // four partial sums a row: columns 4k, 4k+1 (ea) and 4k+2, 4k+3 (eb), each pair one packed FMA
      float2 ea[4], eb[4];
#pragma unroll
      for (int u = 0; u < 4; u++) ea[u] = eb[u] = make_float2(0.f, 0.f);
#pragma unroll
      for (int j4 = 0; j4 < LM / 4; j4++) {
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const float4 mv = row[u * (LM / 4) + j4];
          ea[u] = __ffma2_rn(make_float2(mv.x, mv.y), gp[2 * j4], ea[u]);
          eb[u] = __ffma2_rn(make_float2(mv.z, mv.w), gp[2 * j4 + 1], eb[u]);
        }
      }
      float acc[4];
#pragma unroll
      for (int u = 0; u < 4; u++) acc[u] = (ea[u].x + ea[u].y) + (eb[u].x + eb[u].y);
      if (i + 4 <= L) {
        o[0] = acc[0];
        o[plane] = acc[1];
        o[2 * plane] = acc[2];
        o[3 * plane] = acc[3];
      } else {
#pragma unroll
        for (int u = 0; u < 3; u++)
          if (i + u < L) o[u * plane] = acc[u];
      }
    }
    if (drv) {  // the line ends, read back from this thread's own stores
      const int m = a.io.m0 + f;
      drv[t + nbs * ((m - 1) + 5 * 0)] = out[0];                         // drva(jk,m,0) = sb(is)
      drv[t + nbs * ((m - 1) + 5 * 1)] = out[(int64_t)(L - 1) * plane];  // drva(jk,m,1) = sb(ie)
    }
  }
}

// ---------------------------------------------------------------------------
// mpigo (src/Subroutines3D.f90:16-80): closure values of every face with
// ndf = 1.  The thread of face (A, nn, ip), line jk, field f computes what the
// neighbour B sends from its face 1-ip (the reference's tag pairing) and
// writes it into A's recv; with n45 = 1 it adds A's own boundary value times
// pbcot (periodic coordinate re-basing).
// ---------------------------------------------------------------------------
template <typename TI, typename TC>
__global__ void k_mpigo(const BlockDev *blk, const Coef<TC> *cf, const FaceTask *tasks, int nt, int n45,
                        const TI *src1, const TI *src2, const TI *src3, int64_t fs, TC *recv, int64_t recv_fs,
                        FieldOfs<TI> fo) {
  const FaceTask T = tasks[blockIdx.y];
  const int jk = blockIdx.x * blockDim.x + threadIdx.x;
  if (jk >= T.nline) return;
  const int fld = blockIdx.z;
  const Coef<TC> &C = *cf;
  const BlockDev &A = blk[T.b];
  const BlockDev &Bn = blk[T.nb_b];
  const int nn = T.nn, ip = T.ip, ipp = 1 - ip;
  const TI *src = (nn == 1 ? src1 : (nn == 2 ? src2 : src3)) + fld * fs;
  int a1, a2, a3, b1, b2, b3;
  ijk_of(A, nn, a1, a2, a3);
  ijk_of(Bn, nn, b1, b2, b3);
  const int j = jk % (a2 + 1), k = jk / (a2 + 1);
  const int bcB = Bn.nbc[ipp][nn];
  const int ii = bcB == 40 ? 0 : 1;
  const TC ra0 = bcB == 45 ? (TC)n45 : (TC)0;
  const int isB = ipp * b1, ieB = 1 - 2 * ipp;
  const int mp = nt == 0 ? LMD : LMF;
  const TI ofs = fo.v[fld];
  // the neighbour's line: point index linear in the line position (indx3, src/Subroutineso.f90:364-375)
  const int64_t b0 = Bn.off + idx3(Bn.lxi, Bn.let, 0, j, k, nn);
  const int64_t bs = nn == 1 ? 1 : (nn == 2 ? (int64_t)(Bn.lxi + 1) : (int64_t)(Bn.lxi + 1) * (Bn.let + 1));
  const TI *line = src + b0 + isB * bs;
  const int64_t step = ieB * bs;
  const TC res = ra0 * cvt_in<TI, TC>(line[0], ofs);
  TC s0 = 0, s1 = 0, sap0 = 0;
  for (int i = 0; i <= mp; i++) {
    const TC v = cvt_in<TI, TC>(line[(i + ii) * step], ofs);
    if (i == 0) sap0 = v;
    s0 += C.pbco[nt][0][i] * v;
    s1 += C.pbco[nt][1][i] * v;
  }
  TC r0 = s0 - res * C.pbcot[nt][0];
  TC r1 = s1 - res * C.pbcot[nt][1];
  TC r2 = sap0 - res;
  if (n45 == 1 && A.nbc[ip][nn] == 45) {
    const TC v = cvt_in<TI, TC>(src[A.off + idx3(A.lxi, A.let, ip * a1, j, k, nn)], ofs);
    r0 = r0 + v * C.pbcot[nt][0];
    r1 = r1 + v * C.pbcot[nt][1];
    r2 = r2 + v;
  }
  const int64_t nbs = A.nbsize[nn];
  TC *rc = recv + fld * recv_fs + A.face_off[nn] * 6;
  rc[jk + nbs * (0 + 3 * ip)] = r0;
  rc[jk + nbs * (1 + 3 * ip)] = r1;
  rc[jk + nbs * (2 + 3 * ip)] = r2;
}

// ---------------------------------------------------------------------------
// pointwise stage kernels: each CTA walks the point tiles of the work queue
// (consecutive points of one case, so per-case constants are per tile)
// ---------------------------------------------------------------------------
#define GRID_STRIDE(g, N) \
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < (N); g += (int64_t)gridDim.x * blockDim.x)
#define TILE_LOOP(e, T) \
  for (int t_ = blockIdx.x; t_ < (e).npt; t_ += gridDim.x) \
    if (const PTile T = (e).pt[t_]; true)
#define POINT_LOOP(T, g) for (int64_t g = (T).g0 + threadIdx.x; g < (T).g1; g += blockDim.x)

// ---------------------------------------------------------------------------
// Shared-memory staging of the mixed path's streaming kernels.  Each thread
// copies (cp.async) the input planes of the points it will take STG - 1 points
// ahead into its own column of a ring of STG slots, and waits only for its own
// oldest copies: the loads of the next points are in flight while it computes,
// without holding registers, and no thread waits on another (no barrier).
// A slot is refilled one iteration after it was read, once the values read from
// it have been used.
// ---------------------------------------------------------------------------
template <typename T, int NPL, int STG>
struct Ring {
  T *col;  // this thread's column: slot s, plane p at col[(s * NPL + p) * nt]
  int nt;
  __device__ Ring(T *smem, int nthreads) : col(smem + threadIdx.x), nt(nthreads) {}
  __device__ T *at(int s, int p) const { return col + (s * NPL + p) * nt; }
  __device__ T get(int s, int p) const { return *at(s, p); }
  static constexpr size_t bytes(int nthreads) { return sizeof(T) * NPL * STG * (size_t)nthreads; }
};

// the stage loop of one tile: fetch(slot, g) issues the copies of point g, take(slot, g) consumes them
template <int STG, class Fetch, class Take>
__device__ __forceinline__ void staged_points(const PTile &T, Fetch &&fetch, Take &&take) {
  const int nt = blockDim.x;
  int64_t g = T.g0 + threadIdx.x;
#pragma unroll
  for (int k = 0; k < STG - 1; k++) {
    if (g + (int64_t)k * nt < T.g1) fetch(k, g + (int64_t)k * nt);
    cp_async_commit();
  }
  for (int s = 0; g < T.g1; g += nt, s = s + 1 == STG ? 0 : s + 1) {
    const int64_t gn = g + (int64_t)(STG - 1) * nt;
    if (gn < T.g1) fetch(s == 0 ? STG - 1 : s - 1, gn);
    cp_async_commit();
    cp_async_wait<STG - 1>();
    take(s, g);
  }
}

// primitives, pressure, temperature, Sutherland viscosity (src/Main3D.f90:576-583) of point g from its state
// q[0..4] (as read from qa); false for a non-physical state
template <typename R>
struct PrimConst {  // the scheme constants of prim_point, taken once per tile
  R gamm1, gam, srefp1dre, srefoo, poo;
  double rhoE_inf;
  __device__ explicit PrimConst(const Scheme &S)
      : gamm1((R)S.gamm1), gam((R)S.gam), srefp1dre((R)S.srefp1dre), srefoo((R)S.srefoo), poo((R)S.poo),
        rhoE_inf(S.hamm1 * S.poo) {}
};
template <typename R>
__device__ __forceinline__ bool prim_point(const Eng<R> &e, const PrimConst<R> &C, int64_t N, int64_t g,
                                           const double q[5]) {
  const R gamm1 = C.gamm1, gam = C.gam, srefp1dre = C.srefp1dre, srefoo = C.srefoo;
  const double rhoE_inf = C.rhoE_inf;
  // (the mixed kernel is bound by the FP64 pipe, which also runs the conversion instruction: the state is
  // rounded to FP32 on the integer pipes instead, bit for bit the same)
  auto rnd = [](double v) -> R {
    if constexpr (Freestream<R>::on) return narrow(v);
    else return (R)v;
  };
  // (the FP64 fast build takes its reciprocals and square root from recip_nr / rsqrt_nr: the kernel is bound
  // by the FP64 pipe, and the IEEE division and square root are its largest users)
  constexpr bool NR = kFast && !Freestream<R>::on;
  const R q1 = rnd(q[0]), q2 = rnd(q[1]), q3 = rnd(q[2]), q4 = rnd(q[3]);
  R d1;
  if constexpr (NR) d1 = recip_nr(q1);
  else d1 = (R)1 / q1;
  const R d2 = q2 * d1, d3 = q3 * d1, d4 = q4 * d1;
  R pp, d5;
  if constexpr (Freestream<R>::on) {
    // p - p_inf from rhoE - rhoE_inf (taken in FP64 before rounding); (gamma-1) rhoE_inf = p_inf
    const R re = rnd(q[4] - rhoE_inf);
    pp = gamm1 * (re - (R)0.5 * (q2 * d2 + q3 * d3 + q4 * d4));
    d5 = gam * (C.poo + pp) * d1;
  } else {
    const R q5 = cvt<R>(q[4]);
    pp = gamm1 * (q5 - (R)0.5 * (q2 * d2 + q3 * d3 + q4 * d4));
    d5 = gam * pp * d1;
  }
  // T^1.5 as T*sqrt(T): the value of pow(T,1.5) to ~1 ulp with far fewer instructions
  R mu;
  if constexpr (NR) mu = srefp1dre * (d5 * (d5 * rsqrt_nr(d5))) * recip_nr(d5 + srefoo);
  else mu = srefp1dre * (d5 * sqrt(d5)) / (d5 + srefoo);
  e.prim[g] = d2; e.prim[g + N] = d3; e.prim[g + 2 * N] = d4; e.prim[g + 3 * N] = d5;
  e.p[g] = pp;
  e.mu[g] = mu;
  const R pabs = Freestream<R>::on ? C.poo + pp : pp;
  bool finite;
  if constexpr (Freestream<R>::on) finite = ((__double2hiint(q[4]) >> 20) & 0x7ff) != 0x7ff;
  else finite = fabs(q[4]) < 1e300;
  return q1 > (R)0 && pabs > (R)0 && finite;
}

template <typename R>
__global__ void k_prim(Eng<R> e) {
  const int64_t N = e.N;
  TILE_LOOP(e, T) {
    const PrimConst<R> C(e.sc[T.cs]);
    int bad = 0;
    POINT_LOOP(T, g) {
      const double q[5] = {e.qa[g], e.qa[g + N], e.qa[g + 2 * N], e.qa[g + 3 * N], e.qa[g + 4 * N]};
      if (!prim_point<R>(e, C, N, g, q)) bad = 1;
    }
    if (bad) atomicOr(&e.scal[T.cs].flag, 1);
  }
}

// the mixed path's primitives with the state staged through shared memory (Ring), PRS_STG points ahead
constexpr int PRS_STG = 4;
__global__ void __launch_bounds__(256) k_prim_staged(Eng<float> e) {
  __shared__ double prs_smem[5 * PRS_STG * 256];
  const int64_t N = e.N;
  Ring<double, 5, PRS_STG> rd(prs_smem, blockDim.x);
  auto fetch = [&](int s, int64_t g) {
#pragma unroll
    for (int p = 0; p < 5; p++) cp_async<8>(rd.at(s, p), e.qa + g + p * N);
  };
  TILE_LOOP(e, T) {
    const PrimConst<float> C(e.sc[T.cs]);
    int bad = 0;
    staged_points<PRS_STG>(T, fetch, [&](int s, int64_t g) {
      const double q[5] = {rd.get(s, 0), rd.get(s, 1), rd.get(s, 2), rd.get(s, 3), rd.get(s, 4)};
      if (!prim_point<float>(e, C, N, g, q)) bad = 1;
    });
    if (bad) atomicOr(&e.scal[T.cs].flag, 1);
  }
}

__device__ __forceinline__ void atomic_max_pos(unsigned long long *a, double v) {
  atomicMax(a, (unsigned long long)__double_as_longlong(v));
}

// CFL spectral radii, max over all points (src/Main3D.f90:590-602)
template <typename R>
__global__ void k_cfl(Eng<R> e) {
  const int64_t N = e.N;
  __shared__ double s1[32], s2v[32];
  // maxima of the CTA's tiles of one case, folded into the case's slot when the case changes
  auto flush = [&](int cs, R m1, R m2) {
    double dm1 = (double)m1, dm2 = (double)m2;
    for (int o = 16; o > 0; o >>= 1) {
      dm1 = fmax(dm1, __shfl_xor_sync(0xffffffffu, dm1, o));
      dm2 = fmax(dm2, __shfl_xor_sync(0xffffffffu, dm2, o));
    }
    const int w = threadIdx.x >> 5, ln = threadIdx.x & 31;
    __syncthreads();  // s1/s2v of an earlier flush are read
    if (ln == 0) { s1[w] = dm1; s2v[w] = dm2; }
    __syncthreads();
    if (w == 0) {
      const int nw = blockDim.x >> 5;
      dm1 = ln < nw ? s1[ln] : 0.0;
      dm2 = ln < nw ? s2v[ln] : 0.0;
      for (int o = 16; o > 0; o >>= 1) {
        dm1 = fmax(dm1, __shfl_xor_sync(0xffffffffu, dm1, o));
        dm2 = fmax(dm2, __shfl_xor_sync(0xffffffffu, dm2, o));
      }
      if (ln == 0) {
        atomic_max_pos(&e.scal[cs].cflmax[0], dm1);
        atomic_max_pos(&e.scal[cs].cflmax[1], dm2);
      }
    }
  };
  int cur = -1;
  R m1 = 0, m2 = 0;
  TILE_LOOP(e, T) {
    if (T.cs != cur) {  // uniform over the CTA: every thread walks the same tiles
      if (cur >= 0) flush(cur, m1, m2);
      cur = T.cs;
      m1 = 0;
      m2 = 0;
    }
    Scalars &SC = e.scal[T.cs];
    const R u1 = (R)SC.umf[1], u2 = (R)SC.umf[2], u3 = (R)SC.umf[3];
    POINT_LOOP(T, g) {
      const R x1 = e.xim[g], x2 = e.xim[g + N], x3 = e.xim[g + 2 * N];
      const R e1 = e.etm[g], e2 = e.etm[g + N], e3 = e.etm[g + 2 * N];
      const R z1 = e.zem[g], z2 = e.zem[g + N], z3 = e.zem[g + 2 * N];
      const R d2 = e.prim[g] + u1, d3 = e.prim[g + N] + u2, d4 = e.prim[g + 2 * N] + u3;
      const R r1 = x1 * x1 + x2 * x2 + x3 * x3 + e1 * e1 + e2 * e2 + e3 * e3 + z1 * z1 + z2 * z2 + z3 * z3;
      const R r2 = fabs(x1 * d2 + x2 * d3 + x3 * d4) + fabs(e1 * d2 + e2 * d3 + e3 * d4) + fabs(z1 * d2 + z2 * d3 + z3 * d4);
      const R s2 = fabs(e.yaco[g]);
      const R v1 = (sqrt(e.prim[g + 3 * N] * r1) + r2) * s2;
      const R d1 = (R)1 / cvt<R>(e.qa[g]);
      const R v2 = d1 * e.mu[g] * r1 * s2 * s2;
      m1 = fmax(m1, v1);
      m2 = fmax(m2, v2);
      if (v1 != v1 || v2 != v2) atomicOr(&SC.flag, 4);
    }
  }
  if (cur >= 0) flush(cur, m1, m2);
}

// the scheme constants of the viscous stresses, taken once per tile
template <typename R>
struct ViscConst {
  R gp, tgp, tt, sm1, sm2;
  int les;
  __device__ explicit ViscConst(const Scheme &S)
      : gp((R)S.gamm1prndtli), tgp((R)S.tgamm1prndtli), tt((R)S.two_three), sm1((R)S.smago1), sm2((R)S.smago2),
        les(S.les) {}
};

// a point's inputs of the stresses, read from the engine's planes
template <typename R>
struct PlaneIn {
  const Eng<R> &e;
  int64_t N, g;
  __device__ R dv(int k) const { return e.dv[g + k * N]; }
  __device__ R yac() const { return e.yaco[g]; }
  __device__ R mu() const { return e.mu[g]; }
  __device__ R rho() const { return cvt<R>(e.qa[g]); }
  __device__ R vel(int k) const { return e.prim[g + k * N]; }
};

// physical gradients of u, v, w, T and the viscous stresses and heat fluxes at one point
// (src/Main3D.f90:631-692), from the twelve derivative planes dv and the point's metrics:
// t = txx, tyy, tzz, txy, tyz, tzx and the energy terms hxx, hyy, hzz.  In gives the point's
// inputs (PlaneIn: from the planes; the staged flux kernel: from shared memory).
template <typename R, class In>
__device__ __forceinline__ void stress_point(const In &in, const ViscConst<R> &V, R x1, R x2, R x3, R e1, R e2,
                                             R e3, R z1, R z2, R z3, R t[9]) {
  R c[4][3];
#pragma unroll
  for (int f = 0; f < 4; f++) {
    const R r1 = in.dv(f * 3 + 0), r2 = in.dv(f * 3 + 1), r3 = in.dv(f * 3 + 2);
    c[f][0] = x1 * r1 + e1 * r2 + z1 * r3;
    c[f][1] = x2 * r1 + e2 * r2 + z2 * r3;
    c[f][2] = x3 * r1 + e3 * r2 + z3 * r3;
  }
  // txx,hzz,tzx from u; txy,tyy,hxx from v; hyy,tyz,tzz from w; ss(:,1:3) from T
  R txx = c[0][0], hzz = c[0][1], tzx = c[0][2];
  R txy = c[1][0], tyy = c[1][1], hxx = c[1][2];
  R hyy = c[2][0], tyz = c[2][1], tzz = c[2][2];
  const R yac = in.yac();
  R r1 = in.mu() * yac;
  R r2 = V.gp * r1, r3 = 0, d5;
  if (V.les == 1) {
    const R d1 = txx * txx + tyy * tyy + tzz * tzz + (hzz + txy) * (hzz + txy) + (hyy + tzx) * (hyy + tzx) +
                 (hxx + tyz) * (hxx + tyz);
    const R varr = (R)pow(-1.0 / (double)yac, 1.5);
    const R q1 = in.rho();
    r3 = q1 * (V.sm1 * V.sm1) * varr * sqrt((R)2 * d1);
    r1 = r1 + r3 * yac;
    r2 = r2 + V.tgp * r3 * yac;
    r3 = V.tt * (q1 * V.sm2 * varr * d1);
    d5 = V.tt * (txx + tyy + tzz);
    txx = r1 * ((R)2 * txx - d5) - r3;
    tyy = r1 * ((R)2 * tyy - d5) - r3;
    tzz = r1 * ((R)2 * tzz - d5) - r3;
  } else {
    d5 = V.tt * (txx + tyy + tzz);
    txx = r1 * ((R)2 * txx - d5);
    tyy = r1 * ((R)2 * tyy - d5);
    tzz = r1 * ((R)2 * tzz - d5);
  }
  const R ntxy = r1 * (txy + hzz), ntyz = r1 * (tyz + hxx), ntzx = r1 * (tzx + hyy);
  const R d2 = in.vel(0), d3 = in.vel(1), d4 = in.vel(2);
  t[0] = txx; t[1] = tyy; t[2] = tzz;
  t[3] = ntxy; t[4] = ntyz; t[5] = ntzx;
  t[6] = r2 * c[3][0] + d2 * txx + d3 * ntxy + d4 * ntzx;
  t[7] = r2 * c[3][1] + d2 * ntxy + d3 * tyy + d4 * ntyz;
  t[8] = r2 * c[3][2] + d2 * ntzx + d3 * ntyz + d4 * tzz;
}

// the stress planes tau (plane k holds t[k] of stress_point)
template <typename R>
__global__ void k_visc(Eng<R> e) {
  const int64_t N = e.N;
  TILE_LOOP(e, T) {
    const ViscConst<R> V(e.sc[T.cs]);
    R *tau = e.tau;
    POINT_LOOP(T, g) {
      const R x1 = e.xim[g], x2 = e.xim[g + N], x3 = e.xim[g + 2 * N];
      const R e1 = e.etm[g], e2 = e.etm[g + N], e3 = e.etm[g + 2 * N];
      const R z1 = e.zem[g], z2 = e.zem[g + N], z3 = e.zem[g + 2 * N];
      R t[9];
      stress_point<R>(PlaneIn<R>{e, N, g}, V, x1, x2, x3, e1, e2, e3, z1, z2, z3, t);
#pragma unroll
      for (int k = 0; k < 9; k++) tau[g + k * N] = t[k];
    }
  }
}

// The FP64 fast path's fluxes at one point: the same fifteen components with
// fewer FP64 operations (about 70 instead of 85): pressure and stress
// combined, sigma = p I - tau, and the energy flux as
// (rhoE + p) U - grad(xi) . (p u_inf + h).  VISC is a template argument so
// that only one variant's operations are issued (a branch inside the point
// loop was predicated, both sides executed).  AT_POINT: the stresses are taken
// at the point (stress_point, the operations of k_visc) instead of read from
// the stress planes, which then are neither written nor read in a stage.
template <bool VISC, bool AT_POINT = false>
__device__ __forceinline__ void flux_fast_point(const Eng<double> &e, int64_t N, int64_t g, double u1, double u2,
                                                double u3, const ViscConst<double> *V = nullptr) {
  const double *tp = e.tau;
  double *F = e.flx;
  const double x1 = e.xim[g], x2 = e.xim[g + N], x3 = e.xim[g + 2 * N];
  const double e1 = e.etm[g], e2 = e.etm[g + N], e3 = e.etm[g + 2 * N];
  const double z1 = e.zem[g], z2 = e.zem[g + N], z3 = e.zem[g + 2 * N];
  double tv[9];
  if constexpr (VISC && AT_POINT) {
    stress_point<double>(PlaneIn<double>{e, N, g}, *V, x1, x2, x3, e1, e2, e3, z1, z2, z3, tv);
    // each stress leaves the stress arithmetic rounded, as k_visc stores it: the (empty) register barrier keeps the
    // compiler from contracting its last product into the flux arithmetic, so the fluxes round as when they read the
    // stress planes, bit for bit
#pragma unroll
    for (int k = 0; k < 9; k++) asm volatile("" : "+d"(tv[k]));
  } else if constexpr (VISC) {
#pragma unroll
    for (int k = 0; k < 9; k++) tv[k] = tp[g + k * N];
  }
  const double pp = e.p[g];
  const double r1 = e.prim[g] + u1, r2 = e.prim[g + N] + u2, r3 = e.prim[g + 2 * N] + u3;
  const double s1 = x1 * r1 + x2 * r2 + x3 * r3;
  const double s2 = e1 * r1 + e2 * r2 + e3 * r3;
  const double s3 = z1 * r1 + z2 * r2 + z3 * r3;
  const double q = e.qa[g];
  F[g] = q * s1; F[g + N] = q * s2; F[g + 2 * N] = q * s3;
  double w1, w2, w3, sg[3][3];
  if constexpr (VISC) {
    const double txx = tv[0], tyy = tv[1], tzz = tv[2];
    const double txy = tv[3], tyz = tv[4], tzx = tv[5];
    sg[0][0] = pp - txx; sg[1][1] = pp - tyy; sg[2][2] = pp - tzz;
    sg[0][1] = sg[1][0] = -txy; sg[1][2] = sg[2][1] = -tyz; sg[0][2] = sg[2][0] = -tzx;
    w1 = fma(pp, u1, tv[6]); w2 = fma(pp, u2, tv[7]); w3 = fma(pp, u3, tv[8]);
  } else {
    w1 = pp * u1; w2 = pp * u2; w3 = pp * u3;
  }
#pragma unroll
  for (int m = 2; m <= 4; m++) {
    const double qm = e.qa[g + (m - 1) * N];
    const int r = m - 2;
    double a, b, c;
    if constexpr (VISC) {
      a = qm * s1 + x1 * sg[r][0] + x2 * sg[r][1] + x3 * sg[r][2];
      b = qm * s2 + e1 * sg[r][0] + e2 * sg[r][1] + e3 * sg[r][2];
      c = qm * s3 + z1 * sg[r][0] + z2 * sg[r][1] + z3 * sg[r][2];
    } else {
      const double xm = r == 0 ? x1 : (r == 1 ? x2 : x3), em = r == 0 ? e1 : (r == 1 ? e2 : e3);
      const double zm = r == 0 ? z1 : (r == 1 ? z2 : z3);
      a = qm * s1 + xm * pp; b = qm * s2 + em * pp; c = qm * s3 + zm * pp;
    }
    F[g + ((m - 1) * 3 + 0) * N] = a;
    F[g + ((m - 1) * 3 + 1) * N] = b;
    F[g + ((m - 1) * 3 + 2) * N] = c;
  }
  const double d5 = e.qa[g + 4 * N] + pp;
  F[g + 12 * N] = d5 * s1 - (x1 * w1 + x2 * w2 + x3 * w3);
  F[g + 13 * N] = d5 * s2 - (e1 * w1 + e2 * w2 + e3 * w3);
  F[g + 14 * N] = d5 * s3 - (z1 * w1 + z2 * w2 + z3 * w3);
}

// contravariant velocities and the fifteen flux components
// (src/Main3D.f90:710-766): flx plane (m-1)*3 + (nn-1)
// (the FP32 kernel streams: five CTAs of 256 threads an SM, at most 51 registers a thread, keep more loads
// in flight than the 80 registers it would take unbounded; measured 380 -> 296 us a launch on 8.85 M points)
// (the mixed path's viscous fluxes take the stresses at the point instead: k_flux_staged)
template <typename R>
__global__ void __launch_bounds__(256, Freestream<R>::on ? 5 : 1) k_flux(Eng<R> e) {
  const int64_t N = e.N;
  TILE_LOOP(e, T) {
    const Scheme &S = e.sc[T.cs];
    Scalars &SC = e.scal[T.cs];
    const R u1 = (R)SC.umf[1], u2 = (R)SC.umf[2], u3 = (R)SC.umf[3];
    const bool visc = S.nviscous == 1;
    if constexpr (kFast && !Freestream<R>::on) {
      if (visc) { POINT_LOOP(T, g) flux_fast_point<true>(e, N, g, u1, u2, u3); }
      else { POINT_LOOP(T, g) flux_fast_point<false>(e, N, g, u1, u2, u3); }
      continue;
    }
    const R *t = e.tau;
    R *F = e.flx;
    POINT_LOOP(T, g) {
      const R x1 = e.xim[g], x2 = e.xim[g + N], x3 = e.xim[g + 2 * N];
      const R e1 = e.etm[g], e2 = e.etm[g + N], e3 = e.etm[g + 2 * N];
      const R z1 = e.zem[g], z2 = e.zem[g + N], z3 = e.zem[g + 2 * N];
      const R pp = e.p[g];
      R s1, s2, s3;
      // freestream split: contravariant velocities of u and of umf apart
      R su1 = 0, su2 = 0, su3 = 0, sm1 = 0, sm2 = 0, sm3 = 0;
      if constexpr (Freestream<R>::on) {
        const R r1 = e.prim[g], r2 = e.prim[g + N], r3 = e.prim[g + 2 * N];
        su1 = x1 * r1 + x2 * r2 + x3 * r3; sm1 = x1 * u1 + x2 * u2 + x3 * u3;
        su2 = e1 * r1 + e2 * r2 + e3 * r3; sm2 = e1 * u1 + e2 * u2 + e3 * u3;
        su3 = z1 * r1 + z2 * r2 + z3 * r3; sm3 = z1 * u1 + z2 * u2 + z3 * u3;
        s1 = su1 + sm1; s2 = su2 + sm2; s3 = su3 + sm3;
        // rho U - rho_inf (umf . grad xi)
        const double q1 = e.qa[g];
        const R q = cvt<R>(q1), qp = cvt<R>(q1 - S.rhooo);
        F[g] = q * su1 + qp * sm1; F[g + N] = q * su2 + qp * sm2; F[g + 2 * N] = q * su3 + qp * sm3;
      } else {
        const R r1 = e.prim[g] + u1, r2 = e.prim[g + N] + u2, r3 = e.prim[g + 2 * N] + u3;
        s1 = x1 * r1 + x2 * r2 + x3 * r3;
        s2 = e1 * r1 + e2 * r2 + e3 * r3;
        s3 = z1 * r1 + z2 * r2 + z3 * r3;
        const R q = cvt<R>(e.qa[g]);
        F[g] = q * s1; F[g + N] = q * s2; F[g + 2 * N] = q * s3;
      }
      R ta[3] = {0, 0, 0}, tb[3] = {0, 0, 0}, tc[3] = {0, 0, 0};
      if (visc) {
        ta[0] = t[g]; tb[0] = t[g + 3 * N]; tc[0] = t[g + 5 * N];
        ta[1] = t[g + 3 * N]; tb[1] = t[g + N]; tc[1] = t[g + 4 * N];
        ta[2] = t[g + 5 * N]; tb[2] = t[g + 4 * N]; tc[2] = t[g + 2 * N];
      }
      const R xm[3] = {x1, x2, x3}, em[3] = {e1, e2, e3}, zm[3] = {z1, z2, z3};
  #pragma unroll
      for (int m = 2; m <= 4; m++) {
        const R q = cvt<R>(e.qa[g + (m - 1) * N]);
        R a = q * s1 + xm[m - 2] * pp;
        R b = q * s2 + em[m - 2] * pp;
        R c = q * s3 + zm[m - 2] * pp;
        if (visc) {
          a = a - x1 * ta[m - 2] - x2 * tb[m - 2] - x3 * tc[m - 2];
          b = b - e1 * ta[m - 2] - e2 * tb[m - 2] - e3 * tc[m - 2];
          c = c - z1 * ta[m - 2] - z2 * tb[m - 2] - z3 * tc[m - 2];
        }
        F[g + ((m - 1) * 3 + 0) * N] = a;
        F[g + ((m - 1) * 3 + 1) * N] = b;
        F[g + ((m - 1) * 3 + 2) * N] = c;
      }
      {
        R a, b, c;
        if constexpr (Freestream<R>::on) {
          // (rhoE + p) U - p (umf . grad xi) - rhoE_inf (umf . grad xi)
          const double q5 = e.qa[g + 4 * N];
          const R d5 = cvt<R>(q5) + (R)S.poo + pp, re = cvt<R>(q5 - S.hamm1 * S.poo);
          a = d5 * su1 + re * sm1;
          b = d5 * su2 + re * sm2;
          c = d5 * su3 + re * sm3;
        } else {
          const R d5 = cvt<R>(e.qa[g + 4 * N]) + pp;
          a = d5 * s1 - pp * (u1 * x1 + u2 * x2 + u3 * x3);
          b = d5 * s2 - pp * (u1 * e1 + u2 * e2 + u3 * e3);
          c = d5 * s3 - pp * (u1 * z1 + u2 * z2 + u3 * z3);
        }
        if (visc) {
          const R ha = t[g + 6 * N], hb = t[g + 7 * N], hc = t[g + 8 * N];
          a = a - x1 * ha - x2 * hb - x3 * hc;
          b = b - e1 * ha - e2 * hb - e3 * hc;
          c = c - z1 * ha - z2 * hb - z3 * hc;
        }
        F[g + 12 * N] = a; F[g + 13 * N] = b; F[g + 14 * N] = c;
      }
    }
  }
}

// the FP64 fast path's viscous fluxes with the stresses taken at the point (k_visc and k_flux in one pass: the
// nine stress planes are neither written nor read)
__global__ void __launch_bounds__(256) k_flux_visc(Eng<double> e) {
  const int64_t N = e.N;
  TILE_LOOP(e, T) {
    const Scheme &S = e.sc[T.cs];
    const Scalars &SC = e.scal[T.cs];
    const double u1 = SC.umf[1], u2 = SC.umf[2], u3 = SC.umf[3];
    if (S.nviscous == 1) {
      const ViscConst<double> V(S);
      POINT_LOOP(T, g) flux_fast_point<true, true>(e, N, g, u1, u2, u3, &V);
    } else {
      POINT_LOOP(T, g) flux_fast_point<false>(e, N, g, u1, u2, u3);
    }
  }
}

// the mixed path's viscous fluxes (k_flux with the stresses of k_visc taken at the point), inputs staged:
// 5 FP64 state planes and 27 FP32 planes a point (metrics 9, derivative planes 12, Jacobian, viscosity,
// velocity 3, pressure); no stress plane is written or read
constexpr int FXS_STG = 2, FXS_ND = 5, FXS_NF = 27;
struct FluxStageIn {
  const float *f;  // the point's FP32 planes in shared memory, plane stride nt
  const double *d;
  int nt;
  __device__ float at(int p) const { return f[p * nt]; }
  __device__ float dv(int k) const { return at(9 + k); }
  __device__ float yac() const { return at(21); }
  __device__ float mu() const { return at(22); }
  __device__ float rho() const { return cvt<float>(d[0]); }
  __device__ float vel(int k) const { return at(23 + k); }
};
size_t flux_staged_smem(int nt) {
  return Ring<double, FXS_ND, FXS_STG>::bytes(nt) + Ring<float, FXS_NF, FXS_STG>::bytes(nt);
}

__global__ void __launch_bounds__(256, 3) k_flux_staged(Eng<float> e) {
  extern __shared__ __align__(16) unsigned char fxs_smem[];
  const int nt = blockDim.x;
  const int64_t N = e.N;
  Ring<double, FXS_ND, FXS_STG> rd((double *)fxs_smem, nt);
  Ring<float, FXS_NF, FXS_STG> rf((float *)(fxs_smem + Ring<double, FXS_ND, FXS_STG>::bytes(nt)), nt);
  float *F = e.flx;
  auto fetch = [&](int s, int64_t g) {
#pragma unroll
    for (int p = 0; p < 5; p++) cp_async<8>(rd.at(s, p), e.qa + g + p * N);
#pragma unroll
    for (int p = 0; p < 3; p++) {
      cp_async<4>(rf.at(s, p), e.xim + g + p * N);
      cp_async<4>(rf.at(s, 3 + p), e.etm + g + p * N);
      cp_async<4>(rf.at(s, 6 + p), e.zem + g + p * N);
      cp_async<4>(rf.at(s, 23 + p), e.prim + g + p * N);
    }
#pragma unroll
    for (int p = 0; p < 12; p++) cp_async<4>(rf.at(s, 9 + p), e.dv + g + p * N);
    cp_async<4>(rf.at(s, 21), e.yaco + g);
    cp_async<4>(rf.at(s, 22), e.mu + g);
    cp_async<4>(rf.at(s, 26), e.p + g);
  };
  TILE_LOOP(e, T) {
    const Scheme &S = e.sc[T.cs];
    const Scalars &SC = e.scal[T.cs];
    const float u1 = (float)SC.umf[1], u2 = (float)SC.umf[2], u3 = (float)SC.umf[3];
    const ViscConst<float> V(S);
    const double rhooo = S.rhooo, rhoE_inf = S.hamm1 * S.poo;
    const float poo = (float)S.poo;
    staged_points<FXS_STG>(T, fetch, [&](int s, int64_t g) {
      const FluxStageIn in{rf.at(s, 0), rd.at(s, 0), nt};
      const float x1 = in.at(0), x2 = in.at(1), x3 = in.at(2);
      const float e1 = in.at(3), e2 = in.at(4), e3 = in.at(5);
      const float z1 = in.at(6), z2 = in.at(7), z3 = in.at(8);
      float tv[9];
      stress_point<float>(in, V, x1, x2, x3, e1, e2, e3, z1, z2, z3, tv);
      const float pp = in.at(26);
      // contravariant velocities of u and of umf apart (the freestream split of k_flux)
      const float r1 = in.vel(0), r2 = in.vel(1), r3 = in.vel(2);
      const float su1 = x1 * r1 + x2 * r2 + x3 * r3, sm1 = x1 * u1 + x2 * u2 + x3 * u3;
      const float su2 = e1 * r1 + e2 * r2 + e3 * r3, sm2 = e1 * u1 + e2 * u2 + e3 * u3;
      const float su3 = z1 * r1 + z2 * r2 + z3 * r3, sm3 = z1 * u1 + z2 * u2 + z3 * u3;
      const float s1 = su1 + sm1, s2 = su2 + sm2, s3 = su3 + sm3;
      const double q1 = rd.get(s, 0);
      const float q = cvt<float>(q1), qp = cvt<float>(q1 - rhooo);
      F[g] = q * su1 + qp * sm1; F[g + N] = q * su2 + qp * sm2; F[g + 2 * N] = q * su3 + qp * sm3;
      // the viscous terms are summed before they meet the inviscid flux (small terms first)
      const float ta[3] = {tv[0], tv[3], tv[5]}, tb[3] = {tv[3], tv[1], tv[4]}, tc[3] = {tv[5], tv[4], tv[2]};
      const float xm[3] = {x1, x2, x3}, em[3] = {e1, e2, e3}, zm[3] = {z1, z2, z3};
#pragma unroll
      for (int m = 2; m <= 4; m++) {
        const float qm = cvt<float>(rd.get(s, m - 1));
        const float a = qm * s1 + xm[m - 2] * pp - (x1 * ta[m - 2] + x2 * tb[m - 2] + x3 * tc[m - 2]);
        const float b = qm * s2 + em[m - 2] * pp - (e1 * ta[m - 2] + e2 * tb[m - 2] + e3 * tc[m - 2]);
        const float c = qm * s3 + zm[m - 2] * pp - (z1 * ta[m - 2] + z2 * tb[m - 2] + z3 * tc[m - 2]);
        F[g + ((m - 1) * 3 + 0) * N] = a;
        F[g + ((m - 1) * 3 + 1) * N] = b;
        F[g + ((m - 1) * 3 + 2) * N] = c;
      }
      // (rhoE + p) U - p (umf . grad xi) - rhoE_inf (umf . grad xi), less the heat-flux terms
      const double q5 = rd.get(s, 4);
      const float d5 = cvt<float>(q5) + poo + pp, re = cvt<float>(q5 - rhoE_inf);
      const float ha = tv[6], hb = tv[7], hc = tv[8];
      F[g + 12 * N] = d5 * su1 + re * sm1 - (x1 * ha + x2 * hb + x3 * hc);
      F[g + 13 * N] = d5 * su2 + re * sm2 - (e1 * ha + e2 * hb + e3 * hc);
      F[g + 14 * N] = d5 * su3 + re * sm3 - (z1 * ha + z2 * hb + z3 * hc);
    });
  }
}

// divergence de(:,m) = rr1+rr2+rr3 (src/Main3D.f90:722...) plus the sponge of
// spongego (src/SingleTurbulence3D.f90:368-372) on sponge points
template <typename R>
// (the kernel streams: eight CTAs of 256 threads an SM, at most 32 registers a thread)
__global__ void __launch_bounds__(256, 8) k_div(Eng<R> e) {
  const int64_t N = e.N;
  TILE_LOOP(e, T) {
    const Scheme &S = e.sc[T.cs];
    Scalars &SC = e.scal[T.cs];
    const R ham = (R)S.ham;
    const R *F = e.flx;
    R u1 = 0, u2 = 0, u3 = 0;
    if constexpr (Freestream<R>::on) {
      u1 = (R)SC.umf[1]; u2 = (R)SC.umf[2]; u3 = (R)SC.umf[3];
    }
    POINT_LOOP(T, g) {
      const R as = e.asz[g], bs = e.bsz[g];
      const bool sponge = as != (R)0 || bs != (R)0;
      // the mixed path: the sponge zone is a thin layer, and warps without a sponge point skip its FP64
      // subtractions and conversions (a warp vote makes the branch a real one; a per-point test was
      // predicated and issued that FP64 work everywhere).  The FP64 kernel streams and keeps one variant.
      const bool any_sponge = Freestream<R>::on ? __any_sync(__activemask(), sponge) : true;
      R fs[5] = {0, 0, 0, 0, 0};
      if constexpr (Freestream<R>::on) {
        // divergence of the freestream fluxes: rho_inf, p_inf, rhoE_inf times the metric divergence
        const R g1 = e.gm[g], g2 = e.gm[g + N], g3 = e.gm[g + 2 * N];
        const R ug = u1 * g1 + u2 * g2 + u3 * g3;
        fs[0] = (R)S.rhooo * ug;
        fs[1] = (R)S.poo * g1; fs[2] = (R)S.poo * g2; fs[3] = (R)S.poo * g3;
        fs[4] = (R)(S.hamm1 * S.poo) * ug;
      }
      // two versions of the point's update, chosen per warp
      auto update = [&](auto with_sponge) {
  #pragma unroll
        for (int m = 1; m <= 5; m++) {
          R d = F[g + ((m - 1) * 3 + 0) * N] + F[g + ((m - 1) * 3 + 1) * N] + F[g + ((m - 1) * 3 + 2) * N];
          if constexpr (Freestream<R>::on) d = d + fs[m - 1];
          if (decltype(with_sponge)::value && sponge) {
            if constexpr (Freestream<R>::on) {  // the pressure plane already holds p - p_inf, p_inf = 1/gamma
              if (m == 1) d = d + as * cvt<R>(e.qa[g] - 1.0);
              else if (m <= 4) d = d + as * cvt<R>(e.qa[g + (m - 1) * N]);
              else d = d + bs * e.p[g];
            } else {
              if (m == 1) d = d + as * (cvt<R>(e.qa[g]) - (R)1);
              else if (m <= 4) d = d + as * (cvt<R>(e.qa[g + (m - 1) * N]) - (R)0);
              else d = d + bs * (e.p[g] - ham * (R)1);
            }
          }
          e.de[g + (m - 1) * N] = d;
        }
      };
      if (!Freestream<R>::on || any_sponge) update(std::true_type{});
      else update(std::false_type{});
    }
  }
}

// RK update (src/Main3D.f90:876-881): FP64 state, FP64 Jacobian
template <typename R>
__global__ void k_rk(Eng<R> e) {
  const int64_t N = e.N;
  TILE_LOOP(e, T) {
    const Scheme &S = e.sc[T.cs];
    Scalars &SC = e.scal[T.cs];
    const double dtk = SC.dtk;
    POINT_LOOP(T, g) {
      const double r1 = dtk * e.yacod[g];
      double qo[5];
      R de[5];
#pragma unroll
      for (int q = 0; q < 5; q++) { qo[q] = e.qo[g + q * N]; de[q] = e.de[g + q * N]; }  // reads before the stores
#pragma unroll
      for (int q = 0; q < 5; q++) e.qa[g + q * N] = qo[q] - r1 * cvt<double>(de[q]);
    }
  }
}

// ---------------------------------------------------------------------------
// characteristic boundary treatment: eleme, xtq2r, xtr2q
// (src/Subroutines3D.f90:235-324) and the GCBC/GCIC loops of
// src/Main3D.f90:780-869
// ---------------------------------------------------------------------------
// The face items (one face line or corner-line point each) are real functions, not inlined: the per-face kernels and
// the fused face chains call the same compiled code, so the two give the same roundings bit for bit.
// Reads of the arrays the face items modify (de, the face buffers, qa and the visit counts) bypass the SM's L1
// cache (ld.global.cg): in a fused face chain a phase reads values that other SMs wrote in an earlier phase of the
// same launch, and a line this SM cached before could be stale.  The per-face kernels read the same way.
template <typename T>
__device__ __forceinline__ T ldm(const T *p) {
  return __ldcg(p);
}

template <typename R>
struct Elem {
  R rhoi, ao, aoi, ve[3], hv2, vn, vs;
};

template <typename R>
__device__ __forceinline__ void eleme(const Scheme &S, const Eng<R> &e, int64_t g, const R cm[3], const R umf[4],
                                      Elem<R> &el) {
  const int64_t N = e.N;
  el.rhoi = (R)1 / cvt<R>(e.qa[g]);
  const R pabs = Freestream<R>::on ? (R)S.poo + e.p[g] : e.p[g];
  el.ao = sqrt((R)S.gam * el.rhoi * pabs);
  el.aoi = (R)1 / el.ao;
  el.ve[0] = el.rhoi * cvt<R>(e.qa[g + N]);
  el.ve[1] = el.rhoi * cvt<R>(e.qa[g + 2 * N]);
  el.ve[2] = el.rhoi * cvt<R>(e.qa[g + 3 * N]);
  el.hv2 = (R)0.5 * (el.ve[0] * el.ve[0] + el.ve[1] * el.ve[1] + el.ve[2] * el.ve[2]);
  el.vn = cm[0] * el.ve[0] + cm[1] * el.ve[1] + cm[2] * el.ve[2];
  el.vs = cm[0] * umf[1] + cm[1] * umf[2] + cm[2] * umf[3];
}

template <typename R>
__device__ __forceinline__ void xtq2r(const Scheme &S, const Elem<R> &el, const R cm[3], R xt[5][5]) {
  const R ho = (R)S.gamm1 * el.aoi * el.aoi, bo = (R)1 - ho * el.hv2, co = el.aoi * el.vn;
  const R dm0 = el.aoi * cm[0], dm1 = el.aoi * cm[1], dm2 = el.aoi * cm[2];
  const R rv0 = ho * el.ve[0], rv1 = ho * el.ve[1], rv2 = ho * el.ve[2];
  const R *ve = el.ve;
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
  xt[3][0] = (R)1 - bo - co;
  xt[3][1] = dm0 - rv0;
  xt[3][2] = dm1 - rv1;
  xt[3][3] = dm2 - rv2;
  xt[3][4] = ho;
  xt[4][0] = (R)1 - bo + co;
  xt[4][1] = -dm0 - rv0;
  xt[4][2] = -dm1 - rv1;
  xt[4][3] = -dm2 - rv2;
  xt[4][4] = ho;
}

template <typename R>
__device__ __forceinline__ void xtr2q(const Scheme &S, const Elem<R> &el, const R cm[3], R xt[5][5]) {
  const R bo = el.hv2 + (R)S.hamm1 * el.ao * el.ao, co = el.ao * el.vn;
  const R dm0 = el.ao * cm[0], dm1 = el.ao * cm[1], dm2 = el.ao * cm[2];
  const R *ve = el.ve;
  const R h = (R)0.5;
  xt[0][0] = cm[0]; xt[0][1] = cm[1]; xt[0][2] = cm[2]; xt[0][3] = h; xt[0][4] = h;
  xt[1][0] = cm[0] * ve[0];
  xt[1][1] = cm[1] * ve[0] - dm2;
  xt[1][2] = cm[2] * ve[0] + dm1;
  xt[1][3] = h * (ve[0] + dm0);
  xt[1][4] = xt[1][3] - dm0;
  xt[2][0] = cm[0] * ve[1] + dm2;
  xt[2][1] = cm[1] * ve[1];
  xt[2][2] = cm[2] * ve[1] - dm0;
  xt[2][3] = h * (ve[1] + dm1);
  xt[2][4] = xt[2][3] - dm1;
  xt[3][0] = cm[0] * ve[2] - dm1;
  xt[3][1] = cm[1] * ve[2] + dm0;
  xt[3][2] = cm[2] * ve[2];
  xt[3][3] = h * (ve[2] + dm2);
  xt[3][4] = xt[3][3] - dm2;
  xt[4][0] = el.hv2 * cm[0] + dm2 * ve[1] - dm1 * ve[2];
  xt[4][1] = el.hv2 * cm[1] + dm0 * ve[2] - dm2 * ve[0];
  xt[4][2] = el.hv2 * cm[2] + dm1 * ve[0] - dm0 * ve[1];
  xt[4][3] = h * (bo + co);
  xt[4][4] = xt[4][3] - co;
}

__device__ __forceinline__ void face_point(const BlockDev &B, int nn, int ip, int jk, int &i, int &j, int &k) {
  int a1, a2, a3;
  ijk_of(B, nn, a1, a2, a3);
  j = jk % (a2 + 1);
  k = jk / (a2 + 1);
  i = ip * a1;
}

// drva = X * (J * (ra0*drva + ra1*de)) (src/Main3D.f90:780-795)
template <typename R>
__device__ __noinline__ void gcbc_prep_item(const Eng<R> &e, const FaceTask &T, int jk) {
  const BlockDev &B = e.blk[T.b];
  const Scheme &S = e.sc[B.cs];
  const Scalars &SC = e.scal[B.cs];
  const int nn = T.nn, ip = T.ip, np = T.bc;
  int i, j, k;
  face_point(B, nn, ip, jk, i, j, k);
  const int64_t g = B.off + idx3(B.lxi, B.let, i, j, k, nn), N = e.N, nbs = T.nline;
  const R ra0 = (R)((20 - np) * (25 - np) * (30 - np) / 3000), ra1 = (R)1 - ra0;
  R *drva = e.drva + B.face_off[nn] * 10;
  const R *cmv = e.cm + B.face_off[nn] * 6;
  const R cm[3] = {cmv[jk + nbs * (0 + 3 * ip)], cmv[jk + nbs * (1 + 3 * ip)], cmv[jk + nbs * (2 + 3 * ip)]};
  const R umf[4] = {0, (R)SC.umf[1], (R)SC.umf[2], (R)SC.umf[3]};
  Elem<R> el;
  eleme(S, e, g, cm, umf, el);
  R xt[5][5];
  xtq2r(S, el, cm, xt);
  R v[5], dinf[5] = {0, 0, 0, 0, 0};
  if constexpr (Freestream<R>::on) {
    // normal derivative of the freestream fluxes at the line end (from the metric derivative)
    const R *dm = e.drvm + B.face_off[nn] * 10;
    const R m1 = dm[jk + nbs * (0 + 5 * ip)], m2 = dm[jk + nbs * (1 + 5 * ip)], m3 = dm[jk + nbs * (2 + 5 * ip)];
    const R ug = umf[1] * m1 + umf[2] * m2 + umf[3] * m3;
    dinf[0] = (R)S.rhooo * ug;
    dinf[1] = (R)S.poo * m1; dinf[2] = (R)S.poo * m2; dinf[3] = (R)S.poo * m3;
    dinf[4] = (R)(S.hamm1 * S.poo) * ug;
  }
  const R yac = e.yaco[g];
#pragma unroll
  for (int q = 0; q < 5; q++) {
    if constexpr (Freestream<R>::on)
      v[q] = yac * (ra0 * (ldm(drva + jk + nbs * (q + 5 * ip)) + dinf[q]) + ra1 * ldm(e.de + g + q * N));
    else v[q] = yac * (ra0 * ldm(drva + jk + nbs * (q + 5 * ip)) + ra1 * ldm(e.de + g + q * N));
  }
#pragma unroll
  for (int r = 0; r < 5; r++) {
    R s = 0;
#pragma unroll
    for (int q = 0; q < 5; q++) s += xt[r][q] * v[q];
    drva[jk + nbs * (r + 5 * ip)] = s;
  }
}

template <typename R>
__global__ void k_gcbc_prep(const __grid_constant__ Eng<R> e, const FaceTask *tasks) {
  const FaceTask T = tasks[blockIdx.y];
  const int jk = blockIdx.x * blockDim.x + threadIdx.x;
  if (jk < T.nline) gcbc_prep_item<R>(e, T, jk);
}

// GCBC/GCIC application for the faces of one direction (src/Main3D.f90:817-869),
// launched once per direction in the reference's order so that edge points
// touched by faces of two directions accumulate in the same order
template <typename R>
__device__ __noinline__ void gcbc_apply_item(const Eng<R> &e, const FaceTask &T, int jk) {
  const BlockDev &B = e.blk[T.b];
  const Scheme &S = e.sc[B.cs];
  const Scalars &SC = e.scal[B.cs];
  const int nn = T.nn, ip = T.ip, np = T.bc, iq = 1 - 2 * ip;
  const R ra0 = (R)iq;
  int i, j, k;
  face_point(B, nn, ip, jk, i, j, k);
  const int64_t g = B.off + idx3(B.lxi, B.let, i, j, k, nn), N = e.N, nbs = T.nline;
  const R *drva = e.drva + B.face_off[nn] * 10;
  const R *cmv = e.cm + B.face_off[nn] * 6;
  const R cm[3] = {cmv[jk + nbs * (0 + 3 * ip)], cmv[jk + nbs * (1 + 3 * ip)], cmv[jk + nbs * (2 + 3 * ip)]};
  const R umf[4] = {0, (R)SC.umf[1], (R)SC.umf[2], (R)SC.umf[3]};
  Elem<R> el;
  eleme(S, e, g, cm, umf, el);
  R cha[5], d0[5];
#pragma unroll
  for (int q = 0; q < 5; q++) { d0[q] = ldm(drva + jk + nbs * (q + 5 * ip)); cha[q] = d0[q]; }
  if (np == 10) {
    if (ra0 * (el.vn + el.vs + el.ao) > (R)0) cha[3] = 0;
    if (ra0 * (el.vn + el.vs - el.ao) > (R)0) cha[4] = 0;
  } else if (np == 20 || np == 25) {
    if (e.rpex[T.wall_off + jk] == (R)0) {
      const R s = cm[0] * (R)SC.dudtmf[1] + cm[1] * (R)SC.dudtmf[2] + cm[2] * (R)SC.dudtmf[3];
      cha[3 + ip] = cha[4 - ip] + (R)2 * ra0 * el.aoi * cvt<R>(e.qa[g]) * (s + (R)50 * (el.vn + el.vs));
    }
  } else {  // 30: characteristic interface, incoming waves from the neighbour
    const BlockDev &Bn = e.blk[T.nb_b];
    const R *nbr = e.drva + Bn.face_off[nn] * 10;
    R *drvb = e.drvb + B.face_off[nn] * 10;
    R dha[5];
#pragma unroll
    for (int q = 0; q < 5; q++) {
      dha[q] = ldm(nbr + jk + nbs * (q + 5 * (1 - ip)));
      drvb[jk + nbs * (q + 5 * ip)] = dha[q];
    }
    if (ra0 * (el.vn + el.vs) > (R)0) { cha[0] = dha[0]; cha[1] = dha[1]; cha[2] = dha[2]; }
    if (ra0 * (el.vn + el.vs + el.ao) > (R)0) cha[3] = dha[3];
    if (ra0 * (el.vn + el.vs - el.ao) > (R)0) cha[4] = dha[4];
  }
  R xt[5][5];
  xtr2q(S, el, cm, xt);
  R dif[5], dh[5];
#pragma unroll
  for (int q = 0; q < 5; q++) dif[q] = cha[q] - d0[q];
#pragma unroll
  for (int r = 0; r < 5; r++) {
    R s = 0;
#pragma unroll
    for (int q = 0; q < 5; q++) s += xt[r][q] * dif[q];
    dh[r] = s;
  }
  // spread dq over the boundary point and the next MBCI points (the reads of all of them first: the stores
  // of one point would otherwise hold back the reads of the next)
  const R *w = e.sbcc + T.sbcc_off + (int64_t)jk * (MBCI + 1);
  int64_t g2[MBCI + 1];
  R dv[MBCI + 1][5];
#pragma unroll
  for (int ii = 0; ii <= MBCI; ii++) {
    g2[ii] = B.off + idx3(B.lxi, B.let, i + iq * ii, j, k, nn);
#pragma unroll
    for (int q = 0; q < 5; q++) dv[ii][q] = ldm(e.de + g2[ii] + q * N);
  }
#pragma unroll
  for (int ii = 0; ii <= MBCI; ii++) {
    const R wv = w[ii];
#pragma unroll
    for (int q = 0; q < 5; q++) e.de[g2[ii] + q * N] = dv[ii][q] + wv * dh[q];
  }
}

template <typename R>
__global__ void k_gcbc_apply(const __grid_constant__ Eng<R> e, const FaceTask *tasks) {
  const FaceTask T = tasks[blockIdx.y];
  const int jk = blockIdx.x * blockDim.x + threadIdx.x;
  if (jk < T.nline) gcbc_apply_item<R>(e, T, jk);
}

// wall temperature and velocity (src/Main3D.f90:886-895), FP64 state
__device__ __noinline__ void wall_item(const Eng<double> &e, const FaceTask &T, int jk) {
  const BlockDev &B = e.blk[T.b];
  const Scheme &S = e.sc[B.cs];
  const Scalars &SC = e.scal[B.cs];
  int i, j, k;
  face_point(B, T.nn, T.ip, jk, i, j, k);
  const int64_t g = B.off + idx3(B.lxi, B.let, i, j, k, T.nn), N = e.N;
  const double ra0 = S.ham * S.hamm1 * S.wtemp;
  const double ra1 = (double)((T.bc - 20) / 5);
  const double rp = e.rpex[T.wall_off + jk];
  const double ra2 = 1.0 - rp, ra3 = 1.0 - ra1 * ra2;
  // the point's state read before any store (rho is not written here)
  const double q1 = ldm(e.qa + g), m2 = ldm(e.qa + g + N), m3 = ldm(e.qa + g + 2 * N), m4 = ldm(e.qa + g + 3 * N),
               q5 = ldm(e.qa + g + 4 * N);
  const double fctr = (1.0 - ra3) * q1;
  const double q2 = ra3 * m2 - fctr * SC.umf[1];
  const double q3 = ra3 * m3 - fctr * SC.umf[2];
  const double q4 = ra3 * m4 - fctr * SC.umf[3];
  e.qa[g + N] = q2; e.qa[g + 2 * N] = q3; e.qa[g + 3 * N] = q4;
  e.qa[g + 4 * N] = rp * q5 + ra2 * (ra0 * q1 + 0.5 * (q2 * q2 + q3 * q3 + q4 * q4) / q1);
}

__global__ void k_wall(const __grid_constant__ Eng<double> e, const FaceTask *tasks) {
  const FaceTask T = tasks[blockIdx.y];
  const int jk = blockIdx.x * blockDim.x + threadIdx.x;
  if (jk < T.nline) wall_item(e, T, jk);
}

// junction averaging of the corner lines shared by four blocks
// (src/SingleTurbulence3D.f90:378-443)
__device__ __noinline__ void junction_item(const Eng<double> &e, const JunctionDev &J, int k) {
  const int64_t N = e.N;
  int64_t g[4];
#pragma unroll
  for (int q = 0; q < 4; q++) g[q] = J.base[q] + (int64_t)k * J.kstr[q];
  double avg[5];
#pragma unroll
  for (int m = 0; m < 5; m++) {
    const double d1 = ldm(e.qa + g[0] + m * N), d2 = ldm(e.qa + g[1] + m * N), d3 = ldm(e.qa + g[2] + m * N),
                 d4 = ldm(e.qa + g[3] + m * N);
    if (m == 0 || m == 4) avg[m] = 0.25 * (d1 + d2 + d3 + d4);
    else avg[m] = 0.5 * (ldm(e.qa + g[J.pa - 1] + m * N) + ldm(e.qa + g[J.pb - 1] + m * N));
  }
#pragma unroll
  for (int q = 0; q < 4; q++)
#pragma unroll
    for (int m = 0; m < 5; m++) e.qa[g[q] + m * N] = avg[m];
}

__global__ void k_junction(const __grid_constant__ Eng<double> e, const JunctionDev *jn, int njct) {
  const int jx = blockIdx.y;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (jx >= njct) return;
  const JunctionDev J = jn[jx];
  if (k < J.nk) junction_item(e, J, k);
}

// interface averaging: pack qa of every BC 30/35/45 face (src/Main3D.f90:908-914)
// into the FP64 face buffer drva of the set-up engine
__device__ __noinline__ void pack_item(const Eng<double> &e, const FaceTask &T, int jk) {
  const BlockDev &B = e.blk[T.b];
  int i, j, k;
  face_point(B, T.nn, T.ip, jk, i, j, k);
  const int64_t g = B.off + idx3(B.lxi, B.let, i, j, k, T.nn), N = e.N, nbs = T.nline;
  double *drva = e.drva + B.face_off[T.nn] * 10;
  double qv[5];
#pragma unroll
  for (int q = 0; q < 5; q++) qv[q] = ldm(e.qa + g + q * N);  // (the reads first, then the stores)
#pragma unroll
  for (int q = 0; q < 5; q++) drva[jk + nbs * (q + 5 * T.ip)] = qv[q];
  e.cnt[g] = 1.0;
}

__global__ void k_pack(const __grid_constant__ Eng<double> e, const FaceTask *tasks) {
  const FaceTask T = tasks[blockIdx.y];
  const int jk = blockIdx.x * blockDim.x + threadIdx.x;
  if (jk < T.nline) pack_item(e, T, jk);
}

// interface averaging of the faces of one direction (src/Main3D.f90:926-952)
__device__ __noinline__ void avg_item(const Eng<double> &e, const FaceTask &T, int jk) {
  const BlockDev &B = e.blk[T.b];
  const BlockDev &Bn = e.blk[T.nb_b];
  int i, j, k;
  face_point(B, T.nn, T.ip, jk, i, j, k);
  const int64_t g = B.off + idx3(B.lxi, B.let, i, j, k, T.nn), N = e.N, nbs = T.nline;
  const double *nbr = e.drva + Bn.face_off[T.nn] * 10;
  double *drvb = e.drvb + B.face_off[T.nn] * 10;
  // every read first (the neighbour's packed face, the point's state and count), then the stores
  double dv[5], qv[5];
#pragma unroll
  for (int q = 0; q < 5; q++) {
    dv[q] = ldm(nbr + jk + nbs * (q + 5 * (1 - T.ip)));
    qv[q] = ldm(e.qa + g + q * N);
  }
  const double cnt = ldm(e.cnt + g) + 1.0;
  e.cnt[g] = cnt;
  const double w = 1.0 / cnt;
  e.cnt[g + N] = w;
#pragma unroll
  for (int q = 0; q < 5; q++) {
    drvb[jk + nbs * (q + 5 * T.ip)] = dv[q];
    e.qa[g + q * N] = w * ((cnt - 1.0) * qv[q] + dv[q]);
  }
}

__global__ void k_avg(const __grid_constant__ Eng<double> e, const FaceTask *tasks) {
  const FaceTask T = tasks[blockIdx.y];
  const int jk = blockIdx.x * blockDim.x + threadIdx.x;
  if (jk < T.nline) avg_item(e, T, jk);
}

// ---------------------------------------------------------------------------
// time-marching scalars: movef/pitch (src/Subroutineso.f90:192-259) and the
// dt schedule (src/Main3D.f90:571-610, 873-874, 964-965), one thread
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

__device__ void scalar_op(const Scheme &S, Scalars &s, int op, int nk) {
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

__global__ void k_scalar(const Scheme *sc, Scalars *scal, int ncase, int op, int nk) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;  // one thread per case
  if (c < ncase) scalar_op(sc[c], scal[c], op, nk);
}

// ---------------------------------------------------------------------------
// Fused face chains.  The face and scalar work around the RK update is a chain of short, latency-bound steps
// (src/Main3D.f90:780-952): GCBC preparation, the application of each direction in turn, the frame update; then,
// after the update, the wall, the junctions, the face packing and the averaging of each direction.  Each chain is
// one cooperative launch (all CTAs resident) whose phases are separated by grid barriers.  A barrier's wait is
// bounded: after `limit` polls the CTA gives up, stops working, and every case of the handle gets FLAG_TIMEOUT
// (the host returns ATI_ETIMEDOUT); the other CTAs then time out at the same or the next barrier, so the launch
// always ends.  The items are those of the per-face kernels, in the same order per point, so the results are
// bit-identical to the unfused chain.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// arrive at the grid barrier (count: CTA arrivals so far) and wait until `target` arrivals, at most `limit`
// polls; true if all arrived
__device__ bool grid_barrier(unsigned *count, unsigned target, unsigned limit) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();  // this CTA's writes before its arrival
    atomicAdd(count, 1u);
    int ok = 1;
    for (unsigned k = 0; ld_acquire_u32(count) < target; k++) {
      if (k >= limit) {
        ok = 0;
        break;
      }
      __nanosleep(32);
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// the face lines of a task range as one index space: item idx lies in task q with cum[q] - cum[0] <= idx
__device__ __forceinline__ int span_find(const TaskSpan &sp, int64_t idx) {
  const int64_t base = sp.cum[0];
  int lo = 0, hi = sp.n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (sp.cum[mid] - base <= idx) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}
template <class F>
__device__ __forceinline__ void span_for(const TaskSpan &sp, F &&f) {
  const int64_t gs = (int64_t)gridDim.x * blockDim.x;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < sp.total; idx += gs) {
    const int q = span_find(sp, idx);
    f(sp.t[q], (int)(idx - (sp.cum[q] - sp.cum[0])));
  }
}

__device__ __forceinline__ void flag_all_timeout(Scalars *scal, int ncase) {
  if (threadIdx.x == 0)
    for (int c = 0; c < ncase; c++) atomicOr(&scal[c].flag, FLAG_TIMEOUT);
}

// before the RK update: GCBC preparation, application per direction, frame update (SC_MOVEF_B)
template <typename R>
__global__ void __launch_bounds__(256) k_face_pre(const __grid_constant__ Eng<R> e, const __grid_constant__ FaceChain c) {
  unsigned target = 0;
  bool ok = true;
  auto sync = [&]() {
    target += gridDim.x;
    ok = grid_barrier(c.bar, target, c.limit);
  };
  if (c.prep.total) {
    span_for(c.prep, [&](const FaceTask &T, int jk) { gcbc_prep_item<R>(e, T, jk); });
    sync();
  }
  for (int d = 1; d <= 3 && ok; d++) {
    if (!c.dir[d].total) continue;
    span_for(c.dir[d], [&](const FaceTask &T, int jk) { gcbc_apply_item<R>(e, T, jk); });
    sync();
  }
  if (!ok) {
    flag_all_timeout(e.scal, e.ncase);
    return;
  }
  if (blockIdx.x == 0)
    for (int cs = threadIdx.x; cs < e.ncase; cs += blockDim.x) scalar_op(e.sc[cs], e.scal[cs], SC_MOVEF_B, c.nk);
}

// after the RK update: wall, junctions, face packing, averaging per direction
__global__ void __launch_bounds__(256) k_face_post(const __grid_constant__ Eng<double> e,
                                                   const __grid_constant__ FaceChain c) {
  unsigned target = 0;
  bool ok = true;
  auto sync = [&]() {
    target += gridDim.x;
    ok = grid_barrier(c.bar, target, c.limit);
  };
  if (c.prep.total) {  // (the wall faces)
    span_for(c.prep, [&](const FaceTask &T, int jk) { wall_item(e, T, jk); });
    sync();
  }
  if (ok && c.njct) {
    const int64_t gs = (int64_t)gridDim.x * blockDim.x;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < (int64_t)c.njct * c.jnk; idx += gs) {
      const JunctionDev J = c.jn[idx / c.jnk];
      const int k = (int)(idx % c.jnk);
      if (k < J.nk) junction_item(e, J, k);
    }
    sync();
  }
  if (ok && c.pack.total) {
    span_for(c.pack, [&](const FaceTask &T, int jk) { pack_item(e, T, jk); });
    sync();
  }
  int last = 0;
  for (int d = 1; d <= 3; d++)
    if (c.dir[d].total) last = d;
  for (int d = 1; d <= 3 && ok; d++) {
    if (!c.dir[d].total) continue;
    span_for(c.dir[d], [&](const FaceTask &T, int jk) { avg_item(e, T, jk); });
    if (d != last) sync();
  }
  if (!ok) flag_all_timeout(e.scal, e.ncase);
}

// metrics (src/Main3D.f90:378-413): non-conservative cross products and J from
// the coordinate derivatives held in qo(1:3) (x), qa(1:3) (y), de(1:3) (z)
__global__ void k_metrics(Eng<double> e, double *xim, double *etm, double *zem, double *yaco) {
  const int64_t N = e.N;
  GRID_STRIDE(g, N) {
    const double qo1 = e.qo[g], qo2 = e.qo[g + N], qo3 = e.qo[g + 2 * N];
    const double qa1 = e.qa[g], qa2 = e.qa[g + N], qa3 = e.qa[g + 2 * N];
    const double de1 = e.de[g], de2 = e.de[g + N], de3 = e.de[g + 2 * N];
    const double x1 = qa2 * de3 - de2 * qa3, x2 = de2 * qo3 - qo2 * de3, x3 = qo2 * qa3 - qa2 * qo3;
    const double e1 = qa3 * de1 - de3 * qa1, e2 = de3 * qo1 - qo3 * de1, e3 = qo3 * qa1 - qa3 * qo1;
    const double z1 = qa1 * de2 - de1 * qa2, z2 = de1 * qo2 - qo1 * de2, z3 = qo1 * qa2 - qa1 * qo2;
    xim[g] = x1; xim[g + N] = x2; xim[g + 2 * N] = x3;
    etm[g] = e1; etm[g + N] = e2; etm[g + 2 * N] = e3;
    zem[g] = z1; zem[g + N] = z2; zem[g + 2 * N] = z3;
    yaco[g] = 3.0 / (qo1 * x1 + qo2 * e1 + qo3 * z1 + qa1 * x2 + qa2 * e2 + qa3 * z2 + de1 * x3 + de2 * e3 + de3 * z3);
  }
}

// clpost wall integrals (src/rpt.f90:1017-1056), one CTA per wall face,
// fixed-order tree sum; out[face*2 + dir]
template <typename R>
__global__ void k_forces(Eng<R> e, const FaceTask *tasks, const double *area, const double *wnor,
                         const int64_t *woff, double *out) {
  const FaceTask T = tasks[blockIdx.x];
  const BlockDev &B = e.blk[T.b];
  const int64_t N = e.N, nw = T.nline;
  const double *ar = area + woff[blockIdx.x], *wn = wnor + 3 * woff[blockIdx.x];
  double acc[2] = {0.0, 0.0};
  for (int64_t ll = threadIdx.x; ll < nw; ll += blockDim.x) {
    // wall list order of wallArea: k over lze, i over lxi (src/rpt.f90:802-803)
    const int kk = (int)(ll / (B.lxi + 1)), ii = (int)(ll % (B.lxi + 1));
    const int jw = T.ip * B.let;
    const int64_t g = B.off + ((int64_t)kk * (B.let + 1) + jw) * (B.lxi + 1) + ii;
    const double w1 = wn[ll], w2 = wn[ll + nw], w3 = wn[ll + 2 * nw];
    for (int dir = 0; dir < 2; dir++) {
      const double pw = Freestream<R>::on ? (double)e.p[g] + e.sc[B.cs].poo : (double)e.p[g];
      double v = pw * (dir == 0 ? w1 : w2) * ar[ll];
      if (e.sc[B.cs].nviscous == 1) {
        const R *t = e.tau;
        double tw;
        if (dir == 0) tw = e.qa[g] * ((double)t[g] * w1 + (double)t[g + 3 * N] * w2 + (double)t[g + 5 * N] * w3);
        else tw = e.qa[g] * ((double)t[g + 3 * N] * w1 + (double)t[g + N] * w2 + (double)t[g + 4 * N] * w3);
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

// metric divergence of the mixed path: gm(k) = D_xi(xim_k) + D_eta(etm_k) +
// D_zeta(zem_k), from three FP64 derivative sets d3 (planes 0-2: xi, 3-5: eta,
// 6-8: zeta), rounded once to FP32
__global__ void k_metric_div(const double *d3, int64_t N, float *gm) {
  GRID_STRIDE(g, N) {
#pragma unroll
    for (int k = 0; k < 3; k++) gm[g + k * N] = (float)(d3[g + k * N] + d3[g + (3 + k) * N] + d3[g + (6 + k) * N]);
  }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
template <typename TI, typename TO, typename TC>
static void sweep_t(const Eng<TC> &e, cudaStream_t st, int nn, bool filt, const SweepIO<TI, TO> &io) {
  if (e.nlt[nn] == 0) return;
  SweepArgs<TI, TO, TC> a;
  a.blk = e.blk;
  a.lt = e.lt[nn];
  a.cf = e.cf;
  a.fac = filt ? e.facf : e.facd;
  a.facu = filt ? e.facuf : e.facud;
  a.io = io;
  a.fw = e.fw + (nn - 1) * e.fw_dir;  // sweeps of different directions may run at once
  a.fw_fs = e.N;
  a.recv = e.recv;
  a.recv_fs = e.F * 6;
  a.drva = e.drva;
  a.tmap = nullptr;
  a.scal = e.scal;
  a.rowtiles = false;
  if constexpr (std::is_same<TC, float>::value) {
    if constexpr (std::is_same<TI, float>::value && std::is_same<TO, float>::value) {
      // the zeta derivative by the blocks' dense operators (every zeta line periodic onto its block; k_sweep_dense)
      if (nn == 3 && !filt && e.dense && e.dzl > 0 && !io.out2) {
        const int lm = e.dzl <= 16 ? 16 : e.dzl <= 24 ? 24 : e.dzl <= 32 ? 32 : e.dzl <= 48 ? 48 : 64;
        const size_t smem = sizeof(float) * lm * lm;
        if (lm == 16) k_sweep_dense<16><<<e.nlt[3], e.sg_lines[3], smem, st>>>(a, e.dzm);
        else if (lm == 24) k_sweep_dense<24><<<e.nlt[3], e.sg_lines[3], smem, st>>>(a, e.dzm);
        else if (lm == 32) k_sweep_dense<32><<<e.nlt[3], e.sg_lines[3], smem, st>>>(a, e.dzm);
        else if (lm == 48) k_sweep_dense<48><<<e.nlt[3], e.sg_lines[3], smem, st>>>(a, e.dzm);
        else k_sweep_dense<64><<<e.nlt[3], e.sg_lines[3], smem, st>>>(a, e.dzm);
        return;
      }
    }
    // the mixed path: segmented solves over tiles of SEG_LINES lines
    const float *seg = filt ? e.segf : e.segd;
    a.rowtiles = e.eta_rowtiles;
    if (seg && e.nsegc[nn] > 0 && (filt || !io.out2)) {  // (a derivative with a second output: sequential kernels)
      for (int c = 0; c < e.nsegc[nn]; c++) {  // one launch per class of equal segment counts
        const SegClass &C = e.segc[nn][c];
        if (C.n == 0) continue;
        a.lt = e.lts[nn] + C.off;
        const int G = C.groups;
        const int nt = SEG_LINES * (G > 1 ? G : seg_count(C.maxlen));
        const size_t smem = seg_smem_bytes(C.maxlen, G);
        const dim3 g(C.n, io.nf);
#define ATI_SEG(D, F) k_sweep_seg<D, F, false, TI, TO><<<g, nt, smem, st>>>(a, seg, G)
        if constexpr (std::is_same<TI, float>::value) {
          // eta/zeta derivative sweeps of an array with tensor maps: tiles staged by TMA
          const int arr = io.in == e.prim ? 0 : (io.in == e.flx + (int64_t)(nn - 1) * e.N ? 1 : -1);
          const bool tma = !filt && nn >= 2 && e.tma[nn] && arr >= 0;
          // paired lines: a CTA solves two groups of lines, lane l line l of each (lines of up to PAIR_MAX_SEG
          // segments: longer ones would halve the CTAs an SM holds, measured slower)
          const size_t psm = pair_smem_bytes(C.maxlen, G > 1) + 128;
          if (!filt && e.pairs && seg_count(C.maxlen) <= PAIR_MAX_SEG && psm <= SEG_SMEM_MAX) {
            const int single = G > 1 ? 1 : 0;
            const dim3 gp(single ? C.n : C.n / 2, io.nf);
            const int ntp = SEG_LINES * (single ? 1 : seg_count(C.maxlen));
            const bool adj = nn == 3 || (nn == 2 && e.eta_rowtiles);
            if (tma) a.tmap = e.tmaps + (int64_t)(arr * 2 + nn - 2) * e.nblk;
#define ATI_PAIR(D, T, J) k_sweep_pair<D, T, J><<<gp, ntp, psm, st>>>(a, seg, single)
            if (nn == 1) ATI_PAIR(1, false, false);
            else if (nn == 2) {
              if (tma) ATI_PAIR(2, true, true);
              else if (adj) ATI_PAIR(2, false, true);
              else ATI_PAIR(2, false, false);
            } else {
              if (tma) ATI_PAIR(3, true, true);
              else ATI_PAIR(3, false, true);
            }
#undef ATI_PAIR
            continue;
          }
          if (tma) {
            a.tmap = e.tmaps + (int64_t)(arr * 2 + nn - 2) * e.nblk;
            const size_t sm = smem + 128;  // (alignment of the tensor copies' destination)
            if (nn == 2) k_sweep_seg<2, false, true, TI, TO><<<g, nt, sm, st>>>(a, seg, G);
            else k_sweep_seg<3, false, true, TI, TO><<<g, nt, sm, st>>>(a, seg, G);
            continue;
          }
        }
        if (!filt) { if (nn == 1) ATI_SEG(1, false); else if (nn == 2) ATI_SEG(2, false); else ATI_SEG(3, false); }
        else { if (nn == 1) ATI_SEG(1, true); else if (nn == 2) ATI_SEG(2, true); else ATI_SEG(3, true); }
#undef ATI_SEG
      }
      return;
    }
  }
  const dim3 grid(e.nlt[nn], io.nf);
  if (nn == 1) {
    if (filt) k_sweep_xc<true, TI, TO, TC><<<grid, XC_NL, 0, st>>>(a);
    else k_sweep_xc<false, TI, TO, TC><<<grid, XC_NL, 0, st>>>(a);
    return;
  }
  const int tpb = e.sg_lines[nn];
  const size_t smem = (size_t)e.maxlen[nn] * tpb * sizeof(TC);
  if (smem <= SG_SMEM_FW) {  // short lines: forward values in shared memory
#define ATI_SG(D, F) k_sweep_g<D, F, true, TI, TO, TC><<<grid, tpb, smem, st>>>(a)
    if (!filt) { if (nn == 2) ATI_SG(2, false); else ATI_SG(3, false); }
    else { if (nn == 2) ATI_SG(2, true); else ATI_SG(3, true); }
#undef ATI_SG
    return;
  }
  if (!filt) {
    if (nn == 2) k_sweep_g<2, false, false, TI, TO, TC><<<grid, tpb, 0, st>>>(a);
    else k_sweep_g<3, false, false, TI, TO, TC><<<grid, tpb, 0, st>>>(a);
  } else {
    if (nn == 2) k_sweep_g<2, true, false, TI, TO, TC><<<grid, tpb, 0, st>>>(a);
    else k_sweep_g<3, true, false, TI, TO, TC><<<grid, tpb, 0, st>>>(a);
  }
}

// the segmented sweeps may take more than the default 48 KB of dynamic shared memory: each kernel may use what the
// device allows a block beyond the kernel's own static shared memory
template <typename K>
static cudaError_t seg_attr_one(K kernel) {
  int dev = 0, optin = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaFuncAttributes fa{};
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, kernel);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
}
template <typename TI, typename TO>
static cudaError_t seg_attr() {
  cudaError_t e = seg_attr_one(k_sweep_seg<1, false, false, TI, TO>);
  if (e == cudaSuccess) e = seg_attr_one(k_sweep_seg<2, false, false, TI, TO>);
  if (e == cudaSuccess) e = seg_attr_one(k_sweep_seg<3, false, false, TI, TO>);
  if (e == cudaSuccess) e = seg_attr_one(k_sweep_seg<1, true, false, TI, TO>);
  if (e == cudaSuccess) e = seg_attr_one(k_sweep_seg<2, true, false, TI, TO>);
  if (e == cudaSuccess) e = seg_attr_one(k_sweep_seg<3, true, false, TI, TO>);
  if constexpr (std::is_same<TI, float>::value) {
    if (e == cudaSuccess) e = seg_attr_one(k_sweep_seg<2, false, true, TI, TO>);
    if (e == cudaSuccess) e = seg_attr_one(k_sweep_seg<3, false, true, TI, TO>);
    if (e == cudaSuccess) e = seg_attr_one(k_sweep_pair<1, false, false>);
    if (e == cudaSuccess) e = seg_attr_one(k_sweep_pair<2, false, false>);
    if (e == cudaSuccess) e = seg_attr_one(k_sweep_pair<2, false, true>);
    if (e == cudaSuccess) e = seg_attr_one(k_sweep_pair<3, false, true>);
    if (e == cudaSuccess) e = seg_attr_one(k_sweep_pair<2, true, true>);
    if (e == cudaSuccess) e = seg_attr_one(k_sweep_pair<3, true, true>);
  }
  return e;
}
// the mixed path's kernels with more than 48 KB of dynamic shared memory: the segmented sweeps and the staged
// flux kernel
cudaError_t seg_init() {
  cudaError_t e = seg_attr<float, float>();
  if (e == cudaSuccess) e = seg_attr<double, double>();
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_flux_staged, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)flux_staged_smem(256));
  return e;
}

void sweep_ddd(const Eng<double> &e, cudaStream_t st, int nn, bool filt, const SweepIO<double, double> &io) {
  sweep_t<double, double, double>(e, st, nn, filt, io);
}
void sweep_fff(const Eng<float> &e, cudaStream_t st, int nn, bool filt, const SweepIO<float, float> &io) {
  sweep_t<float, float, float>(e, st, nn, filt, io);
}
void sweep_ddf(const Eng<float> &e, cudaStream_t st, int nn, bool filt, const SweepIO<double, double> &io) {
  sweep_t<double, double, float>(e, st, nn, filt, io);
}

template <typename TI, typename TC>
static void mpigo_t(const Eng<TC> &e, cudaStream_t st, const FaceTask *tasks, int ntask, int maxline, int nt, int n45,
                    const TI *s1, const TI *s2, const TI *s3, int64_t fs, int nf, const FieldOfs<TI> &fo = {}) {
  if (ntask == 0 || nf == 0) return;
  const int tpb = 128;
  k_mpigo<TI, TC><<<dim3((maxline + tpb - 1) / tpb, ntask, nf), tpb, 0, st>>>(e.blk, e.cf, tasks, nt, n45, s1, s2, s3,
                                                                              fs, e.recv, e.F * 6, fo);
}
void mpigo_ddd(const Eng<double> &e, cudaStream_t st, const FaceTask *tasks, int ntask, int maxline, int nt, int n45,
               const double *s1, const double *s2, const double *s3, int64_t fs, int nf) {
  mpigo_t<double, double>(e, st, tasks, ntask, maxline, nt, n45, s1, s2, s3, fs, nf);
}
void mpigo_fff(const Eng<float> &e, cudaStream_t st, const FaceTask *tasks, int ntask, int maxline, int nt, int n45,
               const float *s1, const float *s2, const float *s3, int64_t fs, int nf) {
  mpigo_t<float, float>(e, st, tasks, ntask, maxline, nt, n45, s1, s2, s3, fs, nf);
}
void mpigo_ddf(const Eng<float> &e, cudaStream_t st, const FaceTask *tasks, int ntask, int maxline, int nt, int n45,
               const double *s1, const double *s2, const double *s3, int64_t fs, int nf, const FieldOfs<double> &ofs) {
  mpigo_t<double, float>(e, st, tasks, ntask, maxline, nt, n45, s1, s2, s3, fs, nf, ofs);
}

static int pw_grid(int64_t N) {
  int64_t b = (N + 255) / 256;
  const int64_t cap = 152 * 16;
  return (int)(b < cap ? (b < 1 ? 1 : b) : cap);
}

template <typename R>
static void pointwise_t(const Eng<R> &eng, cudaStream_t st, int which) {
  Eng<R> e = eng;
  if (eng.ptk[which]) {  // the kernel's own tile size
    e.pt = eng.ptk[which];
    e.npt = eng.nptk[which];
  }
  if (e.npt == 0) return;
  const int g = e.npt < 152 * 16 ? e.npt : 152 * 16, t = 256;  // CTAs walk the point tiles, stride gridDim.x
  switch (which) {
    case PW_PRIM:
      if constexpr (Freestream<R>::on) k_prim_staged<<<g, t, 0, st>>>(e);
      else k_prim<R><<<g, t, 0, st>>>(e);
      break;
    case PW_CFL: k_cfl<R><<<g, t, 0, st>>>(e); break;
    case PW_VISC: k_visc<R><<<g, t, 0, st>>>(e); break;
    case PW_FLUX: k_flux<R><<<g, t, 0, st>>>(e); break;
    case PW_FLUX_STRESS:  // viscous fluxes with the stresses taken at the point (the strict FP64 path: k_visc)
      if constexpr (Freestream<R>::on) k_flux_staged<<<g, t, flux_staged_smem(t), st>>>(e);
      else if constexpr (kFast) k_flux_visc<<<g, t, 0, st>>>(e);
      break;
    case PW_DIV: k_div<R><<<g, t, 0, st>>>(e); break;
    case PW_RK: k_rk<R><<<g, t, 0, st>>>(e); break;
  }
}
void pointwise_d(const Eng<double> &e, cudaStream_t st, int which) { pointwise_t<double>(e, st, which); }
void pointwise_f(const Eng<float> &e, cudaStream_t st, int which) { pointwise_t<float>(e, st, which); }

void face_d(const Eng<double> &e, cudaStream_t st, int which, const FaceTask *tasks, int ntask, int maxline) {
  if (ntask == 0) return;
  const int tpb = 128;
  dim3 grid((maxline + tpb - 1) / tpb, ntask);
  switch (which) {
    case FK_GCBC_PREP: k_gcbc_prep<double><<<grid, tpb, 0, st>>>(e, tasks); break;
    case FK_GCBC_APPLY: k_gcbc_apply<double><<<grid, tpb, 0, st>>>(e, tasks); break;
    case FK_WALL: k_wall<<<grid, tpb, 0, st>>>(e, tasks); break;
    case FK_PACK: k_pack<<<grid, tpb, 0, st>>>(e, tasks); break;
    case FK_AVG: k_avg<<<grid, tpb, 0, st>>>(e, tasks); break;
  }
}
void face_f(const Eng<float> &e, cudaStream_t st, int which, const FaceTask *tasks, int ntask, int maxline) {
  if (ntask == 0) return;
  const int tpb = 128;
  dim3 grid((maxline + tpb - 1) / tpb, ntask);
  switch (which) {
    case FK_GCBC_PREP: k_gcbc_prep<float><<<grid, tpb, 0, st>>>(e, tasks); break;
    case FK_GCBC_APPLY: k_gcbc_apply<float><<<grid, tpb, 0, st>>>(e, tasks); break;
    default: break;  // wall, pack and averaging act on the FP64 state: face_d
  }
}

// cooperative launch of a fused chain: CTAs of 256 threads, as many as the kernel can keep resident at once (the
// chains' items are chains of dependent loads: the more of them in flight, the shorter each phase)
static int coop_cap(const void *kernel) {
  static std::mutex mu;
  static std::map<std::pair<int, const void *>, int> cap;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(mu);
  auto it = cap.find({dev, kernel});
  if (it != cap.end()) return it->second;
  int nsm = 0, per_sm = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 256, 0) != cudaSuccess) {
    cudaGetLastError();
    per_sm = 0;
  }
  const int c = per_sm >= 1 ? per_sm * (nsm > 0 ? nsm : 1) : 0;  // (0: the kernel cannot run)
  cap[{dev, kernel}] = c;
  return c;
}
template <typename K, typename... A>
static cudaError_t coop_launch(K kernel, int want, cudaStream_t st, A... args) {
  const int cap = coop_cap((const void *)kernel);
  if (cap < 1) return cudaErrorCooperativeLaunchTooLarge;
  const int g = want < 1 ? 1 : (want < cap ? want : cap);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(g);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}
static int chain_ctas(const FaceChain &c) {
  int64_t items = c.prep.total;
  for (int d = 1; d <= 3; d++) items = items > c.dir[d].total ? items : c.dir[d].total;
  items = items > c.pack.total ? items : c.pack.total;
  items = items > (int64_t)c.njct * c.jnk ? items : (int64_t)c.njct * c.jnk;
  return (int)((items + 255) / 256);
}
cudaError_t face_pre_d(const Eng<double> &e, cudaStream_t st, const FaceChain &c) {
  return coop_launch(k_face_pre<double>, chain_ctas(c), st, e, c);
}
cudaError_t face_pre_f(const Eng<float> &e, cudaStream_t st, const FaceChain &c) {
  return coop_launch(k_face_pre<float>, chain_ctas(c), st, e, c);
}
cudaError_t face_post(const Eng<double> &e, cudaStream_t st, const FaceChain &c) {
  return coop_launch(k_face_post, chain_ctas(c), st, e, c);
}

void metric_divergence(const Eng<double> &e, cudaStream_t st, const double *d3, float *gm) {
  k_metric_div<<<pw_grid(e.N), 256, 0, st>>>(d3, e.N, gm);
}

void junction(const Eng<double> &e, cudaStream_t st, const JunctionDev *jn, int njct, int nk) {
  if (njct == 0) return;
  const int tpb = 64;
  k_junction<<<dim3((nk + tpb - 1) / tpb, njct), tpb, 0, st>>>(e, jn, njct);
}

void scalar(const Eng<double> &e, cudaStream_t st, int op, int nk) {
  k_scalar<<<(e.ncase + 63) / 64, 64, 0, st>>>(e.sc, e.scal, e.ncase, op, nk);
}

void metrics(const Eng<double> &e, cudaStream_t st, const double *xyz) {
  (void)xyz;
  k_metrics<<<pw_grid(e.N), 256, 0, st>>>(e, const_cast<double *>(e.xim), const_cast<double *>(e.etm),
                                           const_cast<double *>(e.zem), const_cast<double *>(e.yaco));
}

void forces_d(const Eng<double> &e, cudaStream_t st, const FaceTask *tasks, int ntask, const double *area,
              const double *wnor, const int64_t *woff, double *out) {
  if (ntask == 0) return;
  k_forces<double><<<ntask, 256, 0, st>>>(e, tasks, area, wnor, woff, out);
}
void forces_f(const Eng<float> &e, cudaStream_t st, const FaceTask *tasks, int ntask, const double *area,
              const double *wnor, const int64_t *woff, double *out) {
  if (ntask == 0) return;
  k_forces<float><<<ntask, 256, 0, st>>>(e, tasks, area, wnor, woff, out);
}

}  // namespace ATI_KNS
}  // namespace ati
