// ati_scheme.cpp — host-side construction of the compact-scheme coefficients
// and LU factors that the kernels consume.
//
// The coefficient formulas are the reference's (they define the numerical
// method): the optimised interior/boundary derivative rows
// (src/MainVar3D.f90:34-68, src/Main3D.f90:71-73,295-301), the filter rows
// of fcint/fcbcm (src/Subroutineso.f90:71-103), the sub-domain closure
// coefficients of sbcco (src/Subroutineso.f90:107-159) and the pentadiagonal
// factorisation of penta (src/Subroutineso.f90:15-67).  The dense linear
// algebra around them (the inverse inside sbcco, the GCBC weight solve) is
// a restatement of the reference's Gauss–Jordan mtrxi, so that the
// coefficients match the reference's bit for bit.
#include <cmath>
#include <cstring>
#include <vector>

#include "ati_scheme.h"

namespace ati {
namespace {

constexpr double kAlpha = 0.5862704032801503, kBeta = 0.09549533555017055;
constexpr double kAa = 0.6431406736919156, kAb = 0.2586011023495066, kAc = 0.007140953479797375;
constexpr double kBeta20 = 0.03250008295108466, kAlpha21 = 0.3998040493524358, kAlpha23 = 0.7719261277615860,
                 kBeta24 = 0.1626635931256900;
constexpr double kA20 = -0.1219006056449124, kA21 = -0.6301651351188667, kA23 = 0.6521195063966084,
                 kA24 = 0.3938843551210350, kA25 = 0.01904944407973912, kA26 = -0.001027260523947668;
constexpr double kAlpha10 = 0.08360703307833438, kAlpha12 = 2.058102869495757, kBeta13 = 0.9704052014790193;
constexpr double kA10 = -0.3177447290722621, kA12 = -0.02807631929593225, kA13 = 1.593461635747659,
                 kA14 = 0.2533027046976367, kA15 = -0.03619652460174756, kA16 = 0.004080281419108407;
constexpr double kAlpha01 = 5.912678614078549, kBeta02 = 3.775623951744012;
constexpr double kA01 = -3.456878182643609, kA02 = 5.839043358834730, kA03 = 1.015886726041007,
                 kA04 = -0.2246526470654333, kA05 = 0.08564940889936562, kA06 = -0.01836710059356763;

struct Dense {
  int n;
  std::vector<double> v;
  explicit Dense(int n_) : n(n_), v((size_t)n_ * n_, 0.0) {}
  double &operator()(int r, int c) { return v[(size_t)r * n + c]; }
  double operator()(int r, int c) const { return v[(size_t)r * n + c]; }
};

// In-place Gauss-Jordan inversion with partial pivoting and a final column
// permutation: the elimination of mtrxi (src/Subroutineso.f90:163-188), kept
// operation-for-operation so the closure coefficients come out bit-identical
// to the reference's.
Dense inverse(const Dense &A) {
  const int n = A.n;
  Dense r = A, out(n);
  std::vector<int> ipvt(n);
  std::vector<double> temp(n);
  for (int i = 0; i < n; i++) ipvt[i] = i;
  for (int i = 0; i < n; i++) {
    int m = i;
    double best = std::fabs(r(i, i));
    for (int q = i + 1; q < n; q++)
      if (std::fabs(r(q, i)) > best) { best = std::fabs(r(q, i)); m = q; }
    if (m != i) {
      std::swap(ipvt[m], ipvt[i]);
      for (int c = 0; c < n; c++) std::swap(r(m, c), r(i, c));
    }
    const double ra0 = 1.0 / r(i, i);
    for (int q = 0; q < n; q++) temp[q] = r(q, i);
    for (int j = 0; j < n; j++) {
      const double ra1 = ra0 * r(i, j);
      for (int q = 0; q < n; q++) r(q, j) = r(q, j) - ra1 * temp[q];
      r(i, j) = ra1;
    }
    for (int q = 0; q < n; q++) r(q, i) = -ra0 * temp[q];
    r(i, i) = ra0;
  }
  for (int c = 0; c < n; c++)
    for (int q = 0; q < n; q++) out(q, ipvt[c]) = r(q, c);
  return out;
}

Dense mul(const Dense &A, const Dense &B) {
  const int n = A.n;
  Dense C(n);
  for (int j = 0; j < n; j++)
    for (int i = 0; i < n; i++) {
      double s = 0.0;
      for (int k = 0; k < n; k++) s += A(i, k) * B(k, j);
      C(i, j) = s;
    }
  return C;
}

}  // namespace

void filter_coeffs(double fltk, double fltr, double &alphz, double &betz, double &za, double &zb, double &zc) {
  // src/Subroutineso.f90:91-103
  const double c1 = std::cos(fltk), c2 = std::cos(2 * fltk), c3 = std::cos(3 * fltk);
  const double fctr = 1 / (30 + 5 * (7 - 16 * fltr) * c1 + 2 * (1 + 8 * fltr) * c2 - 3 * c3);
  alphz = fctr * (20 * (2 * fltr - 1) - 30 * c1 + 12 * (2 * fltr - 1) * c2 - 2 * c3);
  betz = 0.5 * fctr * (2 * (13 - 8 * fltr) + (33 - 48 * fltr) * c1 + 6 * c2 - c3);
  const double ch = std::cos(0.5 * fltk), ch2 = ch * ch;
  za = 60 * (1 - fltr) * (ch2 * ch2) * fctr;
  zb = -2 * za / 5;
  zc = za / 15;
}

void build_scheme(const ati_config_t &cfg, SchemeHost &H) {
  Scheme &S = H.s;
  std::memset(&S, 0, sizeof(S));
  const double pi = std::acos(-1.0);
  const double fltk = pi * cfg.fltk, fltkbc = pi * cfg.fltkbc;
  // interior and one-sided boundary rows (src/Main3D.f90:71-73, 295-301)
  const double r0[6] = {kA01, kA02, kA03, kA04, kA05, kA06};
  const double r1[6] = {kA10, kA12, kA13, kA14, kA15, kA16};
  const double r2[6] = {kA20, kA21, kA23, kA24, kA25, kA26};
  for (int q = 0; q < 6; q++) { S.abc[0][q] = r0[q]; S.abc[1][q] = r1[q]; S.abc[2][q] = r2[q]; }
  S.aa = kAa; S.ab = kAb; S.ac = kAc;
  const double bd[2][3][5] = {{{0, 0, 1, kAlpha01, kBeta02}, {0, kAlpha10, 1, kAlpha12, kBeta13},
                               {kBeta20, kAlpha21, 1, kAlpha23, kBeta24}},
                              {{0, 0, 1, kAlpha, kBeta}, {0, kAlpha, 1, kAlpha, kBeta}, {kBeta, kAlpha, 1, kAlpha, kBeta}}};
  std::memcpy(H.albed, bd, sizeof(bd));
  // filter rows (fcbcm, fcint)
  {
    double al, be, za, zb, zc;
    const double res = (fltkbc - fltk) / 9, c2 = fltk + res, c1 = fltk + 4 * res, c0 = fltk + 9 * res;
    filter_coeffs(c0, 0.5, al, be, za, zb, zc);
    const double f = 1.0 / (1.0 + al / 2 + be / 4);
    const double row0[5] = {0, 0, 1, al * f, be * f};
    std::memcpy(H.albef[0][0], row0, sizeof(row0));
    S.fam[0] = za * f; S.fbm[0] = zb * f; S.fcm[0] = zc * f;
    filter_coeffs(c1, 0.5, al, be, za, zb, zc);
    const double row1[5] = {0, al + be / 2, 1, al, be};
    std::memcpy(H.albef[0][1], row1, sizeof(row1));
    S.fam[1] = za; S.fbm[1] = zb; S.fcm[1] = zc;
    filter_coeffs(c2, 0.5, al, be, za, zb, zc);
    const double row2[5] = {be, al, 1, al, be};
    std::memcpy(H.albef[0][2], row2, sizeof(row2));
    S.fam[2] = za; S.fbm[2] = zb; S.fcm[2] = zc;
    filter_coeffs(fltk, 0.5, H.alphf, H.betf, S.fa, S.fb, S.fc);
    const double a = H.alphf, b = H.betf;
    const double e0[5] = {0, 0, 1, a, b}, e1[5] = {0, a, 1, a, b}, e2[5] = {b, a, 1, a, b};
    std::memcpy(H.albef[1][0], e0, sizeof(e0));
    std::memcpy(H.albef[1][1], e1, sizeof(e1));
    std::memcpy(H.albef[1][2], e2, sizeof(e2));
  }
  // sub-domain closure coefficients (sbcco)
  for (int nt = 0; nt <= 1; nt++) {
    const int lp = 2 * nt - 1, ll = nt == 0 ? LMD : LMF, n = 2 * (ll + 1);
    Dense ax(n), bx(n);
    if (nt == 0) {
      double s[3] = {0, 0, 0};
      for (int r = 0; r < 3; r++)
        for (int q = 0; q < 6; q++) s[r] += S.abc[r][q];
      for (int q = 0; q <= 2; q++) ax(0, q) = H.albed[0][0][q + 2];
      const double b0[7] = {-s[0], kA01, kA02, kA03, kA04, kA05, kA06};
      const double b1[7] = {kA10, -s[1], kA12, kA13, kA14, kA15, kA16};
      const double b2[7] = {kA20, kA21, -s[2], kA23, kA24, kA25, kA26};
      for (int q = 0; q <= 3; q++) ax(1, q) = H.albed[0][1][q + 1];
      for (int q = 0; q <= 4; q++) ax(2, q) = H.albed[0][2][q];
      for (int q = 0; q < 7; q++) { bx(0, q) = b0[q]; bx(1, q) = b1[q]; bx(2, q) = b2[q]; }
      for (int i = 3; i <= n - 4; i++) {
        const double ar[5] = {kBeta, kAlpha, 1, kAlpha, kBeta}, br[7] = {-kAc, -kAb, -kAa, 0, kAa, kAb, kAc};
        for (int q = 0; q < 5; q++) ax(i, i - 2 + q) = ar[q];
        for (int q = 0; q < 7; q++) bx(i, i - 3 + q) = br[q];
      }
    } else {
      double al, be, za, zb, zc;
      filter_coeffs(fltk, 0.5, al, be, za, zb, zc);
      const double zv[5] = {zb + 5 * zc, za - 10 * zc, za - 5 * zc, zb + zc, zc};
      const double A2 = al * al, A3 = al * al * al, B2 = be * be, B3 = be * be * be;
      double f = 1 / (1 + 5 * A3 + A2 * (8 + 22 * be) + be * (5 + 4 * be + 60 * B2) + 5 * al * (1 + be * (3 + 10 * be)));
      double q0 = (al * (1 + al) * (1 + 4 * al) + 2 * al * (7 + 3 * al) * be + 24 * (1 - al) * B2 - 80 * B3) * f;
      double q1 = (A3 + be + 14 * A2 * be + 60 * B3 + al * be * (3 + 46 * be)) * f;
      ax(0, 0) = 1; ax(0, 1) = q0; ax(0, 2) = q1;
      f = 1 / (1 + A2 * (9 - 5 * be) + al * (5 + (35 - 29 * be) * be) + be * (5 + 6 * (9 - 10 * be) * be));
      q0 = (9 * A3 + 10 * B2 * (8 * be - 1) + 5 * A2 * (1 + 8 * be) + al * (1 + be * (4 + 81 * be))) * f;
      q1 = (al * (1 + al * (5 + 9 * al)) + al * (5 + 36 * al) * be + (55 * al - 1) * B2 + 10 * B3) * f;
      const double q2 = be * (1 + al * (5 + 9 * al) + 5 * be + 35 * al * be + 50 * B2) * f;
      ax(1, 0) = q0; ax(1, 1) = 1; ax(1, 2) = q1; ax(1, 3) = q2;
      const double ar[5] = {be, al, 1, al, be};
      for (int q = 0; q < 5; q++) ax(2, q) = ar[q];
      const double sz = zv[0] + zv[1] + zv[2] + zv[3] + zv[4];
      const double br2[6] = {zv[0], zv[1], -sz, zv[2], zv[3], zv[4]};
      for (int q = 0; q < 6; q++) bx(2, q) = br2[q];
      for (int i = 3; i <= n - 4; i++) {
        const double br[7] = {zc, zb, za, -2 * (za + zb + zc), za, zb, zc};
        for (int q = 0; q < 5; q++) ax(i, i - 2 + q) = ar[q];
        for (int q = 0; q < 7; q++) bx(i, i - 3 + q) = br[q];
      }
    }
    for (int r = 0; r < 3; r++)  // mirrored end rows
      for (int q = 0; q < n; q++) {
        ax(n - 1 - r, n - 1 - q) = ax(r, q);
        bx(n - 1 - r, n - 1 - q) = lp * bx(r, q);
      }
    Dense sx = inverse(ax), rx = ax;
    int i = n / 2 - 2;  // 1-based ie/2-1
    rx(i, i + 2) = 0; rx(i + 1, i + 2) = 0; rx(i + 1, i + 3) = 0;
    i = n / 2 + 1;      // 1-based ie/2+2
    rx(i, i - 2) = 0; rx(i - 1, i - 2) = 0; rx(i - 1, i - 3) = 0;
    Dense cx = mul(rx, mul(sx, bx));
    for (int j = 0; j <= 1; j++) {
      const int row = n / 2 + j;  // 1-based ie/2+1 and ie/2+2
      for (int q = 0; q <= ll; q++) {
        S.pbco[nt][j][ll - q] = cx(row, q);
        S.pbci[nt][j][q] = cx(row, ll + 1 + q);
      }
      double s = 0;
      for (int q = 0; q <= ll; q++) s += S.pbco[nt][j][q];
      S.pbcot[nt][j] = s;
    }
  }
  // filte constants (src/Subroutines3D.f90:148-150)
  S.fex[1] = 45 / 30.0; S.fex[2] = -9 / 30.0; S.fex[3] = 1 / 30.0;
  const double l2 = 8 * std::log(2.0);
  S.ffx[1] = 4 / l2; S.ffx[2] = 6 / l2; S.ffx[3] = 7 / l2;
  // GCBC weights (src/Main3D.f90:443-459)
  {
    Dense cb(MBCI);
    cb(0, 0) = H.albed[0][0][3]; cb(0, 1) = H.albed[0][0][4];
    cb(1, 0) = H.albed[0][1][2]; cb(1, 1) = H.albed[0][1][3]; cb(1, 2) = H.albed[0][1][4];
    cb(2, 0) = H.albed[0][2][1]; cb(2, 1) = H.albed[0][2][2]; cb(2, 2) = H.albed[0][2][3];
    const double rb[3] = {1.0, H.albed[0][1][1], H.albed[0][2][0]};
    Dense ci = inverse(cb);
    for (int r = 0; r < MBCI; r++) {
      double s = 0;
      for (int q = 0; q < MBCI; q++) s += ci(r, q) * rb[q];
      H.sbci[r + 1] = -s;
    }
    const double f = pi / (MBCI + 1);
    double res = 0.0;
    for (int r = 1; r <= MBCI; r++) {
      res += 1.0;
      H.sbci[r] = 0.5 * H.sbci[r] * (1.0 + std::cos(res * f));
    }
    H.sbci[0] = 1.0;
  }
  // physics (src/MainVar3D.f90:27-32, src/Main3D.f90:60-63)
  S.pi = pi;
  S.gam = 1.4; S.gamm1 = S.gam - 1.0; S.ham = 1.0 / S.gam; S.hamm1 = 1.0 / S.gamm1;
  S.gamm1prndtli = 1.0 / (S.gamm1 * 0.71);
  S.tgamm1prndtli = 1.0 / (S.gamm1 * 0.99);
  S.two_three = 2.0 / 3.0;
  S.rhooo = 1.0; S.poo = 1.0 / S.gam;
  const double aoo = std::sqrt(S.gam * S.poo / S.rhooo);
  S.amachoo = std::sqrt(cfg.amach1 * cfg.amach1 + cfg.amach2 * cfg.amach2 + cfg.amach3 * cfg.amach3);
  S.srefoo = 111 / cfg.tempoo;
  S.srefp1dre = (S.srefoo + 1.0) / cfg.reoo;
  S.uoo[1] = cfg.amach1 * aoo; S.uoo[2] = cfg.amach2 * aoo; S.uoo[3] = cfg.amach3 * aoo;
  S.cfl = cfg.cfl; S.dto = cfg.dto; S.timf = cfg.timf; S.wtemp = cfg.wtemp;
  S.aoa0 = cfg.aoa0; S.aoa1 = cfg.aoa1; S.tps = cfg.tps; S.tp = cfg.tp;
  S.smago1 = cfg.smago1; S.smago2 = cfg.smago2;
  S.nkrk = cfg.nkrk; S.nviscous = cfg.nviscous; S.nsmf = cfg.nsmf; S.les = cfg.les;
}

void penta_factors(const double albes[3][5], const double albee[3][5], double al, double be, int len, double *fac) {
  // src/Subroutineso.f90:15-67 on positions 0..len-1; fac[i*5 + {l1,l2,u1,u2,u3}]
  std::vector<double> xu1(len, 1.0), xu2(len, 1.0), xu3(len, 1.0), xl1(len, 1.0), xl2(len, 1.0);
  auto AS = [&](int o, int r) { return albes[r][o + 2]; };
  auto AE = [&](int o, int r) { return albee[r][o + 2]; };
  const int is = 0, ie = len - 1;
  int i = is;
  xu1[i] = 1.0; xu2[i] = AS(1, 0); xu3[i] = AS(2, 0);
  i = is + 1;
  xl2[i] = AS(-1, 1) * xu1[i - 1];
  xu1[i] = 1.0 / (1.0 - xu2[i - 1] * xl2[i]);
  xu2[i] = AS(1, 1) - xu3[i - 1] * xl2[i];
  xu3[i] = AS(2, 1);
  i = is + 2;
  xl1[i] = AS(-2, 2) * xu1[i - 2];
  xl2[i] = (AS(-1, 2) - xu2[i - 2] * xl1[i]) * xu1[i - 1];
  xu1[i] = 1.0 / (1.0 - xu3[i - 2] * xl1[i] - xu2[i - 1] * xl2[i]);
  xu2[i] = AS(1, 2) - xu3[i - 1] * xl2[i];
  xu3[i] = AS(2, 2);
  for (i = is + 3; i <= ie - 3; i++) {
    xl1[i] = be * xu1[i - 2];
    xl2[i] = (al - xu2[i - 2] * xl1[i]) * xu1[i - 1];
    xu1[i] = 1.0 / (1.0 - xu3[i - 2] * xl1[i] - xu2[i - 1] * xl2[i]);
    xu2[i] = al - xu3[i - 1] * xl2[i];
    xu3[i] = be;
  }
  const int rows[3] = {ie - 2, ie - 1, ie};
  for (int r = 0; r < 3; r++) {
    const int k = 2 - r;  // boundary row index of the mirrored end
    i = rows[r];
    xl1[i] = AE(2, k) * xu1[i - 2];
    xl2[i] = (AE(1, k) - xu2[i - 2] * xl1[i]) * xu1[i - 1];
    xu1[i] = 1.0 / (1.0 - xu3[i - 2] * xl1[i] - xu2[i - 1] * xl2[i]);
    if (r < 2) xu2[i] = AE(-1, k) - xu3[i - 1] * xl2[i];
    if (r == 0) xu3[i] = AE(-2, k);
  }
  for (i = 0; i < len; i++) {
    fac[i * 5 + 0] = xl1[i];
    fac[i * 5 + 1] = xl2[i];
    fac[i * 5 + 2] = xu1[i];
    fac[i * 5 + 3] = xu2[i] * xu1[i];
    fac[i * 5 + 4] = xu3[i] * xu1[i];
  }
}

}  // namespace ati
