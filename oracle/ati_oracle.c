/*
 * ati_oracle.c — CPU restatement (C99, FP64, OpenMP over lines and points)
 * of the ATI3D per-Runge–Kutta-stage path of rpt1g12/tandemProject.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path and the timed CPU
 * baseline.  Nothing in the product links or calls it.
 *
 * PARITY UNPINNED against the reference itself: the Fortran reference cannot
 * be compiled here (no Fortran compiler or MPI) and ships no tests or golden
 * outputs.  This file follows the reference's loops and expression order
 * statement by statement (each function cites the lines it restates); it is
 * pinned by known-answer tests derived from the source and by an independent
 * dense-matrix numpy restatement of the line operators.
 *
 * Compile with -ffp-contract=off so that x86 and Arm give identical results
 * (no fused multiply-add contraction, as in the Fortran expressions).
 *
 * Multi-block: the reference runs one MPI rank per block (npc = 1).  Here all
 * blocks live in one process; each MPI exchange becomes a copy between the
 * blocks' face buffers with the reference's tag matching (a face ip receives
 * what the neighbour sent from its face 1-ip).
 */
#include "ati_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- constants: src/MainVar3D.f90:18-68 ---------------------------------- */
#define LMD 11
#define LMF 8
#define LMP 11
#define MBCI 3
#define NTDRV 0
#define NTFLT 1
#define NRALL 0
#define NRONE 1
#define N45NO 0
#define N45GO 1

static const double zero = 0.0, one = 1.0, two = 2.0, three = 3.0, half = 0.5;
static double pi, gam, gamm1, ham, hamm1, prndtl, gamm1prndtli, tgamm1prndtli, two_three, sml;

static const double alpha = 0.5862704032801503;
static const double beta = 0.09549533555017055;
static const double aa = 0.6431406736919156;
static const double ab = 0.2586011023495066;
static const double ac = 0.007140953479797375;
static const double beta20 = 0.03250008295108466;
static const double alpha21 = 0.3998040493524358;
static const double alpha23 = 0.7719261277615860;
static const double beta24 = 0.1626635931256900;
static const double a20 = -0.1219006056449124;
static const double a21 = -0.6301651351188667;
static const double a23 = 0.6521195063966084;
static const double a24 = 0.3938843551210350;
static const double a25 = 0.01904944407973912;
static const double a26 = -0.001027260523947668;
static const double alpha10 = 0.08360703307833438;
static const double alpha12 = 2.058102869495757;
static const double beta13 = 0.9704052014790193;
static const double a10 = -0.3177447290722621;
static const double a12 = -0.02807631929593225;
static const double a13 = 1.593461635747659;
static const double a14 = 0.2533027046976367;
static const double a15 = -0.03619652460174756;
static const double a16 = 0.004080281419108407;
static const double alpha01 = 5.912678614078549;
static const double beta02 = 3.775623951744012;
static const double a01 = -3.456878182643609;
static const double a02 = 5.839043358834730;
static const double a03 = 1.015886726041007;
static const double a04 = -0.2246526470654333;
static const double a05 = 0.08564940889936562;
static const double a06 = -0.01836710059356763;

static void init_constants(void) {
  pi = acos(-one);
  gam = 1.4;
  gamm1 = gam - one;
  ham = one / gam;
  hamm1 = one / gamm1;
  prndtl = 0.71;
  gamm1prndtli = one / (gamm1 * prndtl);
  tgamm1prndtli = 1.0 / (gamm1 * 0.99);
  two_three = two / three;
  sml = 1.0e-6;
}

static int g_threads = 0;
void orc_set_threads(int n) { g_threads = n; }
int orc_get_threads(void) {
#ifdef _OPENMP
  return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
  return 1;
#endif
}
#ifdef _OPENMP
#define OMP_NT num_threads(orc_get_threads())
#endif

/* ---- data ----------------------------------------------------------------- */
typedef struct {
  int lxi, let, lze;
  long np; /* lmx + 1 */
  int lim;
  int ijk[4][4];      /* ijk[c][nn], 1-based as ijk(c,nn) */
  long nbsize[4];
  int nbc[2][4], ncd[2][4], ndf[2][2][4];
  int nbcs[4], nbce[4];
  double *qo, *qa, *de, *xim, *etm, *zem, *rr, *ss, *p, *yaco, *xyz;
  double *tau; /* 9 planes: txx,tyy,tzz,txy,tyz,tzx,hxx,hyy,hzz */
  double *xu, *xl, *yu, *yl;
  double *drva[4], *drvb[4], *send[4], *recv[4], *cm[4];
  double *sbcc;
  long nsbcc;
  double *rpex;
  long nrpex;
  double *asz, *bsz; /* dense sponge coefficients */
  /* wall data (wallArea/walldir) */
  int wflag;
  long nwall;
  long *lwall;
  double *area, *wnor;
  int grid_set;
} OBlock;

struct orc_case {
  ati_config_t cfg;
  int nb, bkx, bky, bkz, mbk;
  OBlock *b;
  /* scheme coefficients */
  double abc[3][6];             /* abc(0:5,r) -> abc[r][c] */
  double albed[2][3][5];        /* albed(-2:2,row,ns) -> [ns][row][off+2] */
  double albef[2][3][5];
  double pbci[2][2][LMP + 1];   /* pbci(i,j,nt) -> [nt][j][i] */
  double pbco[2][2][LMP + 1];
  double pbcot[2][2];           /* pbcot(j,nt) -> [nt][j] */
  double fam[3], fbm[3], fcm[3], fa, fb, fc, alphf, betf;
  double sbci[MBCI + 1];
  double fex[4], ffx[4];
  /* freestream and time state */
  double rhooo, poo, aoo, amachoo, srefoo, srefp1dre, fltk, fltkbc;
  double uoo[4], umf[4], dudtmf[4], aoa;
  long n, ndt;
  double dt, dts, dte, timo;
  int inited;
  /* inflow turbulence (no counterpart in the reference, whose eddy generator is off): the mode table of the
   * GPU library, summed in FP64; the gust points and their velocity, held between evaluations */
  int nmodes;
  double *modes;          /* 8 per mode: k_x, k_y, k_z, s_x, s_y, s_z, a, psi */
  long ngust;
  int *gblk;              /* block of gust point q */
  long *gl;               /* its point in the block */
  double *gx, *gatz, *gv; /* x, y, z (3 per point), atz, velocity (3 per point) */
  long *gidx;             /* per block, dense: gust index of each point or -1 (block offsets in goff) */
  long *goff;
  long steps_done;
};

#define F(ptr, np, l, m) (ptr)[(size_t)((m) - 1) * (size_t)(np) + (size_t)(l)]

static long indx3(const OBlock *b, int i, int j, int k, int nn) {
  /* src/Subroutineso.f90:364-375 */
  switch (nn) {
    case 1: return ((long)k * (b->let + 1) + j) * (b->lxi + 1) + i;
    case 2: return ((long)j * (b->let + 1) + i) * (b->lxi + 1) + k;
    default: return ((long)i * (b->let + 1) + k) * (b->lxi + 1) + j;
  }
}

static int line_start(const OBlock *b, int nn) {
  /* is for direction nn in the concatenated factor index (src/Subroutines3D.f90:90-94) */
  return nn == 1 ? 0 : (nn == 2 ? b->lxi + 1 : b->lxi + b->let + 2);
}

/* ---- src/Subroutineso.f90:15-67 penta ------------------------------------ */
static void penta(double *xu, double *xl, int lim1, const double albes[3][5], const double albee[3][5],
                  double al, double be, int is, int ie) {
#define XU(i, c) xu[(i) + (size_t)lim1 * ((c) - 1)]
#define XL(i, c) xl[(i) + (size_t)lim1 * ((c) - 1)]
#define AS(o, r) albes[r][(o) + 2]
#define AE(o, r) albee[r][(o) + 2]
  int i;
  for (i = is; i <= ie; i++) {
    XL(i, 1) = one; XL(i, 2) = one;
    XU(i, 1) = one; XU(i, 2) = one; XU(i, 3) = one;
  }
  i = is;
  XU(i, 1) = one; XU(i, 2) = AS(1, 0); XU(i, 3) = AS(2, 0);
  i = is + 1;
  XL(i, 2) = AS(-1, 1) * XU(i - 1, 1);
  XU(i, 1) = one / (one - XU(i - 1, 2) * XL(i, 2));
  XU(i, 2) = AS(1, 1) - XU(i - 1, 3) * XL(i, 2);
  XU(i, 3) = AS(2, 1);
  i = is + 2;
  XL(i, 1) = AS(-2, 2) * XU(i - 2, 1);
  XL(i, 2) = (AS(-1, 2) - XU(i - 2, 2) * XL(i, 1)) * XU(i - 1, 1);
  XU(i, 1) = one / (one - XU(i - 2, 3) * XL(i, 1) - XU(i - 1, 2) * XL(i, 2));
  XU(i, 2) = AS(1, 2) - XU(i - 1, 3) * XL(i, 2);
  XU(i, 3) = AS(2, 2);
  for (i = is + 3; i <= ie - 3; i++) {
    XL(i, 1) = be * XU(i - 2, 1);
    XL(i, 2) = (al - XU(i - 2, 2) * XL(i, 1)) * XU(i - 1, 1);
    XU(i, 1) = one / (one - XU(i - 2, 3) * XL(i, 1) - XU(i - 1, 2) * XL(i, 2));
    XU(i, 2) = al - XU(i - 1, 3) * XL(i, 2);
    XU(i, 3) = be;
  }
  i = ie - 2;
  XL(i, 1) = AE(2, 2) * XU(i - 2, 1);
  XL(i, 2) = (AE(1, 2) - XU(i - 2, 2) * XL(i, 1)) * XU(i - 1, 1);
  XU(i, 1) = one / (one - XU(i - 2, 3) * XL(i, 1) - XU(i - 1, 2) * XL(i, 2));
  XU(i, 2) = AE(-1, 2) - XU(i - 1, 3) * XL(i, 2);
  XU(i, 3) = AE(-2, 2);
  i = ie - 1;
  XL(i, 1) = AE(2, 1) * XU(i - 2, 1);
  XL(i, 2) = (AE(1, 1) - XU(i - 2, 2) * XL(i, 1)) * XU(i - 1, 1);
  XU(i, 1) = one / (one - XU(i - 2, 3) * XL(i, 1) - XU(i - 1, 2) * XL(i, 2));
  XU(i, 2) = AE(-1, 1) - XU(i - 1, 3) * XL(i, 2);
  i = ie;
  XL(i, 1) = AE(2, 0) * XU(i - 2, 1);
  XL(i, 2) = (AE(1, 0) - XU(i - 2, 2) * XL(i, 1)) * XU(i - 1, 1);
  XU(i, 1) = one / (one - XU(i - 2, 3) * XL(i, 1) - XU(i - 1, 2) * XL(i, 2));
  for (i = is; i <= ie; i++) {
    XU(i, 2) = XU(i, 2) * XU(i, 1);
    XU(i, 3) = XU(i, 3) * XU(i, 1);
  }
#undef XU
#undef XL
#undef AS
#undef AE
}

/* ---- src/Subroutineso.f90:91-103 fcint ---------------------------------- */
static void fcint(double fltk, double fltr, double *alphz, double *betz, double *za, double *zb, double *zc) {
  double c1 = cos(fltk), c2 = cos(2 * fltk), c3 = cos(3 * fltk);
  double fctr = 1 / (30 + 5 * (7 - 16 * fltr) * c1 + 2 * (1 + 8 * fltr) * c2 - 3 * c3);
  *alphz = fctr * (20 * (2 * fltr - 1) - 30 * c1 + 12 * (2 * fltr - 1) * c2 - 2 * c3);
  *betz = half * fctr * (2 * (13 - 8 * fltr) + (33 - 48 * fltr) * c1 + 6 * c2 - c3);
  double ch = cos(half * fltk);
  double ch2 = ch * ch;
  *za = 60 * (1 - fltr) * (ch2 * ch2) * fctr;
  *zb = -2 * (*za) / 5;
  *zc = (*za) / 15;
}

/* ---- src/Subroutineso.f90:71-87 fcbcm ----------------------------------- */
static void fcbcm(double fltk, double fltkbc, double albef0[3][5], double fa_[3], double fb_[3], double fc_[3]) {
  double alphz, betz, za, zb, zc, fctr;
  double res = (fltkbc - fltk) / 9, ra2 = fltk + res, ra1 = fltk + 4 * res, ra0 = fltk + 9 * res;
  fcint(ra0, half, &alphz, &betz, &za, &zb, &zc);
  fctr = one / (one + alphz / 2 + betz / 4);
  albef0[0][0] = zero; albef0[0][1] = zero; albef0[0][2] = one; albef0[0][3] = alphz * fctr; albef0[0][4] = betz * fctr;
  fa_[0] = za * fctr; fb_[0] = zb * fctr; fc_[0] = zc * fctr;
  fcint(ra1, half, &alphz, &betz, &za, &zb, &zc);
  albef0[1][0] = zero; albef0[1][1] = alphz + betz / 2; albef0[1][2] = one; albef0[1][3] = alphz; albef0[1][4] = betz;
  fa_[1] = za; fb_[1] = zb; fc_[1] = zc;
  fcint(ra2, half, &alphz, &betz, &za, &zb, &zc);
  albef0[2][0] = betz; albef0[2][1] = alphz; albef0[2][2] = one; albef0[2][3] = alphz; albef0[2][4] = betz;
  fa_[2] = za; fb_[2] = zb; fc_[2] = zc;
}

/* ---- src/Subroutineso.f90:163-188 mtrxi (Gauss-Jordan, partial pivoting) - */
static void mtrxi(const double *ax, double *sx, int n) {
  /* column-major n x n, 0-based indices for rows/cols 1..n of the reference */
#define A(r, c) rx[(r) + (size_t)n * (c)]
  double *rx = (double *)malloc(sizeof(double) * n * n);
  double *temp = (double *)malloc(sizeof(double) * n);
  int *ipvt = (int *)malloc(sizeof(int) * n);
  memcpy(rx, ax, sizeof(double) * n * n);
  for (int i = 0; i < n; i++) ipvt[i] = i;
  for (int i = 0; i < n; i++) {
    int m = i;
    double best = fabs(A(i, i));
    for (int r = i + 1; r < n; r++)
      if (fabs(A(r, i)) > best) { best = fabs(A(r, i)); m = r; }
    if (m != i) {
      int t = ipvt[m]; ipvt[m] = ipvt[i]; ipvt[i] = t;
      for (int c = 0; c < n; c++) { double s = A(m, c); A(m, c) = A(i, c); A(i, c) = s; }
    }
    double ra0 = one / A(i, i);
    for (int r = 0; r < n; r++) temp[r] = A(r, i);
    for (int j = 0; j < n; j++) {
      double ra1 = ra0 * A(i, j);
      for (int r = 0; r < n; r++) A(r, j) = A(r, j) - ra1 * temp[r];
      A(i, j) = ra1;
    }
    for (int r = 0; r < n; r++) A(r, i) = -ra0 * temp[r];
    A(i, i) = ra0;
  }
  for (int c = 0; c < n; c++)
    for (int r = 0; r < n; r++) sx[r + (size_t)n * ipvt[c]] = A(r, c);
  free(rx); free(temp); free(ipvt);
#undef A
}

static void matmul(const double *a, const double *b, double *c, int n) {
  /* c = a*b, column-major, summed in index order */
  for (int j = 0; j < n; j++)
    for (int i = 0; i < n; i++) {
      double s = 0;
      for (int k = 0; k < n; k++) s += a[i + (size_t)n * k] * b[k + (size_t)n * j];
      c[i + (size_t)n * j] = s;
    }
}

/* ---- src/Subroutineso.f90:107-159 sbcco ---------------------------------- */
static void sbcco(orc_case *c) {
  for (int nt = 0; nt <= 1; nt++) {
    int lp = 2 * nt - 1, ll = nt == 0 ? LMD : LMF, ie = 2 * (ll + 1), n = ie;
    double *ax = (double *)calloc((size_t)n * n, sizeof(double));
    double *bx = (double *)calloc((size_t)n * n, sizeof(double));
    double *rx = (double *)calloc((size_t)n * n, sizeof(double));
    double *sx = (double *)calloc((size_t)n * n, sizeof(double));
    double *tx = (double *)calloc((size_t)n * n, sizeof(double));
#define AX(r, cc) ax[((r) - 1) + (size_t)n * ((cc) - 1)]
#define BX(r, cc) bx[((r) - 1) + (size_t)n * ((cc) - 1)]
#define RX(r, cc) rx[((r) - 1) + (size_t)n * ((cc) - 1)]
    int is = 1;
    if (nt == 0) {
      double s0 = 0, s1 = 0, s2 = 0;
      for (int q = 0; q < 6; q++) { s0 += c->abc[0][q]; }
      for (int q = 0; q < 6; q++) { s1 += c->abc[1][q]; }
      for (int q = 0; q < 6; q++) { s2 += c->abc[2][q]; }
      for (int q = 0; q <= 2; q++) AX(is, is + q) = c->albed[0][0][q + 2];
      double b0[7] = {-s0, a01, a02, a03, a04, a05, a06};
      for (int q = 0; q < 7; q++) BX(is, is + q) = b0[q];
      for (int q = 0; q <= 3; q++) AX(is + 1, is + q) = c->albed[0][1][q - 1 + 2];
      double b1[7] = {a10, -s1, a12, a13, a14, a15, a16};
      for (int q = 0; q < 7; q++) BX(is + 1, is + q) = b1[q];
      for (int q = 0; q <= 4; q++) AX(is + 2, is + q) = c->albed[0][2][q];
      double b2[7] = {a20, a21, -s2, a23, a24, a25, a26};
      for (int q = 0; q < 7; q++) BX(is + 2, is + q) = b2[q];
      for (int i = is + 3; i <= ie - 3; i++) {
        double ar[5] = {beta, alpha, one, alpha, beta};
        double br[7] = {-ac, -ab, -aa, zero, aa, ab, ac};
        for (int q = 0; q < 5; q++) AX(i, i - 2 + q) = ar[q];
        for (int q = 0; q < 7; q++) BX(i, i - 3 + q) = br[q];
      }
    } else {
      double alphz, betz, za, zb, zc;
      fcint(c->fltk, half, &alphz, &betz, &za, &zb, &zc);
      double zv[5] = {zb + 5 * zc, za - 10 * zc, za - 5 * zc, zb + zc, zc};
      double A2 = alphz * alphz, A3 = alphz * alphz * alphz, B2 = betz * betz, B3 = betz * betz * betz;
      double fctr = 1 / (1 + 5 * A3 + A2 * (8 + 22 * betz) + betz * (5 + 4 * betz + 60 * B2) +
                         5 * alphz * (1 + betz * (3 + 10 * betz)));
      double ra0 = (alphz * (1 + alphz) * (1 + 4 * alphz) + 2 * alphz * (7 + 3 * alphz) * betz +
                    24 * (1 - alphz) * B2 - 80 * B3) * fctr;
      double ra1 = (A3 + betz + 14 * A2 * betz + 60 * B3 + alphz * betz * (3 + 46 * betz)) * fctr;
      AX(is, is) = one; AX(is, is + 1) = ra0; AX(is, is + 2) = ra1;
      fctr = 1 / (1 + A2 * (9 - 5 * betz) + alphz * (5 + (35 - 29 * betz) * betz) +
                  betz * (5 + 6 * (9 - 10 * betz) * betz));
      ra0 = (9 * A3 + 10 * B2 * (8 * betz - 1) + 5 * A2 * (1 + 8 * betz) + alphz * (1 + betz * (4 + 81 * betz))) * fctr;
      ra1 = (alphz * (1 + alphz * (5 + 9 * alphz)) + alphz * (5 + 36 * alphz) * betz + (55 * alphz - 1) * B2 +
             10 * B3) * fctr;
      double ra2 = betz * (1 + alphz * (5 + 9 * alphz) + 5 * betz + 35 * alphz * betz + 50 * B2) * fctr;
      AX(is + 1, is) = ra0; AX(is + 1, is + 1) = one; AX(is + 1, is + 2) = ra1; AX(is + 1, is + 3) = ra2;
      double ar[5] = {betz, alphz, one, alphz, betz};
      for (int q = 0; q < 5; q++) AX(is + 2, is + q) = ar[q];
      double sz = 0;
      for (int q = 0; q < 5; q++) sz += zv[q];
      double br2[6] = {zv[0], zv[1], -sz, zv[2], zv[3], zv[4]};
      for (int q = 0; q < 6; q++) BX(is + 2, is + q) = br2[q];
      for (int i = is + 3; i <= ie - 3; i++) {
        double br[7] = {zc, zb, za, -2 * (za + zb + zc), za, zb, zc};
        for (int q = 0; q < 5; q++) AX(i, i - 2 + q) = ar[q];
        for (int q = 0; q < 7; q++) BX(i, i - 3 + q) = br[q];
      }
    }
    /* mirrored end rows (src/Subroutineso.f90:144-146) */
    for (int q = 1; q <= n; q++) {
      AX(ie - 2, ie - q + 1) = AX(is + 2, q);
      BX(ie - 2, ie - q + 1) = lp * BX(is + 2, q);
      AX(ie - 1, ie - q + 1) = AX(is + 1, q);
      BX(ie - 1, ie - q + 1) = lp * BX(is + 1, q);
      AX(ie, ie - q + 1) = AX(is, q);
      BX(ie, ie - q + 1) = lp * BX(is, q);
    }
    mtrxi(ax, sx, n);
    memcpy(rx, ax, sizeof(double) * n * n);
    int i = ie / 2 - 1;
    RX(i, i + 2) = 0; RX(i + 1, i + 2) = 0; RX(i + 1, i + 3) = 0;
    i = ie / 2 + 2;
    RX(i, i - 2) = 0; RX(i - 1, i - 2) = 0; RX(i - 1, i - 3) = 0;
    matmul(sx, bx, tx, n);
    matmul(rx, tx, ax, n);
    i = ie / 2 + 1;
    for (int q = 0; q <= ll; q++) c->pbco[nt][0][ll - q] = AX(i, is + q);
    for (int q = 0; q <= ll; q++) c->pbci[nt][0][q] = AX(i, is + ll + 1 + q);
    i = ie / 2 + 2;
    for (int q = 0; q <= ll; q++) c->pbco[nt][1][ll - q] = AX(i, is + q);
    for (int q = 0; q <= ll; q++) c->pbci[nt][1][q] = AX(i, is + ll + 1 + q);
#undef AX
#undef BX
#undef RX
    free(ax); free(bx); free(rx); free(sx); free(tx);
  }
}

/* ---- scheme set-up: src/Main3D.f90:60-73, 295-312, 443-459 ---------------- */
static void scheme_setup(orc_case *c) {
  double r0[6] = {a01, a02, a03, a04, a05, a06};
  double r1[6] = {a10, a12, a13, a14, a15, a16};
  double r2[6] = {a20, a21, a23, a24, a25, a26};
  memcpy(c->abc[0], r0, sizeof r0); memcpy(c->abc[1], r1, sizeof r1); memcpy(c->abc[2], r2, sizeof r2);
  double d00[5] = {zero, zero, one, alpha01, beta02};
  double d01[5] = {zero, alpha10, one, alpha12, beta13};
  double d02[5] = {beta20, alpha21, one, alpha23, beta24};
  double d10[5] = {zero, zero, one, alpha, beta};
  double d11[5] = {zero, alpha, one, alpha, beta};
  double d12[5] = {beta, alpha, one, alpha, beta};
  memcpy(c->albed[0][0], d00, sizeof d00); memcpy(c->albed[0][1], d01, sizeof d01);
  memcpy(c->albed[0][2], d02, sizeof d02); memcpy(c->albed[1][0], d10, sizeof d10);
  memcpy(c->albed[1][1], d11, sizeof d11); memcpy(c->albed[1][2], d12, sizeof d12);
  fcbcm(c->fltk, c->fltkbc, c->albef[0], c->fam, c->fbm, c->fcm);
  fcint(c->fltk, half, &c->alphf, &c->betf, &c->fa, &c->fb, &c->fc);
  double f0[5] = {zero, zero, one, c->alphf, c->betf};
  double f1[5] = {zero, c->alphf, one, c->alphf, c->betf};
  double f2[5] = {c->betf, c->alphf, one, c->alphf, c->betf};
  memcpy(c->albef[1][0], f0, sizeof f0); memcpy(c->albef[1][1], f1, sizeof f1);
  memcpy(c->albef[1][2], f2, sizeof f2);
  memset(c->pbci, 0, sizeof c->pbci);
  memset(c->pbco, 0, sizeof c->pbco);
  sbcco(c);
  for (int nt = 0; nt <= 1; nt++)
    for (int j = 0; j <= 1; j++) {
      int ii = LMD + nt * (LMF - LMD);
      double s = 0;
      for (int q = 0; q <= ii; q++) s += c->pbco[nt][j][q];
      c->pbcot[nt][j] = s;
    }
  /* filte: fex, ffx (src/Subroutines3D.f90:148-150), mfbi = 1 */
  c->fex[1] = 45 / (1 * 30.0); c->fex[2] = -9 / (1 * 30.0); c->fex[3] = 1 / (1 * 30.0);
  double l2 = 8 * log(two);
  c->ffx[1] = 4 / l2; c->ffx[2] = 6 / l2; c->ffx[3] = 7 / l2;
  /* GCBC weights (src/Main3D.f90:443-459) */
  double cbca[9] = {0}, cbcs[9], rbci[3];
#define CB(r, cc) cbca[((r) - 1) + 3 * ((cc) - 1)]
  CB(1, 1) = c->albed[0][0][1 + 2]; CB(1, 2) = c->albed[0][0][2 + 2];
  CB(2, 1) = c->albed[0][1][0 + 2]; CB(2, 2) = c->albed[0][1][1 + 2]; CB(2, 3) = c->albed[0][1][2 + 2];
  CB(3, 1) = c->albed[0][2][-1 + 2]; CB(3, 2) = c->albed[0][2][0 + 2]; CB(3, 3) = c->albed[0][2][1 + 2];
#undef CB
  rbci[0] = one; rbci[1] = c->albed[0][1][-1 + 2]; rbci[2] = c->albed[0][2][-2 + 2];
  mtrxi(cbca, cbcs, 3);
  for (int i = 0; i < 3; i++) {
    double s = 0;
    for (int k = 0; k < 3; k++) s += cbcs[i + 3 * k] * rbci[k];
    c->sbci[i + 1] = -s;
  }
  double fctr = pi / (MBCI + 1), res = zero;
  for (int i = 1; i <= MBCI; i++) {
    res = res + one;
    c->sbci[i] = half * c->sbci[i] * (one + cos(res * fctr));
  }
}

/* ---- topology: domdcomp (src/SingleTurbulence3D.f90:121-164) with npc = 1
 *      (src/Main3D.f90:148-178), ndf (src/Main3D.f90:322-327) ------------- */
static void domdcomp(orc_case *c, int mb, OBlock *b) {
  int bkx = c->bkx, bky = c->bky, mbk = c->mbk;
  int bcw = 20 + 5 * c->cfg.nviscous, bcinout = 10, bcperiod = 45, bcinter = 30;
  int ms[4], me[4];
  int ll = mb % bkx;
  if (ll == 0) { ms[1] = mb + (bkx - 1); me[1] = mb + 1; b->nbcs[1] = bcinout; b->nbce[1] = bcinter; }
  else if (ll == bkx - 1) { ms[1] = mb - 1; me[1] = mb - (bkx - 1); b->nbcs[1] = bcinter; b->nbce[1] = bcinout; }
  else { ms[1] = mb - 1; me[1] = mb + 1; b->nbcs[1] = bcinter; b->nbce[1] = bcinter; }
  if (mb < bkx) { ms[2] = mb + bkx * (bky - 1); me[2] = mb + bkx; b->nbcs[2] = bcinout; b->nbce[2] = bcinter; }
  else if (mb > mbk - bkx) { ms[2] = mb - bkx; me[2] = mb - bkx * (bky - 1); b->nbcs[2] = bcinter; b->nbce[2] = bcinout; }
  else { ms[2] = mb - bkx; me[2] = mb + bkx; b->nbcs[2] = bcinter; b->nbce[2] = bcinter; }
  b->nbcs[3] = bcperiod; b->nbce[3] = bcperiod; ms[3] = mb; me[3] = mb;
  if (mb == 1) b->nbce[2] = bcw;
  if (mb == 4) b->nbcs[2] = bcw;
  for (int nn = 1; nn <= 3; nn++) {
    b->nbc[0][nn] = b->nbcs[nn]; b->nbc[1][nn] = b->nbce[nn];
    b->ncd[0][nn] = ms[nn]; b->ncd[1][nn] = me[nn];
    for (int ip = 0; ip <= 1; ip++) {
      int np = b->nbc[ip][nn], v = 0;
      if (np == 35 || np == 40 || np == 45) v = 1;
      b->ndf[ip][0][nn] = v; b->ndf[ip][1][nn] = v;
    }
  }
}

static double *dalloc(size_t n) { return (double *)calloc(n ? n : 1, sizeof(double)); }

static int block_setup(orc_case *c, int mb) {
  OBlock *b = &c->b[mb];
  int i = mb % c->bkx, j = (mb / c->bkx) % c->bky, k = mb / (c->bkx * c->bky);
  b->lxi = c->cfg.lxibk[i]; b->let = c->cfg.letbk[j]; b->lze = c->cfg.lzebk[k];
  if (b->lxi < 6 || b->let < 6 || b->lze < 12) return ATI_EINVAL;
  domdcomp(c, mb, b);
  b->np = (long)(b->lxi + 1) * (b->let + 1) * (b->lze + 1);
  b->lim = (b->lxi + 1) + (b->let + 1) + (b->lze + 1) - 1;
  b->ijk[1][1] = b->lxi; b->ijk[2][1] = b->let; b->ijk[3][1] = b->lze;
  b->ijk[1][2] = b->let; b->ijk[2][2] = b->lze; b->ijk[3][2] = b->lxi;
  b->ijk[1][3] = b->lze; b->ijk[2][3] = b->lxi; b->ijk[3][3] = b->let;
  for (int nn = 1; nn <= 3; nn++) b->nbsize[nn] = (long)(b->ijk[2][nn] + 1) * (b->ijk[3][nn] + 1);
  size_t np = b->np;
  b->qo = dalloc(5 * np); b->qa = dalloc(5 * np); b->de = dalloc(5 * np);
  b->xim = dalloc(3 * np); b->etm = dalloc(3 * np); b->zem = dalloc(3 * np);
  b->rr = dalloc(3 * np); b->ss = dalloc(3 * np); b->p = dalloc(np); b->yaco = dalloc(np);
  b->xyz = dalloc(3 * np); b->tau = dalloc(9 * np); b->asz = dalloc(np); b->bsz = dalloc(np);
  int lim1 = b->lim + 1;
  b->xu = dalloc(3 * (size_t)lim1); b->xl = dalloc(2 * (size_t)lim1);
  b->yu = dalloc(3 * (size_t)lim1); b->yl = dalloc(2 * (size_t)lim1);
  for (int nn = 1; nn <= 3; nn++) {
    size_t nb = b->nbsize[nn];
    b->drva[nn] = dalloc(nb * 10); b->drvb[nn] = dalloc(nb * 10);
    b->send[nn] = dalloc(nb * 6); b->recv[nn] = dalloc(nb * 6); b->cm[nn] = dalloc(nb * 6);
  }
  if (!b->qo || !b->qa || !b->de || !b->tau) return ATI_ENOMEM;
  /* LU factors per direction (src/Main3D.f90:316-332) */
  for (int nn = 1; nn <= 3; nn++) {
    int is = line_start(b, nn), ie = is + b->ijk[1][nn];
    int ns = b->ndf[0][0][nn], ne = b->ndf[1][0][nn];
    penta(b->xu, b->xl, lim1, (const double(*)[5])c->albed[ns], (const double(*)[5])c->albed[ne], alpha, beta, is, ie);
    ns = b->ndf[0][1][nn]; ne = b->ndf[1][1][nn];
    penta(b->yu, b->yl, lim1, (const double(*)[5])c->albef[ns], (const double(*)[5])c->albef[ne], c->alphf, c->betf,
          is, ie);
  }
  return ATI_OK;
}

static void block_free(OBlock *b) {
  free(b->qo); free(b->qa); free(b->de); free(b->xim); free(b->etm); free(b->zem); free(b->rr); free(b->ss);
  free(b->p); free(b->yaco); free(b->xyz); free(b->tau); free(b->asz); free(b->bsz);
  free(b->xu); free(b->xl); free(b->yu); free(b->yl);
  for (int nn = 1; nn <= 3; nn++) { free(b->drva[nn]); free(b->drvb[nn]); free(b->send[nn]); free(b->recv[nn]); free(b->cm[nn]); }
  free(b->sbcc); free(b->rpex); free(b->lwall); free(b->area); free(b->wnor);
}

int orc_create(const ati_config_t *cfg, orc_case **out) {
  init_constants();
  if (!cfg || !out) return ATI_EINVAL;
  if (cfg->bkx != 3 || cfg->bky != 2 || cfg->bkz != 1) return ATI_EINVAL;
  if (cfg->nkrk < 1 || cfg->nkrk > 8) return ATI_EINVAL;
  orc_case *c = (orc_case *)calloc(1, sizeof(orc_case));
  c->cfg = *cfg;
  c->bkx = cfg->bkx; c->bky = cfg->bky; c->bkz = cfg->bkz;
  c->nb = c->bkx * c->bky * c->bkz; c->mbk = c->nb - 1;
  /* src/Main3D.f90:60-63 */
  c->fltk = pi * cfg->fltk; c->fltkbc = pi * cfg->fltkbc;
  c->rhooo = one; c->poo = one / gam; c->aoo = sqrt(gam * c->poo / c->rhooo);
  c->amachoo = sqrt(cfg->amach1 * cfg->amach1 + cfg->amach2 * cfg->amach2 + cfg->amach3 * cfg->amach3);
  c->srefoo = 111 / cfg->tempoo; c->srefp1dre = (c->srefoo + one) / cfg->reoo;
  c->uoo[1] = cfg->amach1 * c->aoo; c->uoo[2] = cfg->amach2 * c->aoo; c->uoo[3] = cfg->amach3 * c->aoo;
  c->aoa = cfg->aoa0;
  scheme_setup(c);
  c->b = (OBlock *)calloc(c->nb, sizeof(OBlock));
  for (int mb = 0; mb < c->nb; mb++) {
    int rc = block_setup(c, mb);
    if (rc) { orc_destroy(c); return rc; }
  }
  *out = c;
  return ATI_OK;
}

void orc_destroy(orc_case *c) {
  if (!c) return;
  if (c->b)
    for (int mb = 0; mb < c->nb; mb++) block_free(&c->b[mb]);
  free(c->b);
  free(c->modes); free(c->gblk); free(c->gl); free(c->gx); free(c->gatz); free(c->gv); free(c->gidx); free(c->goff);
  free(c);
}

int orc_nblocks(const orc_case *c) { return c->nb; }

int orc_block_dims(const orc_case *c, int blk, int32_t dims[3], int64_t *npts) {
  if (blk < 0 || blk >= c->nb) return ATI_EINVAL;
  dims[0] = c->b[blk].lxi; dims[1] = c->b[blk].let; dims[2] = c->b[blk].lze;
  if (npts) *npts = c->b[blk].np;
  return ATI_OK;
}

/* ---- mpigo: src/Subroutines3D.f90:16-80 ------------------------------------ */
static void mpigo_send(orc_case *c, OBlock *b, int nt, int nrt, int n45) {
  int mp = nt == 0 ? LMD : LMF;
  for (int nn = 1; nn <= 3; nn++) {
    int nz = (1 - nrt) * (nn - 1) + 1;
    double *send = b->send[nn];
    long nbs = b->nbsize[nn];
    for (int ip = 0; ip <= 1; ip++) {
      int is = ip * b->ijk[1][nn], ie = 1 - 2 * ip, ii = 0;
      double ra0 = zero;
      switch (b->nbc[ip][nn]) {
        case 35: ra0 = zero; ii = 1; break;
        case 40: ra0 = zero; ii = 0; break;
        case 45: ra0 = n45; ii = 1; break;
      }
      if (b->ndf[ip][nt][nn] != 1) continue;
      int K = b->ijk[3][nn], J = b->ijk[2][nn];
#pragma omp parallel for collapse(2) OMP_NT
      for (int k = 0; k <= K; k++)
        for (int j = 0; j <= J; j++) {
          long jk = (long)k * (J + 1) + j;
          long l = indx3(b, is, j, k, nn);
          double res = ra0 * F(b->rr, b->np, l, nz);
          double sap[LMP + 1];
          for (int i = 0; i <= mp; i++) {
            long l2 = indx3(b, is + ie * (i + ii), j, k, nn);
            sap[i] = F(b->rr, b->np, l2, nz);
          }
          double s0 = 0, s1 = 0;
          for (int i = 0; i <= mp; i++) s0 += c->pbco[nt][0][i] * sap[i];
          for (int i = 0; i <= mp; i++) s1 += c->pbco[nt][1][i] * sap[i];
          send[jk + nbs * (0 + 3 * ip)] = s0 - res * c->pbcot[nt][0];
          send[jk + nbs * (1 + 3 * ip)] = s1 - res * c->pbcot[nt][1];
          send[jk + nbs * (2 + 3 * ip)] = sap[0] - res;
        }
    }
  }
}

int orc_mpigo(orc_case *c, int nt, int nrt, int n45) {
  if (nt < 0 || nt > 1 || nrt < 0 || nrt > 1 || n45 < 0 || n45 > 1) return ATI_EINVAL;
  for (int mb = 0; mb < c->nb; mb++) mpigo_send(c, &c->b[mb], nt, nrt, n45);
  /* ISEND/IRECV pairing: face ip of block A receives what block ncd(ip) sent from its face 1-ip */
  for (int mb = 0; mb < c->nb; mb++) {
    OBlock *b = &c->b[mb];
    for (int nn = 1; nn <= 3; nn++)
      for (int ip = 0; ip <= 1; ip++) {
        if (b->ndf[ip][nt][nn] != 1) continue;
        OBlock *o = &c->b[b->ncd[ip][nn]];
        long nbs = b->nbsize[nn];
        int iq = 1 - ip;
        for (int q = 0; q < 3; q++)
          memcpy(b->recv[nn] + nbs * (q + 3 * ip), o->send[nn] + nbs * (q + 3 * iq), sizeof(double) * nbs);
      }
  }
  if (n45 == N45GO) {
    for (int mb = 0; mb < c->nb; mb++) {
      OBlock *b = &c->b[mb];
      for (int nn = 1; nn <= 3; nn++) {
        int nz = (1 - nrt) * (nn - 1) + 1;
        long nbs = b->nbsize[nn];
        for (int ip = 0; ip <= 1; ip++) {
          int is = ip * b->ijk[1][nn];
          if (b->nbc[ip][nn] != 45) continue;
          int K = b->ijk[3][nn], J = b->ijk[2][nn];
          for (int k = 0; k <= K; k++)
            for (int j = 0; j <= J; j++) {
              long jk = (long)k * (J + 1) + j;
              long l = indx3(b, is, j, k, nn);
              double v = F(b->rr, b->np, l, nz);
              double *r = b->recv[nn];
              r[jk + nbs * (0 + 3 * ip)] = r[jk + nbs * (0 + 3 * ip)] + v * c->pbcot[nt][0];
              r[jk + nbs * (1 + 3 * ip)] = r[jk + nbs * (1 + 3 * ip)] + v * c->pbcot[nt][1];
              r[jk + nbs * (2 + 3 * ip)] = r[jk + nbs * (2 + 3 * ip)] + v;
            }
        }
      }
    }
  }
  return ATI_OK;
}

/* ---- deriv: src/Subroutines3D.f90:84-141 ----------------------------------- */
static void deriv_blk(orc_case *c, OBlock *b, int nn, int nz, int m) {
  const int nt = 0, ns = b->ndf[0][0][nn], ne = b->ndf[1][0][nn];
  const int is = line_start(b, nn), ie = is + b->ijk[1][nn];
  const long nbs = b->nbsize[nn];
  const int lim1 = b->lim + 1;
  const double *xu = b->xu, *xl = b->xl, *recv = b->recv[nn];
  double *drva = b->drva[nn];
  const int K = b->ijk[3][nn], J = b->ijk[2][nn];
#define XU(i, cc) xu[(i) + (size_t)lim1 * ((cc) - 1)]
#define XL(i, cc) xl[(i) + (size_t)lim1 * ((cc) - 1)]
#pragma omp parallel OMP_NT
  {
    double *sa = (double *)malloc(sizeof(double) * lim1);
    double *sb = (double *)malloc(sizeof(double) * lim1);
    long *li = (long *)malloc(sizeof(long) * lim1);
#pragma omp for collapse(2)
    for (int k = 0; k <= K; k++)
      for (int j = 0; j <= J; j++) {
        long jk = (long)k * (J + 1) + j;
        for (int i = is; i <= ie; i++) {
          long l = indx3(b, i - is, j, k, nn);
          li[i] = l;
          sa[i] = F(b->rr, b->np, l, nz);
        }
        if (ns == 0) {
          double s;
          s = 0; { const int o[6] = {1, 2, 3, 4, 5, 6}; for (int q = 0; q < 6; q++) s += c->abc[0][q] * (sa[is + o[q]] - sa[is]); } sb[is] = s;
          s = 0; { const int o[6] = {0, 2, 3, 4, 5, 6}; for (int q = 0; q < 6; q++) s += c->abc[1][q] * (sa[is + o[q]] - sa[is + 1]); } sb[is + 1] = s;
          s = 0; { const int o[6] = {0, 1, 3, 4, 5, 6}; for (int q = 0; q < 6; q++) s += c->abc[2][q] * (sa[is + o[q]] - sa[is + 2]); } sb[is + 2] = s;
        } else {
          double s0 = 0, s1 = 0;
          for (int q = 0; q <= LMD; q++) s0 += c->pbci[nt][0][q] * sa[is + q];
          for (int q = 0; q <= LMD; q++) s1 += c->pbci[nt][1][q] * sa[is + q];
          sb[is] = s0 + recv[jk + nbs * (0 + 3 * 0)];
          sb[is + 1] = s1 + recv[jk + nbs * (1 + 3 * 0)];
          sb[is + 2] = aa * (sa[is + 3] - sa[is + 1]) + ab * (sa[is + 4] - sa[is]) +
                       ac * (sa[is + 5] - recv[jk + nbs * (2 + 3 * 0)]);
        }
        for (int i = is + 3; i <= ie - 3; i++)
          sb[i] = aa * (sa[i + 1] - sa[i - 1]) + ab * (sa[i + 2] - sa[i - 2]) + ac * (sa[i + 3] - sa[i - 3]);
        if (ne == 0) {
          double s;
          s = 0; { const int o[6] = {1, 2, 3, 4, 5, 6}; for (int q = 0; q < 6; q++) s += c->abc[0][q] * (sa[ie] - sa[ie - o[q]]); } sb[ie] = s;
          s = 0; { const int o[6] = {0, 2, 3, 4, 5, 6}; for (int q = 0; q < 6; q++) s += c->abc[1][q] * (sa[ie - 1] - sa[ie - o[q]]); } sb[ie - 1] = s;
          s = 0; { const int o[6] = {0, 1, 3, 4, 5, 6}; for (int q = 0; q < 6; q++) s += c->abc[2][q] * (sa[ie - 2] - sa[ie - o[q]]); } sb[ie - 2] = s;
        } else {
          double s0 = 0, s1 = 0;
          for (int q = 0; q <= LMD; q++) s0 += c->pbci[nt][0][q] * sa[ie - q];
          for (int q = 0; q <= LMD; q++) s1 += c->pbci[nt][1][q] * sa[ie - q];
          sb[ie] = -s0 - recv[jk + nbs * (0 + 3 * 1)];
          sb[ie - 1] = -s1 - recv[jk + nbs * (1 + 3 * 1)];
          sb[ie - 2] = aa * (sa[ie - 1] - sa[ie - 3]) + ab * (sa[ie] - sa[ie - 4]) +
                       ac * (recv[jk + nbs * (2 + 3 * 1)] - sa[ie - 5]);
        }
        sa[is] = sb[is];
        sa[is + 1] = sb[is + 1] - XL(is + 1, 2) * sa[is];
        for (int i = is + 2; i <= ie; i++) sa[i] = sb[i] - XL(i, 1) * sa[i - 2] - XL(i, 2) * sa[i - 1];
        sb[ie] = XU(ie, 1) * sa[ie];
        sb[ie - 1] = XU(ie - 1, 1) * sa[ie - 1] - XU(ie - 1, 2) * sb[ie];
        for (int i = ie - 2; i >= is; i--) sb[i] = XU(i, 1) * sa[i] - XU(i, 2) * sb[i + 1] - XU(i, 3) * sb[i + 2];
        for (int i = is; i <= ie; i++) F(b->rr, b->np, li[i], nn) = sb[i];
        drva[jk + nbs * ((m - 1) + 5 * 0)] = sb[is];
        drva[jk + nbs * ((m - 1) + 5 * 1)] = sb[ie];
      }
    free(sa); free(sb); free(li);
  }
#undef XU
#undef XL
}

int orc_deriv(orc_case *c, int nn, int nz, int m) {
  if (nn < 1 || nn > 3 || nz < 1 || nz > 3 || m < 1 || m > 5) return ATI_EINVAL;
  for (int mb = 0; mb < c->nb; mb++) deriv_blk(c, &c->b[mb], nn, nz, m);
  return ATI_OK;
}

/* ---- filte: src/Subroutines3D.f90:145-206 ---------------------------------- */
static void filte_blk(orc_case *c, OBlock *b, int nn, int nz) {
  const int nt = 1, ns = b->ndf[0][1][nn], ne = b->ndf[1][1][nn];
  const int is = line_start(b, nn), ie = is + b->ijk[1][nn];
  const long nbs = b->nbsize[nn];
  const int lim1 = b->lim + 1;
  const double *yu = b->yu, *yl = b->yl, *recv = b->recv[nn];
  const double *fex = c->fex, *ffx = c->ffx, *fam = c->fam, *fbm = c->fbm, *fcm = c->fcm;
  const double fa = c->fa, fb = c->fb, fc = c->fc;
  const int K = b->ijk[3][nn], J = b->ijk[2][nn];
#define YU(i, cc) yu[(i) + (size_t)lim1 * ((cc) - 1)]
#define YL(i, cc) yl[(i) + (size_t)lim1 * ((cc) - 1)]
#pragma omp parallel OMP_NT
  {
    double *sa = (double *)malloc(sizeof(double) * lim1);
    double *sb = (double *)malloc(sizeof(double) * lim1);
    long *li = (long *)malloc(sizeof(long) * lim1);
#pragma omp for collapse(2)
    for (int k = 0; k <= K; k++)
      for (int j = 0; j <= J; j++) {
        long jk = (long)k * (J + 1) + j;
        double ra0, ra1, ra2, res, rv[4];
        for (int i = is; i <= ie; i++) {
          long l = indx3(b, i - is, j, k, nn);
          li[i] = l;
          sa[i] = F(b->rr, b->np, l, nz);
        }
        if (ns == 0) {
          ra0 = two * sa[is]; ra1 = two * sa[is + 1]; ra2 = two * sa[is + 2];
          res = 0;
          for (int q = 1; q <= 3; q++) res += fex[q] * (sa[is + q] - sa[is]);
          for (int q = 1; q <= 3; q++) rv[q] = sa[is] - res * ffx[q];
          sb[is] = fam[0] * (rv[1] + sa[is + 1] - ra0) + fbm[0] * (rv[2] + sa[is + 2] - ra0) +
                   fcm[0] * (rv[3] + sa[is + 3] - ra0);
          sb[is + 1] = fam[1] * (sa[is] + sa[is + 2] - ra1) + fbm[1] * (rv[1] + sa[is + 3] - ra1) +
                       fcm[1] * (rv[2] + sa[is + 4] - ra1);
          sb[is + 2] = fam[2] * (sa[is + 1] + sa[is + 3] - ra2) + fbm[2] * (sa[is] + sa[is + 4] - ra2) +
                       fcm[2] * (rv[1] + sa[is + 5] - ra2);
        } else {
          ra2 = two * sa[is + 2];
          double s0 = 0, s1 = 0;
          for (int q = 0; q <= LMF; q++) s0 += c->pbci[nt][0][q] * sa[is + q];
          for (int q = 0; q <= LMF; q++) s1 += c->pbci[nt][1][q] * sa[is + q];
          sb[is] = s0 + recv[jk + nbs * (0 + 3 * 0)];
          sb[is + 1] = s1 + recv[jk + nbs * (1 + 3 * 0)];
          sb[is + 2] = fa * (sa[is + 1] + sa[is + 3] - ra2) + fb * (sa[is] + sa[is + 4] - ra2) +
                       fc * (recv[jk + nbs * (2 + 3 * 0)] + sa[is + 5] - ra2);
        }
        for (int i = is + 3; i <= ie - 3; i++) {
          res = two * sa[i];
          sb[i] = fa * (sa[i - 1] + sa[i + 1] - res) + fb * (sa[i - 2] + sa[i + 2] - res) +
                  fc * (sa[i - 3] + sa[i + 3] - res);
        }
        if (ne == 0) {
          ra0 = two * sa[ie]; ra1 = two * sa[ie - 1]; ra2 = two * sa[ie - 2];
          res = 0;
          for (int q = 1; q <= 3; q++) res += fex[q] * (sa[ie] - sa[ie - q]);
          for (int q = 1; q <= 3; q++) rv[q] = sa[ie] + res * ffx[q];
          sb[ie] = fam[0] * (sa[ie - 1] + rv[1] - ra0) + fbm[0] * (sa[ie - 2] + rv[2] - ra0) +
                   fcm[0] * (sa[ie - 3] + rv[3] - ra0);
          sb[ie - 1] = fam[1] * (sa[ie - 2] + sa[ie] - ra1) + fbm[1] * (sa[ie - 3] + rv[1] - ra1) +
                       fcm[1] * (sa[ie - 4] + rv[2] - ra1);
          sb[ie - 2] = fam[2] * (sa[ie - 3] + sa[ie - 1] - ra2) + fbm[2] * (sa[ie - 4] + sa[ie] - ra2) +
                       fcm[2] * (sa[ie - 5] + rv[1] - ra2);
        } else {
          ra2 = two * sa[ie - 2];
          double s0 = 0, s1 = 0;
          for (int q = 0; q <= LMF; q++) s0 += c->pbci[nt][0][q] * sa[ie - q];
          for (int q = 0; q <= LMF; q++) s1 += c->pbci[nt][1][q] * sa[ie - q];
          sb[ie] = s0 + recv[jk + nbs * (0 + 3 * 1)];
          sb[ie - 1] = s1 + recv[jk + nbs * (1 + 3 * 1)];
          sb[ie - 2] = fa * (sa[ie - 3] + sa[ie - 1] - ra2) + fb * (sa[ie - 4] + sa[ie] - ra2) +
                       fc * (sa[ie - 5] + recv[jk + nbs * (2 + 3 * 1)] - ra2);
        }
        sa[is] = sb[is];
        sa[is + 1] = sb[is + 1] - YL(is + 1, 2) * sa[is];
        for (int i = is + 2; i <= ie; i++) sa[i] = sb[i] - YL(i, 1) * sa[i - 2] - YL(i, 2) * sa[i - 1];
        sb[ie] = YU(ie, 1) * sa[ie];
        sb[ie - 1] = YU(ie - 1, 1) * sa[ie - 1] - YU(ie - 1, 2) * sb[ie];
        for (int i = ie - 2; i >= is; i--) sb[i] = YU(i, 1) * sa[i] - YU(i, 2) * sb[i + 1] - YU(i, 3) * sb[i + 2];
        for (int i = is; i <= ie; i++) F(b->rr, b->np, li[i], nz) = F(b->rr, b->np, li[i], nz) + sb[i];
      }
    free(sa); free(sb); free(li);
  }
#undef YU
#undef YL
}

int orc_filte(orc_case *c, int nn, int nz) {
  if (nn < 1 || nn > 3 || nz < 1 || nz > 3) return ATI_EINVAL;
  for (int mb = 0; mb < c->nb; mb++) filte_blk(c, &c->b[mb], nn, nz);
  return ATI_OK;
}

/* ---- characteristic helpers: src/Subroutines3D.f90:235-324 --------------- */
typedef struct { double rhoi, ao, aoi, ve[4], hv2, vn, vs; } Elem;

static void eleme(const orc_case *c, const OBlock *b, long l, const double cm[4], Elem *e) {
  e->rhoi = one / F(b->qa, b->np, l, 1);
  e->ao = sqrt(gam * e->rhoi * b->p[l]);
  e->aoi = one / e->ao;
  for (int q = 1; q <= 3; q++) e->ve[q] = e->rhoi * F(b->qa, b->np, l, q + 1);
  e->hv2 = half * (e->ve[1] * e->ve[1] + e->ve[2] * e->ve[2] + e->ve[3] * e->ve[3]);
  e->vn = cm[1] * e->ve[1] + cm[2] * e->ve[2] + cm[3] * e->ve[3];
  e->vs = cm[1] * c->umf[1] + cm[2] * c->umf[2] + cm[3] * c->umf[3];
}

static void xtq2r(const Elem *e, const double cm[4], double xt[6][6]) {
  double ho = gamm1 * e->aoi * e->aoi, bo = 1 - ho * e->hv2, co = e->aoi * e->vn;
  double dm[4], rv[4];
  for (int q = 1; q <= 3; q++) { dm[q] = e->aoi * cm[q]; rv[q] = ho * e->ve[q]; }
  const double *ve = e->ve;
  xt[1][1] = bo * cm[1] + dm[2] * ve[3] - dm[3] * ve[2];
  xt[1][2] = cm[1] * rv[1];
  xt[1][3] = cm[1] * rv[2] + dm[3];
  xt[1][4] = cm[1] * rv[3] - dm[2];
  xt[1][5] = -ho * cm[1];
  xt[2][1] = bo * cm[2] + dm[3] * ve[1] - dm[1] * ve[3];
  xt[2][2] = cm[2] * rv[1] - dm[3];
  xt[2][3] = cm[2] * rv[2];
  xt[2][4] = cm[2] * rv[3] + dm[1];
  xt[2][5] = -ho * cm[2];
  xt[3][1] = bo * cm[3] + dm[1] * ve[2] - dm[2] * ve[1];
  xt[3][2] = cm[3] * rv[1] + dm[2];
  xt[3][3] = cm[3] * rv[2] - dm[1];
  xt[3][4] = cm[3] * rv[3];
  xt[3][5] = -ho * cm[3];
  xt[4][1] = one - bo - co;
  xt[4][2] = dm[1] - rv[1];
  xt[4][3] = dm[2] - rv[2];
  xt[4][4] = dm[3] - rv[3];
  xt[4][5] = ho;
  xt[5][1] = one - bo + co;
  xt[5][2] = -dm[1] - rv[1];
  xt[5][3] = -dm[2] - rv[2];
  xt[5][4] = -dm[3] - rv[3];
  xt[5][5] = ho;
}

static void xtr2q(const Elem *e, const double cm[4], double xt[6][6]) {
  double bo = e->hv2 + hamm1 * e->ao * e->ao, co = e->ao * e->vn, dm[4];
  for (int q = 1; q <= 3; q++) dm[q] = e->ao * cm[q];
  const double *ve = e->ve;
  xt[1][1] = cm[1]; xt[1][2] = cm[2]; xt[1][3] = cm[3]; xt[1][4] = half; xt[1][5] = half;
  xt[2][1] = cm[1] * ve[1];
  xt[2][2] = cm[2] * ve[1] - dm[3];
  xt[2][3] = cm[3] * ve[1] + dm[2];
  xt[2][4] = half * (ve[1] + dm[1]);
  xt[2][5] = xt[2][4] - dm[1];
  xt[3][1] = cm[1] * ve[2] + dm[3];
  xt[3][2] = cm[2] * ve[2];
  xt[3][3] = cm[3] * ve[2] - dm[1];
  xt[3][4] = half * (ve[2] + dm[2]);
  xt[3][5] = xt[3][4] - dm[2];
  xt[4][1] = cm[1] * ve[3] - dm[2];
  xt[4][2] = cm[2] * ve[3] + dm[1];
  xt[4][3] = cm[3] * ve[3];
  xt[4][4] = half * (ve[3] + dm[3]);
  xt[4][5] = xt[4][4] - dm[3];
  xt[5][1] = e->hv2 * cm[1] + dm[3] * ve[2] - dm[2] * ve[3];
  xt[5][2] = e->hv2 * cm[2] + dm[1] * ve[3] - dm[3] * ve[1];
  xt[5][3] = e->hv2 * cm[3] + dm[2] * ve[1] - dm[1] * ve[2];
  xt[5][4] = half * (bo + co);
  xt[5][5] = xt[5][4] - co;
}

static void matvec5(double xt[6][6], const double v[6], double out[6]) {
  for (int r = 1; r <= 5; r++) {
    double s = 0;
    for (int q = 1; q <= 5; q++) s += xt[r][q] * v[q];
    out[r] = s;
  }
}

/* ---- moving frame: src/Subroutineso.f90:192-259 -------------------------- */
static void pitch(orc_case *c, double alpha0, double alpha1, double dtko, double dtk) {
  double daoa = (alpha1 - alpha0) * pi / 180, raoa0 = alpha0 * pi / 180;
  double tps = c->cfg.tps, tp = c->cfg.tp, amachoo = c->amachoo;
  if (c->timo + dtk > tps) {
    double ra3 = c->timo - tps, dtsdt = pi / tp;
    double ts = fmin(dtsdt * ra3, pi), tsdt = fmin(dtsdt * (ra3 + dtko), pi);
    double aoat = raoa0 + half * daoa * (1 - cos(ts));
    double aoatdt = raoa0 + half * daoa * (1 - cos(tsdt));
    double fctr = half * daoa * dtsdt;
    double ut[4] = {0, amachoo * cos(aoat), amachoo * sin(aoat), zero};
    double dudt[4] = {0, -(amachoo * fctr * sin(aoatdt) * sin(tsdt)), amachoo * fctr * cos(aoatdt) * sin(tsdt), zero};
    for (int q = 1; q <= 3; q++) c->umf[q] = ut[q] + dtk * dudt[q];
    double dudt1[4] = {0, -(amachoo * fctr * sin(aoat) * sin(ts)), amachoo * fctr * cos(aoat) * sin(ts), zero};
    double st = sin(tsdt);
    double dudt2[4] = {0, -(amachoo * fctr * (cos(aoatdt) * fctr * (st * st) + dtsdt * sin(aoatdt) * cos(tsdt))),
                       -(amachoo * fctr * (sin(aoatdt) * fctr * (st * st) - dtsdt * cos(aoatdt) * cos(tsdt))), zero};
    for (int q = 1; q <= 3; q++) c->dudtmf[q] = dudt1[q] + dtk * dudt2[q];
    c->aoa = atan(c->umf[2] / c->umf[1]) * 180 / pi;
  }
}

static void movef(orc_case *c, double dtko, double dtk) {
  if (c->cfg.nsmf == 0) {
    double timf = c->cfg.timf;
    double ra0 = pi / timf, ra1 = ra0 * fmin(c->timo, timf), ra2 = ra0 * fmin(c->timo + dtko, timf);
    double fctr = one - cos(ra1), dfdt = ra0 * sin(ra2);
    double progmf = half * (fctr + dtk * dfdt);
    for (int q = 1; q <= 3; q++) c->umf[q] = progmf * c->uoo[q];
    fctr = sin(ra1); dfdt = ra0 * cos(ra2);
    progmf = half * ra0 * (fctr + dtk * dfdt);
    for (int q = 1; q <= 3; q++) c->dudtmf[q] = progmf * c->uoo[q];
    if (c->cfg.tp > 0) pitch(c, c->cfg.aoa0, c->cfg.aoa1, dtko, dtk);
  } else {
    for (int q = 1; q <= 3; q++) { c->umf[q] = c->uoo[q]; c->dudtmf[q] = zero; }
  }
}

/* ---- set-up after the grid: src/Main3D.f90:365-480, spongeup ------------- */
int orc_set_grid(orc_case *c, int blk, const double *xyz) {
  if (blk < 0 || blk >= c->nb || !xyz) return ATI_EINVAL;
  OBlock *b = &c->b[blk];
  memcpy(b->xyz, xyz, sizeof(double) * 3 * b->np);
  memcpy(b->ss, xyz, sizeof(double) * 3 * b->np);
  b->grid_set = 1;
  return ATI_OK;
}

static void metrics(orc_case *c) {
  /* coordinate derivatives (src/Main3D.f90:365-375) */
  double *dst[3];
  for (int m = 1; m <= 3; m++) {
    for (int mb = 0; mb < c->nb; mb++) {
      OBlock *b = &c->b[mb];
      memcpy(b->rr, b->xyz + (size_t)(m - 1) * b->np, sizeof(double) * b->np);
    }
    orc_mpigo(c, NTDRV, NRONE, N45GO);
    orc_deriv(c, 3, 1, m); orc_deriv(c, 2, 1, m); orc_deriv(c, 1, 1, m);
    for (int mb = 0; mb < c->nb; mb++) {
      OBlock *b = &c->b[mb];
      dst[0] = b->qo; dst[1] = b->qa; dst[2] = b->de;
      memcpy(dst[m - 1], b->rr, sizeof(double) * 3 * b->np);
    }
  }
  /* non-conservative metrics and Jacobian (src/Main3D.f90:378-413) */
  for (int mb = 0; mb < c->nb; mb++) {
    OBlock *b = &c->b[mb];
    long np = b->np;
#pragma omp parallel for OMP_NT
    for (long l = 0; l < np; l++) {
      double qo1 = F(b->qo, np, l, 1), qo2 = F(b->qo, np, l, 2), qo3 = F(b->qo, np, l, 3);
      double qa1 = F(b->qa, np, l, 1), qa2 = F(b->qa, np, l, 2), qa3 = F(b->qa, np, l, 3);
      double de1 = F(b->de, np, l, 1), de2 = F(b->de, np, l, 2), de3 = F(b->de, np, l, 3);
      double x1 = qa2 * de3 - de2 * qa3, x2 = de2 * qo3 - qo2 * de3, x3 = qo2 * qa3 - qa2 * qo3;
      double e1 = qa3 * de1 - de3 * qa1, e2 = de3 * qo1 - qo3 * de1, e3 = qo3 * qa1 - qa3 * qo1;
      double z1 = qa1 * de2 - de1 * qa2, z2 = de1 * qo2 - qo1 * de2, z3 = qo1 * qa2 - qa1 * qo2;
      F(b->xim, np, l, 1) = x1; F(b->xim, np, l, 2) = x2; F(b->xim, np, l, 3) = x3;
      F(b->etm, np, l, 1) = e1; F(b->etm, np, l, 2) = e2; F(b->etm, np, l, 3) = e3;
      F(b->zem, np, l, 1) = z1; F(b->zem, np, l, 2) = z2; F(b->zem, np, l, 3) = z3;
      b->yaco[l] = three / (qo1 * x1 + qo2 * e1 + qo3 * z1 + qa1 * x2 + qa2 * e2 + qa3 * z2 + de1 * x3 + de2 * e3 + de3 * z3);
    }
  }
}

static void wall_setup(orc_case *c) {
  /* wallArea / walldir, src/rpt.f90:774-864 (npc = 1) */
  int bcw = 20 + 5 * c->cfg.nviscous;
  for (int mb = 0; mb < c->nb; mb++) {
    OBlock *b = &c->b[mb];
    int bct = b->nbc[1][2], bcb = b->nbc[0][2], j = 0;
    double coef = one;
    b->wflag = 0;
    if (bcb == bcw) { j = 0; b->wflag = 1; coef = one; }
    else if (bct == bcw) { j = b->ijk[1][2]; b->wflag = 1; coef = -one; }
    if (!b->wflag) continue;
    b->nwall = b->nbsize[2];
    b->lwall = (long *)malloc(sizeof(long) * b->nwall);
    b->area = dalloc(b->nwall);
    b->wnor = dalloc(3 * b->nwall);
    long ll = -1, np = b->np;
    for (int k = 0; k <= b->ijk[2][2]; k++)
      for (int i = 0; i <= b->ijk[3][2]; i++) {
        long l = indx3(b, j, k, i, 2);
        double g11 = F(b->qo, np, l, 1) * F(b->qo, np, l, 1) + F(b->qa, np, l, 1) * F(b->qa, np, l, 1) +
                     F(b->de, np, l, 1) * F(b->de, np, l, 1);
        double g33 = F(b->qo, np, l, 3) * F(b->qo, np, l, 3) + F(b->qa, np, l, 3) * F(b->qa, np, l, 3) +
                     F(b->de, np, l, 3) * F(b->de, np, l, 3);
        double g13 = F(b->qo, np, l, 1) * F(b->qo, np, l, 3) + F(b->qa, np, l, 1) * F(b->qa, np, l, 3) +
                     F(b->de, np, l, 1) * F(b->de, np, l, 3);
        ll++;
        b->lwall[ll] = l;
        double ar = sqrt(g11 * g33 - g13 * g13);
        if (i == 0) ar = ar * half;
        else if (i == b->ijk[3][2]) ar = ar * half;
        if (k == 0) ar = ar * half;
        else if (k == b->ijk[2][2]) ar = ar * half;
        b->area[ll] = ar;
      }
    for (ll = 0; ll < b->nwall; ll++) {
      long l = b->lwall[ll];
      double e1 = F(b->etm, np, l, 1), e2 = F(b->etm, np, l, 2), e3 = F(b->etm, np, l, 3);
      double tmp = coef / sqrt(e1 * e1 + e2 * e2 + e3 * e3);
      b->wnor[ll + b->nwall * 0] = e1 * tmp;
      b->wnor[ll + b->nwall * 1] = e2 * tmp;
      b->wnor[ll + b->nwall * 2] = e3 * tmp;
    }
  }
}

static void face_normals(orc_case *c) {
  /* src/Main3D.f90:429-439 */
  for (int mb = 0; mb < c->nb; mb++) {
    OBlock *b = &c->b[mb];
    long np = b->np;
    for (int nn = 1; nn <= 3; nn++) {
      const double *mt = nn == 1 ? b->xim : (nn == 2 ? b->etm : b->zem);
      long nbs = b->nbsize[nn];
      for (int ip = 0; ip <= 1; ip++) {
        int i = ip * b->ijk[1][nn];
        for (int k = 0; k <= b->ijk[3][nn]; k++)
          for (int j = 0; j <= b->ijk[2][nn]; j++) {
            long jk = (long)k * (b->ijk[2][nn] + 1) + j, l = indx3(b, i, j, k, nn);
            double rv[4];
            for (int q = 1; q <= 3; q++) rv[q] = b->yaco[l] * F(mt, np, l, q);
            double fctr = one / sqrt(rv[1] * rv[1] + rv[2] * rv[2] + rv[3] * rv[3]);
            for (int q = 1; q <= 3; q++) b->cm[nn][jk + nbs * ((q - 1) + 3 * ip)] = fctr * rv[q];
          }
      }
    }
  }
}

static int is_gcbc(int np) { return (np - 10) * (np - 20) * (np - 25) * (np - 30) == 0; }
static int is_wall(int np) { return (np - 20) * (np - 25) == 0; }
static int is_avg(int np) { return (np - 30) * (np - 35) * (np - 45) == 0; }

static void gcbc_setup(orc_case *c) {
  /* src/Main3D.f90:460-480 (nextrabc = 0: no wall slots, rpex = 0) */
  for (int mb = 0; mb < c->nb; mb++) {
    OBlock *b = &c->b[mb];
    long np = b->np, nsb = 0, nwp = 0;
    for (int nn = 1; nn <= 3; nn++)
      for (int ip = 0; ip <= 1; ip++)
        if (is_gcbc(b->nbc[ip][nn])) {
          nsb += b->nbsize[nn] * (MBCI + 1);
          if (is_wall(b->nbc[ip][nn])) nwp += b->nbsize[nn];
        }
    double *cnt = dalloc(np), *w = dalloc(nsb);
    long *idx = (long *)malloc(sizeof(long) * (nsb ? nsb : 1));
    long ll = -1;
    for (int nn = 1; nn <= 3; nn++)
      for (int ip = 0; ip <= 1; ip++) {
        int npc = b->nbc[ip][nn], i = ip * b->ijk[1][nn], iq = 1 - 2 * ip;
        if (!is_gcbc(npc)) continue;
        for (int k = 0; k <= b->ijk[3][nn]; k++)
          for (int j = 0; j <= b->ijk[2][nn]; j++) {
            long l = indx3(b, i, j, k, nn);
            ll++;
            double res = one / b->yaco[l];
            cnt[l] = cnt[l] + one; w[ll] = res; idx[ll] = l;
            for (int ii = 1; ii <= MBCI; ii++) {
              l = indx3(b, i + iq * ii, j, k, nn);
              ll++;
              cnt[l] = cnt[l] + one; w[ll] = res * c->sbci[ii]; idx[ll] = l;
            }
          }
      }
    b->nsbcc = nsb;
    b->sbcc = dalloc(nsb);
    for (ll = 0; ll < nsb; ll++) b->sbcc[ll] = w[ll] / cnt[idx[ll]];
    b->nrpex = nwp;
    b->rpex = dalloc(nwp);
    free(cnt); free(w); free(idx);
  }
}

static void sponge_setup(orc_case *c) {
  /* spongeup, src/SingleTurbulence3D.f90:209-249; dense coefficients, zero
   * outside the sponge.  The literal 0.7e0 is default (single) precision. */
  const ati_config_t *g = &c->cfg;
  const double p7 = (double)0.7f, domlen = g->domlen;
  for (int mb = 0; mb < c->nb; mb++) {
    OBlock *b = &c->b[mb];
    double szr[2][4], szp[2][4];
    int nsz[2][4];
    for (int nn = 1; nn <= 3; nn++) {
      nsz[0][nn] = b->nbcs[nn] == 10 ? 1 : 0;
      nsz[1][nn] = b->nbce[nn] == 10 ? 1 : 0;
    }
    szr[0][1] = 1 / g->szth1; szp[0][1] = -p7 * domlen + g->szth1;
    szr[1][1] = 1 / (g->szth1 + g->szxt); szp[1][1] = domlen - g->szth1;
    szr[0][2] = 1 / g->szth2; szp[0][2] = -p7 * domlen + g->szth2;
    szr[1][2] = 1 / g->szth2; szp[1][2] = domlen + g->szxt - g->szth2;
    szr[0][3] = 0; szp[0][3] = 0; szr[1][3] = 0; szp[1][3] = 0;
    double ra1 = 0.25, ra2 = pi / (two * domlen);
    long np = b->np;
#pragma omp parallel for OMP_NT
    for (long l = 0; l < np; l++) {
      double r[4];
      for (int q = 1; q <= 3; q++) {
        double x = F(b->xyz, np, l, q);
        r[q] = nsz[0][q] * szr[0][q] * fmax(szp[0][q] - x, zero) + nsz[1][q] * szr[1][q] * fmax(x - szp[1][q], zero);
      }
      double sig = g->szco * (one - 0.125 * (one + cos(pi * r[1])) * (one + cos(pi * r[2])) * (one + cos(pi * r[3])));
      double lam = ra1 + half * (one - ra1) * (one + cos(ra2 * (fmin(F(b->xyz, np, l, 1), domlen) + domlen)));
      if (sig > zero) {
        double res = one / b->yaco[l];
        b->asz[l] = res * sig * lam;
        b->bsz[l] = res * hamm1 * sig;
      } else {
        b->asz[l] = 0; b->bsz[l] = 0;
      }
    }
  }
}

int orc_init(orc_case *c) {
  for (int mb = 0; mb < c->nb; mb++)
    if (!c->b[mb].grid_set) return ATI_ESTATE;
  metrics(c);
  wall_setup(c);
  face_normals(c);
  gcbc_setup(c);
  sponge_setup(c);
  /* initialo (src/SingleTurbulence3D.f90:203) and src/Main3D.f90:521 */
  for (int mb = 0; mb < c->nb; mb++) {
    OBlock *b = &c->b[mb];
    long np = b->np;
    for (long l = 0; l < np; l++) {
      F(b->qa, np, l, 1) = c->rhooo;
      F(b->qa, np, l, 2) = zero; F(b->qa, np, l, 3) = zero; F(b->qa, np, l, 4) = zero;
      F(b->qa, np, l, 5) = hamm1 * c->poo;
    }
  }
  c->n = 0; c->ndt = 0; c->dt = zero; c->dts = zero; c->dte = zero; c->timo = zero;
  c->steps_done = 0;
  movef(c, 0, 0);
  c->inited = 1;
  return ATI_OK;
}

/* ---- inflow turbulence (new code: the reference's inflow-eddy generator is
 * disabled, src/SingleTurbulence3D.f90:260) ---------------------------------
 * The gust points are the sponge points of the inflow zone, x < -0.7 domlen +
 * szth1, with the streamwise ramp atz = sin^2(min(pi (x + domlen)/szth1,
 * pi/2)); spongego (src/SingleTurbulence3D.f90:355-372) drives them towards the
 * isentropic target of a velocity v.  Here v is the FP64 sum of the given
 * Fourier modes, v = sum_m 2 a_m s_m cos(k_m . x + psi_m - (k_m . U_inf) t),
 * evaluated at the start time of the first step and of every step that takes
 * a new dt (n % 10 == 1), held in between. */
int orc_set_turbulence(orc_case *c, const float *modes, int nmodes) {
  if (!c->inited || nmodes < 0 || (nmodes > 0 && !modes)) return ATI_EINVAL;
  free(c->modes); free(c->gblk); free(c->gl); free(c->gx); free(c->gatz); free(c->gv); free(c->gidx); free(c->goff);
  c->modes = NULL; c->gblk = NULL; c->gl = NULL; c->gx = NULL; c->gatz = NULL; c->gv = NULL; c->gidx = NULL;
  c->goff = NULL; c->ngust = 0; c->nmodes = 0;
  if (nmodes == 0) return ATI_OK;
  const ati_config_t *g = &c->cfg;
  c->nmodes = nmodes;
  c->modes = dalloc(8 * (long)nmodes);
  for (long q = 0; q < 8 * (long)nmodes; q++) c->modes[q] = (double)modes[q];
  const double xg = -(double)0.7f * g->domlen + g->szth1, ra0 = pi / g->szth1;
  long ntot = 0, ng = 0;
  for (int mb = 0; mb < c->nb; mb++) ntot += c->b[mb].np;
  c->goff = (long *)malloc(sizeof(long) * (c->nb + 1));
  c->gidx = (long *)malloc(sizeof(long) * (ntot > 0 ? ntot : 1));
  long off = 0;
  for (int mb = 0; mb < c->nb; mb++) {
    OBlock *b = &c->b[mb];
    c->goff[mb] = off;
    for (long l = 0; l < b->np; l++) {
      const double x = F(b->xyz, b->np, l, 1);
      c->gidx[off + l] = (b->asz[l] == 0.0 || !(x < xg)) ? -1 : ng++;
    }
    off += b->np;
  }
  c->goff[c->nb] = off;
  c->ngust = ng;
  c->gblk = (int *)malloc(sizeof(int) * (ng > 0 ? ng : 1));
  c->gl = (long *)malloc(sizeof(long) * (ng > 0 ? ng : 1));
  c->gx = dalloc(3 * (ng > 0 ? ng : 1)); c->gatz = dalloc(ng > 0 ? ng : 1); c->gv = dalloc(3 * (ng > 0 ? ng : 1));
  for (int mb = 0; mb < c->nb; mb++) {
    OBlock *b = &c->b[mb];
    for (long l = 0; l < b->np; l++) {
      const long q = c->gidx[c->goff[mb] + l];
      if (q < 0) continue;
      const double x = F(b->xyz, b->np, l, 1);
      c->gblk[q] = mb; c->gl[q] = l;
      c->gx[3 * q] = x; c->gx[3 * q + 1] = F(b->xyz, b->np, l, 2); c->gx[3 * q + 2] = F(b->xyz, b->np, l, 3);
      const double sa = sin(fmin(ra0 * (x + g->domlen), half * pi));
      c->gatz[q] = sa * sa;
      c->gv[3 * q] = c->gv[3 * q + 1] = c->gv[3 * q + 2] = zero;
    }
  }
  return ATI_OK;
}

/* The mode table of the inflow turbulence, restating the generator of the GPU library: nmodes = turb_modes
 * wavenumbers log-spaced over [0.1 ke, 20 ke] (ke = 0.747 / turb_length) with amplitudes from the von Karman
 * spectrum E(k) ~ (k/ke)^4 / (1 + (k/ke)^2)^(17/6); directions, polarisation angle and phase uniform from
 * splitmix64 (Steele, Lea and Flood 2014) seeded by turb_seed; k_z rounded to the span's periodic lattice;
 * polarisation normal to k; amplitudes scaled so that sum 2 a^2 = 3 (turb_intensity |U_inf|)^2.  out holds 8
 * floats per mode (k_x, k_y, k_z, s_x, s_y, s_z, a, psi); returns the mode count (0: no turbulence). */
typedef struct { uint64_t s; } orc_splitmix;
static uint64_t smx_next(orc_splitmix *r) {
  uint64_t z = (r->s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static double smx_uniform(orc_splitmix *r) { return (double)(smx_next(r) >> 11) * (1.0 / 9007199254740992.0); }

int orc_build_modes(const ati_config_t *cfg, float *out) {
  const int n = cfg->turb_modes;
  if (n <= 0 || cfg->turb_intensity <= 0.0) return 0;
  if (!out) return n;
  const double pie = acos(-1.0);
  const double uinf = sqrt(cfg->amach1 * cfg->amach1 + cfg->amach2 * cfg->amach2 + cfg->amach3 * cfg->amach3);
  const double urms = cfg->turb_intensity * uinf;
  const double L = cfg->turb_length > 0 ? cfg->turb_length : 0.1;
  const double ke = 0.747 / L, kmin = 0.1 * ke, kmax = 20.0 * ke, lr = log(kmax / kmin);
  const double kz0 = 2.0 * pie / cfg->span;
  orc_splitmix rng = {(uint64_t)(uint32_t)cfg->turb_seed * 0x2545F4914F6CDD1Dull + 1};
  double *mk = dalloc(3 * (long)n), *ms = dalloc(3 * (long)n), *ma = dalloc(n), *mp = dalloc(n);
  double e2 = 0.0;
  for (int m = 0; m < n; m++) {
    const double k = kmin * exp(lr * (m + 0.5) / n), dk = k * lr / n, r = k / ke;
    const double E = r * r * r * r / pow(1.0 + r * r, 17.0 / 6.0);
    const double ct = 1.0 - 2.0 * smx_uniform(&rng), st = sqrt(fmax(0.0, 1.0 - ct * ct));
    const double ph = 2.0 * pie * smx_uniform(&rng), al = 2.0 * pie * smx_uniform(&rng), psi = 2.0 * pie * smx_uniform(&rng);
    double kv[3] = {k * st * cos(ph), k * st * sin(ph), k * ct};
    kv[2] = kz0 * nearbyint(kv[2] / kz0);
    const double kk = sqrt(kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2]);
    const double kh[3] = {kv[0] / kk, kv[1] / kk, kv[2] / kk};
    double e1[3];
    if (fabs(kh[2]) < 0.9) { e1[0] = -kh[1]; e1[1] = kh[0]; e1[2] = 0.0; }
    else { e1[0] = 0.0; e1[1] = -kh[2]; e1[2] = kh[1]; }
    const double n1 = sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
    for (int q = 0; q < 3; q++) e1[q] /= n1;
    const double e2v[3] = {kh[1] * e1[2] - kh[2] * e1[1], kh[2] * e1[0] - kh[0] * e1[2], kh[0] * e1[1] - kh[1] * e1[0]};
    for (int q = 0; q < 3; q++) {
      mk[3 * m + q] = kv[q];
      ms[3 * m + q] = cos(al) * e1[q] + sin(al) * e2v[q];
    }
    ma[m] = sqrt(E * dk);
    mp[m] = psi;
    e2 += 2.0 * ma[m] * ma[m];
  }
  const double scale = sqrt(3.0 * urms * urms / e2);
  for (int m = 0; m < n; m++) {
    for (int q = 0; q < 3; q++) {
      out[8 * m + q] = (float)mk[3 * m + q];
      out[8 * m + 3 + q] = (float)ms[3 * m + q];
    }
    out[8 * m + 6] = (float)(ma[m] * scale);
    out[8 * m + 7] = (float)mp[m];
  }
  free(mk); free(ms); free(ma); free(mp);
  return n;
}

static void gust_eval(orc_case *c, double t) {
  const long ng = c->ngust;
  const int nm = c->nmodes;
  const double u1 = c->uoo[1], u2 = c->uoo[2], u3 = c->uoo[3];
#pragma omp parallel for OMP_NT
  for (long q = 0; q < ng; q++) {
    const double x = c->gx[3 * q], y = c->gx[3 * q + 1], z = c->gx[3 * q + 2];
    double vx = zero, vy = zero, vz = zero;
    for (int m = 0; m < nm; m++) {
      const double *md = c->modes + 8 * (long)m;
      const double w = (md[0] * u1 + md[1] * u2 + md[2] * u3) * t;
      const double ph = md[0] * x + md[1] * y + md[2] * z + md[7] - w;
      const double cc = two * md[6] * cos(ph);
      vx = vx + cc * md[3];
      vy = vy + cc * md[4];
      vz = vz + cc * md[5];
    }
    c->gv[3 * q] = vx; c->gv[3 * q + 1] = vy; c->gv[3 * q + 2] = vz;
  }
}

/* ---- the per-step filter: src/Main3D.f90:555-561 -------------------------- */
int orc_filter_step(orc_case *c) {
  for (int m = 1; m <= 5; m++) {
    for (int mb = 0; mb < c->nb; mb++) {
      OBlock *b = &c->b[mb];
      memcpy(b->rr, b->qa + (size_t)(m - 1) * b->np, sizeof(double) * b->np);
    }
    orc_mpigo(c, NTFLT, NRONE, N45NO);
    orc_filte(c, 1, 1); orc_filte(c, 2, 1); orc_filte(c, 3, 1);
    for (int mb = 0; mb < c->nb; mb++) {
      OBlock *b = &c->b[mb];
      memcpy(b->qa + (size_t)(m - 1) * b->np, b->rr, sizeof(double) * b->np);
    }
  }
  for (int mb = 0; mb < c->nb; mb++) {
    OBlock *b = &c->b[mb];
    memcpy(b->qo, b->qa, sizeof(double) * 5 * b->np);
  }
  return ATI_OK;
}

/* ---- one RK stage: src/Main3D.f90:567-958 ---------------------------------- */
#define TXX 1
#define TYY 2
#define TZZ 3
#define TXY 4
#define TYZ 5
#define TZX 6
#define HXX 7
#define HYY 8
#define HZZ 9

static void grad_combo(OBlock *b, int o1, int o2, int o3, int to_ss) {
  /* three physical-gradient combinations of rr(:,1:3) (src/Main3D.f90:631-651) */
  long np = b->np;
#pragma omp parallel for OMP_NT
  for (long l = 0; l < np; l++) {
    double r1 = F(b->rr, np, l, 1), r2 = F(b->rr, np, l, 2), r3 = F(b->rr, np, l, 3);
    double v1 = F(b->xim, np, l, 1) * r1 + F(b->etm, np, l, 1) * r2 + F(b->zem, np, l, 1) * r3;
    double v2 = F(b->xim, np, l, 2) * r1 + F(b->etm, np, l, 2) * r2 + F(b->zem, np, l, 2) * r3;
    double v3 = F(b->xim, np, l, 3) * r1 + F(b->etm, np, l, 3) * r2 + F(b->zem, np, l, 3) * r3;
    if (to_ss) {
      F(b->ss, np, l, 1) = v1; F(b->ss, np, l, 2) = v2; F(b->ss, np, l, 3) = v3;
    } else {
      F(b->tau, np, l, o1) = v1; F(b->tau, np, l, o2) = v2; F(b->tau, np, l, o3) = v3;
    }
  }
}

static int imin(int a, int b) { return a < b ? a : b; }
static int imax(int a, int b) { return a > b ? a : b; }

static void set_rr1(orc_case *c, const double *(*src)(const OBlock *)) {
  for (int mb = 0; mb < c->nb; mb++) {
    OBlock *b = &c->b[mb];
    memcpy(b->rr, src(b), sizeof(double) * b->np);
  }
}
static const double *src_de2(const OBlock *b) { return b->de + (size_t)1 * b->np; }
static const double *src_de3(const OBlock *b) { return b->de + (size_t)2 * b->np; }
static const double *src_de4(const OBlock *b) { return b->de + (size_t)3 * b->np; }
static const double *src_de5(const OBlock *b) { return b->de + (size_t)4 * b->np; }

static void divergence(orc_case *c, int m) {
  /* de(:,m) = rr(:,1)+rr(:,2)+rr(:,3) (src/Main3D.f90:722 etc.) */
  for (int mb = 0; mb < c->nb; mb++) {
    OBlock *b = &c->b[mb];
    long np = b->np;
#pragma omp parallel for OMP_NT
    for (long l = 0; l < np; l++) F(b->de, np, l, m) = F(b->rr, np, l, 1) + F(b->rr, np, l, 2) + F(b->rr, np, l, 3);
  }
}

int orc_rk_stage(orc_case *c, int nk) {
  if (!c->inited) return ATI_ESTATE;
  const ati_config_t *g = &c->cfg;
  const int nkrk = g->nkrk;
  if (nk < 1 || nk > nkrk) return ATI_EINVAL;

  /* moving frame before time advancing (src/Main3D.f90:571-572) */
  double dtko = c->dt * imin(imax(nk - 2, 0), 1) / (nkrk - nk + 3);
  double dtk = c->dt * imin(nk - 1, 1) / (nkrk - nk + 2);
  movef(c, dtko, dtk);

  /* primitives, pressure, temperature, Sutherland (src/Main3D.f90:576-583) */
  for (int mb = 0; mb < c->nb; mb++) {
    OBlock *b = &c->b[mb];
    long np = b->np;
#pragma omp parallel for OMP_NT
    for (long l = 0; l < np; l++) {
      double q1 = F(b->qa, np, l, 1), q2 = F(b->qa, np, l, 2), q3 = F(b->qa, np, l, 3), q4 = F(b->qa, np, l, 4),
             q5 = F(b->qa, np, l, 5);
      double d1 = one / q1, d2 = q2 * d1, d3 = q3 * d1, d4 = q4 * d1;
      double pp = gamm1 * (q5 - half * (q2 * d2 + q3 * d3 + q4 * d4));
      double d5 = gam * pp * d1;
      F(b->de, np, l, 1) = d1; F(b->de, np, l, 2) = d2; F(b->de, np, l, 3) = d3; F(b->de, np, l, 4) = d4;
      F(b->de, np, l, 5) = d5;
      b->p[l] = pp;
      F(b->ss, np, l, 1) = c->srefp1dre * pow(d5, 1.5) / (d5 + c->srefoo);
    }
  }

  /* time step (src/Main3D.f90:587-610) */
  if (nk == 1) {
    if (c->n % 10 == 1) {
      c->ndt = c->n; c->dts = c->dte;
      if (g->dto < zero) {
        double m1 = 0, m2 = 0;
        for (int mb = 0; mb < c->nb; mb++) {
          OBlock *b = &c->b[mb];
          long np = b->np;
          double u1 = c->umf[1], u2 = c->umf[2], u3 = c->umf[3];
#pragma omp parallel for reduction(max : m1, m2) OMP_NT
          for (long l = 0; l < np; l++) {
            double x1 = F(b->xim, np, l, 1), x2 = F(b->xim, np, l, 2), x3 = F(b->xim, np, l, 3);
            double e1 = F(b->etm, np, l, 1), e2 = F(b->etm, np, l, 2), e3 = F(b->etm, np, l, 3);
            double z1 = F(b->zem, np, l, 1), z2 = F(b->zem, np, l, 2), z3 = F(b->zem, np, l, 3);
            double d2 = F(b->de, np, l, 2) + u1, d3 = F(b->de, np, l, 3) + u2, d4 = F(b->de, np, l, 4) + u3;
            double r1 = x1 * x1 + x2 * x2 + x3 * x3 + e1 * e1 + e2 * e2 + e3 * e3 + z1 * z1 + z2 * z2 + z3 * z3;
            double r2 = fabs(x1 * d2 + x2 * d3 + x3 * d4) + fabs(e1 * d2 + e2 * d3 + e3 * d4) + fabs(z1 * d2 + z2 * d3 + z3 * d4);
            double s2 = fabs(b->yaco[l]);
            F(b->rr, np, l, 1) = r1; F(b->rr, np, l, 2) = r2; F(b->ss, np, l, 2) = s2;
            double v1 = (sqrt(F(b->de, np, l, 5) * r1) + r2) * s2;
            double v2 = F(b->de, np, l, 1) * F(b->ss, np, l, 1) * r1 * s2 * s2;
            if (v1 > m1) m1 = v1;
            if (v2 > m2) m2 = v2;
          }
        }
        double ra0 = g->cfl / m1, ra1 = ra0;
        if (g->nviscous == 1) ra1 = half / m2;
        c->dte = fmin(ra0, ra1);
      } else {
        c->dte = g->dto;
      }
    }
    double s = sin(0.05 * pi * (double)(c->n - c->ndt));
    c->dt = c->dts + (c->dte - c->dts) * (s * s);
  }

  /* viscous shear stresses and heat fluxes (src/Main3D.f90:626-693) */
  if (g->nviscous == 1) {
    for (int mb = 0; mb < c->nb; mb++) {
      OBlock *b = &c->b[mb];
      memcpy(b->de, b->ss, sizeof(double) * b->np); /* de(:,1) = ss(:,1) */
    }
    set_rr1(c, src_de2);
    orc_mpigo(c, NTDRV, NRONE, N45NO); orc_deriv(c, 3, 1, 2); orc_deriv(c, 2, 1, 2); orc_deriv(c, 1, 1, 2);
    for (int mb = 0; mb < c->nb; mb++) grad_combo(&c->b[mb], TXX, HZZ, TZX, 0);
    set_rr1(c, src_de3);
    orc_mpigo(c, NTDRV, NRONE, N45NO); orc_deriv(c, 3, 1, 3); orc_deriv(c, 2, 1, 3); orc_deriv(c, 1, 1, 3);
    for (int mb = 0; mb < c->nb; mb++) grad_combo(&c->b[mb], TXY, TYY, HXX, 0);
    set_rr1(c, src_de4);
    orc_mpigo(c, NTDRV, NRONE, N45NO); orc_deriv(c, 3, 1, 4); orc_deriv(c, 2, 1, 4); orc_deriv(c, 1, 1, 4);
    for (int mb = 0; mb < c->nb; mb++) grad_combo(&c->b[mb], HYY, TYZ, TZZ, 0);
    set_rr1(c, src_de5);
    orc_mpigo(c, NTDRV, NRONE, N45NO); orc_deriv(c, 3, 1, 5); orc_deriv(c, 2, 1, 5); orc_deriv(c, 1, 1, 5);
    for (int mb = 0; mb < c->nb; mb++) grad_combo(&c->b[mb], 0, 0, 0, 1);
    for (int mb = 0; mb < c->nb; mb++) {
      OBlock *b = &c->b[mb];
      long np = b->np;
      double *t = b->tau;
#pragma omp parallel for OMP_NT
      for (long l = 0; l < np; l++) {
        double r1 = F(b->de, np, l, 1) * b->yaco[l];
        double r2 = gamm1prndtli * r1, r3 = 0, d5;
        double txx = F(t, np, l, TXX), tyy = F(t, np, l, TYY), tzz = F(t, np, l, TZZ);
        double txy = F(t, np, l, TXY), tyz = F(t, np, l, TYZ), tzx = F(t, np, l, TZX);
        double hxx = F(t, np, l, HXX), hyy = F(t, np, l, HYY), hzz = F(t, np, l, HZZ);
        if (g->les == 1) {
          double d1 = txx * txx + tyy * tyy + tzz * tzz + (hzz + txy) * (hzz + txy) + (hyy + tzx) * (hyy + tzx) +
                      (hxx + tyz) * (hxx + tyz);
          F(b->de, np, l, 1) = d1;
          double varr = pow(-1 / b->yaco[l], 1.5);
          r3 = F(b->qa, np, l, 1) * (g->smago1 * g->smago1) * varr * sqrt(2 * d1);
          r1 = r1 + r3 * b->yaco[l];
          r2 = r2 + tgamm1prndtli * r3 * b->yaco[l];
          r3 = two_three * (F(b->qa, np, l, 1) * g->smago2 * varr * d1);
          d5 = two_three * (txx + tyy + tzz);
          txx = r1 * (2 * txx - d5) - r3;
          tyy = r1 * (2 * tyy - d5) - r3;
          tzz = r1 * (2 * tzz - d5) - r3;
        } else {
          d5 = two_three * (txx + tyy + tzz);
          txx = r1 * (2 * txx - d5);
          tyy = r1 * (2 * tyy - d5);
          tzz = r1 * (2 * tzz - d5);
        }
        double ntxy = r1 * (txy + hzz), ntyz = r1 * (tyz + hxx), ntzx = r1 * (tzx + hyy);
        F(b->de, np, l, 5) = d5;
        F(b->rr, np, l, 1) = r1; F(b->rr, np, l, 2) = r2;
        if (g->les == 1) F(b->rr, np, l, 3) = r3;
        double d2 = F(b->de, np, l, 2), d3 = F(b->de, np, l, 3), d4 = F(b->de, np, l, 4);
        F(t, np, l, TXX) = txx; F(t, np, l, TYY) = tyy; F(t, np, l, TZZ) = tzz;
        F(t, np, l, TXY) = ntxy; F(t, np, l, TYZ) = ntyz; F(t, np, l, TZX) = ntzx;
        F(t, np, l, HXX) = r2 * F(b->ss, np, l, 1) + d2 * txx + d3 * ntxy + d4 * ntzx;
        F(t, np, l, HYY) = r2 * F(b->ss, np, l, 2) + d2 * ntxy + d3 * tyy + d4 * ntyz;
        F(t, np, l, HZZ) = r2 * F(b->ss, np, l, 3) + d2 * ntzx + d3 * ntyz + d4 * tzz;
      }
    }
  }

  /* flux derivatives (src/Main3D.f90:710-768) and sponge (spongego,
   * src/SingleTurbulence3D.f90:360-372, dense coefficients) */
  for (int mb = 0; mb < c->nb; mb++) {
    OBlock *b = &c->b[mb];
    long np = b->np;
    double u1 = c->umf[1], u2 = c->umf[2], u3 = c->umf[3];
#pragma omp parallel for OMP_NT
    for (long l = 0; l < np; l++) {
      double r1 = F(b->de, np, l, 2) + u1, r2 = F(b->de, np, l, 3) + u2, r3 = F(b->de, np, l, 4) + u3;
      F(b->rr, np, l, 1) = r1; F(b->rr, np, l, 2) = r2; F(b->rr, np, l, 3) = r3;
      F(b->ss, np, l, 1) = F(b->xim, np, l, 1) * r1 + F(b->xim, np, l, 2) * r2 + F(b->xim, np, l, 3) * r3;
      F(b->ss, np, l, 2) = F(b->etm, np, l, 1) * r1 + F(b->etm, np, l, 2) * r2 + F(b->etm, np, l, 3) * r3;
      F(b->ss, np, l, 3) = F(b->zem, np, l, 1) * r1 + F(b->zem, np, l, 2) * r2 + F(b->zem, np, l, 3) * r3;
    }
  }
  for (int m = 1; m <= 5; m++) {
    for (int mb = 0; mb < c->nb; mb++) {
      OBlock *b = &c->b[mb];
      long np = b->np;
      const double *t = b->tau;
      const int visc = g->nviscous == 1;
      double u1 = c->umf[1], u2 = c->umf[2], u3 = c->umf[3];
#pragma omp parallel for OMP_NT
      for (long l = 0; l < np; l++) {
        double s1 = F(b->ss, np, l, 1), s2 = F(b->ss, np, l, 2), s3 = F(b->ss, np, l, 3), pp = b->p[l];
        double x1 = F(b->xim, np, l, 1), x2 = F(b->xim, np, l, 2), x3 = F(b->xim, np, l, 3);
        double e1 = F(b->etm, np, l, 1), e2 = F(b->etm, np, l, 2), e3 = F(b->etm, np, l, 3);
        double z1 = F(b->zem, np, l, 1), z2 = F(b->zem, np, l, 2), z3 = F(b->zem, np, l, 3);
        double r1, r2, r3;
        if (m == 1) {
          double q = F(b->qa, np, l, 1);
          r1 = q * s1; r2 = q * s2; r3 = q * s3;
        } else if (m <= 4) {
          double q = F(b->qa, np, l, m);
          double xm = F(b->xim, np, l, m - 1), em = F(b->etm, np, l, m - 1), zm = F(b->zem, np, l, m - 1);
          r1 = q * s1 + xm * pp; r2 = q * s2 + em * pp; r3 = q * s3 + zm * pp;
          if (visc) {
            double ta, tb, tc;
            if (m == 2) { ta = F(t, np, l, TXX); tb = F(t, np, l, TXY); tc = F(t, np, l, TZX); }
            else if (m == 3) { ta = F(t, np, l, TXY); tb = F(t, np, l, TYY); tc = F(t, np, l, TYZ); }
            else { ta = F(t, np, l, TZX); tb = F(t, np, l, TYZ); tc = F(t, np, l, TZZ); }
            r1 = r1 - x1 * ta - x2 * tb - x3 * tc;
            r2 = r2 - e1 * ta - e2 * tb - e3 * tc;
            r3 = r3 - z1 * ta - z2 * tb - z3 * tc;
          }
        } else {
          double d5 = F(b->qa, np, l, 5) + pp;
          F(b->de, np, l, 5) = d5;
          r1 = d5 * s1 - pp * (u1 * x1 + u2 * x2 + u3 * x3);
          r2 = d5 * s2 - pp * (u1 * e1 + u2 * e2 + u3 * e3);
          r3 = d5 * s3 - pp * (u1 * z1 + u2 * z2 + u3 * z3);
          if (visc) {
            double ha = F(t, np, l, HXX), hb = F(t, np, l, HYY), hc = F(t, np, l, HZZ);
            r1 = r1 - x1 * ha - x2 * hb - x3 * hc;
            r2 = r2 - e1 * ha - e2 * hb - e3 * hc;
            r3 = r3 - z1 * ha - z2 * hb - z3 * hc;
          }
        }
        F(b->rr, np, l, 1) = r1; F(b->rr, np, l, 2) = r2; F(b->rr, np, l, 3) = r3;
      }
    }
    orc_mpigo(c, NTDRV, NRALL, N45NO);
    orc_deriv(c, 1, 1, m); orc_deriv(c, 2, 2, m); orc_deriv(c, 3, 3, m);
    divergence(c, m);
  }
  if (c->ngust > 0 && nk == 1 && (c->n % 10 == 1 || c->steps_done == 0)) gust_eval(c, c->timo);
  const double fctr = half * gamm1;
  for (int mb = 0; mb < c->nb; mb++) {
    OBlock *b = &c->b[mb];
    long np = b->np;
    const long *gi = c->ngust > 0 ? c->gidx + c->goff[mb] : NULL;
#pragma omp parallel for OMP_NT
    for (long l = 0; l < np; l++) {
      double as = b->asz[l], bs = b->bsz[l];
      if (as == 0 && bs == 0) continue; /* not a sponge point */
      const long q = gi ? gi[l] : -1;
      if (q >= 0) {  /* gust point: the isentropic target of v (src/SingleTurbulence3D.f90:362-372) */
        const double *v = c->gv + 3 * q;
        const double rr = pow(one - fctr * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]), hamm1);
        F(b->de, np, l, 1) = F(b->de, np, l, 1) + as * (F(b->qa, np, l, 1) - rr);
        for (int m = 2; m <= 4; m++)
          F(b->de, np, l, m) = F(b->de, np, l, m) + as * (F(b->qa, np, l, m) - c->gatz[q] * rr * v[m - 2]);
        F(b->de, np, l, 5) = F(b->de, np, l, 5) + bs * (b->p[l] - ham * pow(rr, gam));
        continue;
      }
      F(b->de, np, l, 1) = F(b->de, np, l, 1) + as * (F(b->qa, np, l, 1) - one);
      for (int q2 = 2; q2 <= 4; q2++) F(b->de, np, l, q2) = F(b->de, np, l, q2) + as * (F(b->qa, np, l, q2) - zero);
      F(b->de, np, l, 5) = F(b->de, np, l, 5) + bs * (b->p[l] - ham * pow(one, gam));
    }
  }

  /* GCBC/GCIC preparation (src/Main3D.f90:780-795) */
  for (int mb = 0; mb < c->nb; mb++) {
    OBlock *b = &c->b[mb];
    long np = b->np;
    for (int nn = 1; nn <= 3; nn++) {
      long nbs = b->nbsize[nn];
      double *drva = b->drva[nn], *cmv = b->cm[nn];
      for (int ip = 0; ip <= 1; ip++) {
        int npc = b->nbc[ip][nn], i = ip * b->ijk[1][nn];
        if (!is_gcbc(npc)) continue;
        double ra0 = (double)((20 - npc) * (25 - npc) * (30 - npc) / 3000), ra1 = one - ra0;
        int K = b->ijk[3][nn], J = b->ijk[2][nn];
#pragma omp parallel for collapse(2) OMP_NT
        for (int k = 0; k <= K; k++)
          for (int j = 0; j <= J; j++) {
            long jk = (long)k * (J + 1) + j, l = indx3(b, i, j, k, nn);
            double cm[4], xt[6][6], cha[6], v[6], out[6];
            Elem e;
            for (int q = 1; q <= 3; q++) cm[q] = cmv[jk + nbs * ((q - 1) + 3 * ip)];
            eleme(c, b, l, cm, &e);
            xtq2r(&e, cm, xt);
            for (int q = 1; q <= 5; q++) cha[q] = ra0 * drva[jk + nbs * ((q - 1) + 5 * ip)] + ra1 * F(b->de, np, l, q);
            for (int q = 1; q <= 5; q++) v[q] = b->yaco[l] * cha[q];
            matvec5(xt, v, out);
            for (int q = 1; q <= 5; q++) drva[jk + nbs * ((q - 1) + 5 * ip)] = out[q];
          }
      }
    }
  }
  /* GCIC exchange (src/Main3D.f90:799-813): BC 30 faces */
  for (int mb = 0; mb < c->nb; mb++) {
    OBlock *b = &c->b[mb];
    for (int nn = 1; nn <= 3; nn++)
      for (int ip = 0; ip <= 1; ip++) {
        if (b->nbc[ip][nn] != 30) continue;
        OBlock *o = &c->b[b->ncd[ip][nn]];
        long nbs = b->nbsize[nn];
        memcpy(b->drvb[nn] + nbs * 5 * ip, o->drva[nn] + nbs * 5 * (1 - ip), sizeof(double) * 5 * nbs);
      }
  }
  /* GCBC/GCIC application (src/Main3D.f90:817-869) */
  for (int mb = 0; mb < c->nb; mb++) {
    OBlock *b = &c->b[mb];
    long np = b->np, ll0 = 0, lp0 = 0;
    for (int nn = 1; nn <= 3; nn++) {
      long nbs = b->nbsize[nn];
      double *drva = b->drva[nn], *drvb = b->drvb[nn], *cmv = b->cm[nn];
      for (int ip = 0; ip <= 1; ip++) {
        int npc = b->nbc[ip][nn], i = ip * b->ijk[1][nn], iq = 1 - 2 * ip;
        double ra0 = iq;
        if (!is_gcbc(npc)) continue;
        int K = b->ijk[3][nn], J = b->ijk[2][nn];
        /* lines of one face touch distinct points, so they may run in parallel */
#pragma omp parallel for collapse(2) OMP_NT
        for (int k = 0; k <= K; k++)
          for (int j = 0; j <= J; j++) {
            long jk = (long)k * (J + 1) + j, l = indx3(b, i, j, k, nn);
            long ll = ll0 + jk * (MBCI + 1), lp = lp0 + jk;
            double cm[4], xt[6][6], cha[6], dha[6], dif[6];
            Elem e;
            for (int q = 1; q <= 3; q++) cm[q] = cmv[jk + nbs * ((q - 1) + 3 * ip)];
            eleme(c, b, l, cm, &e);
            for (int q = 1; q <= 5; q++) {
              cha[q] = drva[jk + nbs * ((q - 1) + 5 * ip)];
              dha[q] = drvb[jk + nbs * ((q - 1) + 5 * ip)];
            }
            if (npc == 10) {
              if (ra0 * (e.vn + e.vs + e.ao) > zero) cha[4] = zero;
              if (ra0 * (e.vn + e.vs - e.ao) > zero) cha[5] = zero;
            } else if (npc == 20 || npc == 25) {
              if (b->rpex[lp] == zero) {
                double s = cm[1] * c->dudtmf[1] + cm[2] * c->dudtmf[2] + cm[3] * c->dudtmf[3];
                cha[4 + ip] = cha[5 - ip] + two * ra0 * e.aoi * F(b->qa, np, l, 1) * (s + 50.0 * (e.vn + e.vs));
              }
            } else {
              if (ra0 * (e.vn + e.vs) > zero) { cha[1] = dha[1]; cha[2] = dha[2]; cha[3] = dha[3]; }
              if (ra0 * (e.vn + e.vs + e.ao) > zero) cha[4] = dha[4];
              if (ra0 * (e.vn + e.vs - e.ao) > zero) cha[5] = dha[5];
            }
            xtr2q(&e, cm, xt);
            for (int q = 1; q <= 5; q++) dif[q] = cha[q] - drva[jk + nbs * ((q - 1) + 5 * ip)];
            matvec5(xt, dif, dha);
            for (int ii = 0; ii <= MBCI; ii++) {
              long l2 = indx3(b, i + iq * ii, j, k, nn);
              double w = b->sbcc[ll + ii];
              for (int q = 1; q <= 5; q++) F(b->de, np, l2, q) = F(b->de, np, l2, q) + w * dha[q];
            }
          }
        ll0 += nbs * (MBCI + 1);
        if (is_wall(npc)) lp0 += nbs;
      }
    }
  }

  /* RK update (src/Main3D.f90:873-881) */
  dtko = c->dt * imin(nk - 1, 1) / (nkrk - nk + 2);
  dtk = c->dt / (nkrk - nk + 1);
  movef(c, dtko, dtk);
  for (int mb = 0; mb < c->nb; mb++) {
    OBlock *b = &c->b[mb];
    long np = b->np;
#pragma omp parallel for OMP_NT
    for (long l = 0; l < np; l++) {
      double r1 = dtk * b->yaco[l];
      F(b->rr, np, l, 1) = r1;
      for (int q = 1; q <= 5; q++) F(b->qa, np, l, q) = F(b->qo, np, l, q) - r1 * F(b->de, np, l, q);
    }
  }
  /* wall temperature and velocity (src/Main3D.f90:886-895) */
  for (int mb = 0; mb < c->nb; mb++) {
    OBlock *b = &c->b[mb];
    long np = b->np, lp = -1;
    double ra0 = ham * hamm1 * g->wtemp;
    for (int nn = 1; nn <= 3; nn++)
      for (int ip = 0; ip <= 1; ip++) {
        int npc = b->nbc[ip][nn], i = ip * b->ijk[1][nn];
        if (!is_wall(npc)) continue;
        double ra1 = (double)((npc - 20) / 5);
        for (int k = 0; k <= b->ijk[3][nn]; k++)
          for (int j = 0; j <= b->ijk[2][nn]; j++) {
            long l = indx3(b, i, j, k, nn);
            lp++;
            double ra2 = one - b->rpex[lp], ra3 = one - ra1 * ra2;
            double fctr = (one - ra3) * F(b->qa, np, l, 1);
            for (int q = 2; q <= 4; q++) F(b->qa, np, l, q) = ra3 * F(b->qa, np, l, q) - fctr * c->umf[q - 1];
            double q1 = F(b->qa, np, l, 1), q2 = F(b->qa, np, l, 2), q3 = F(b->qa, np, l, 3), q4 = F(b->qa, np, l, 4);
            F(b->qa, np, l, 5) = b->rpex[lp] * F(b->qa, np, l, 5) + ra2 * (ra0 * q1 + half * (q2 * q2 + q3 * q3 + q4 * q4) / q1);
          }
      }
  }
  /* junction (src/SingleTurbulence3D.f90:378-443), bkx = 3, bky = 2, npc = 1 */
  {
    int bkx = c->bkx;
    for (int nn = 0; nn <= (bkx - 1) * (c->bky - 1) - 1; nn++) {
      int njct = nn + nn / (bkx - 1);
      int mm[5], cip[5], cjp[5];
      mm[1] = njct; cip[1] = 1; cjp[1] = 1;
      mm[2] = njct + 1; cip[2] = 0; cjp[2] = 1;
      mm[3] = njct + bkx; cip[3] = 1; cjp[3] = 0;
      mm[4] = njct + bkx + 1; cip[4] = 0; cjp[4] = 0;
      int lze = c->b[mm[1]].lze;
      long kk = 5 * (lze + 1);
      double *d = dalloc(5 * kk);
      for (int q = 1; q <= 4; q++) {
        OBlock *b = &c->b[mm[q]];
        int i = cip[q] * b->lxi, j = cjp[q] * b->let;
        for (int k = 0; k <= lze; k++) {
          long l = indx3(b, i, j, k, 1);
          for (int m = 1; m <= 5; m++) d[q * kk + (m - 1) * (lze + 1) + k] = F(b->qa, b->np, l, m);
        }
      }
      double *avg = d; /* slot 0 */
      for (int jk = 0; jk <= lze; jk++)
        avg[jk] = 0.25 * (d[1 * kk + jk] + d[2 * kk + jk] + d[3 * kk + jk] + d[4 * kk + jk]);
      int pa = (1 - nn) == 1 ? 2 : 1, pb = (1 - nn) == 1 ? 4 : 3; /* drva1(:,1,1-nn), drva1(:,2,1-nn) */
      for (int m = 1; m <= 3; m++) {
        long ll = (long)m * (lze + 1);
        for (long jk = ll; jk <= ll + lze; jk++) avg[jk] = half * (d[pa * kk + jk] + d[pb * kk + jk]);
      }
      for (long jk = 4 * (lze + 1); jk <= kk - 1; jk++)
        avg[jk] = 0.25 * (d[1 * kk + jk] + d[2 * kk + jk] + d[3 * kk + jk] + d[4 * kk + jk]);
      for (int q = 1; q <= 4; q++) {
        OBlock *b = &c->b[mm[q]];
        int i = cip[q] * b->lxi, j = cjp[q] * b->let;
        for (int k = 0; k <= lze; k++) {
          long l = indx3(b, i, j, k, 1);
          for (int m = 1; m <= 5; m++) F(b->qa, b->np, l, m) = avg[(m - 1) * (lze + 1) + k];
        }
      }
      free(d);
    }
  }
  /* interface averaging (src/Main3D.f90:901-952) */
  for (int mb = 0; mb < c->nb; mb++) {
    OBlock *b = &c->b[mb];
    long np = b->np;
    for (int nn = 1; nn <= 3; nn++) {
      long nbs = b->nbsize[nn];
      for (int ip = 0; ip <= 1; ip++) {
        int npc = b->nbc[ip][nn], i = ip * b->ijk[1][nn];
        if (!is_avg(npc)) continue;
        for (int k = 0; k <= b->ijk[3][nn]; k++)
          for (int j = 0; j <= b->ijk[2][nn]; j++) {
            long jk = (long)k * (b->ijk[2][nn] + 1) + j, l = indx3(b, i, j, k, nn);
            for (int q = 1; q <= 5; q++) b->drva[nn][jk + nbs * ((q - 1) + 5 * ip)] = F(b->qa, np, l, q);
            F(b->rr, np, l, 1) = one;
          }
      }
    }
  }
  for (int mb = 0; mb < c->nb; mb++) {
    OBlock *b = &c->b[mb];
    for (int nn = 1; nn <= 3; nn++)
      for (int ip = 0; ip <= 1; ip++) {
        if (!is_avg(b->nbc[ip][nn])) continue;
        OBlock *o = &c->b[b->ncd[ip][nn]];
        long nbs = b->nbsize[nn];
        memcpy(b->drvb[nn] + nbs * 5 * ip, o->drva[nn] + nbs * 5 * (1 - ip), sizeof(double) * 5 * nbs);
      }
  }
  for (int mb = 0; mb < c->nb; mb++) {
    OBlock *b = &c->b[mb];
    long np = b->np;
    for (int nn = 1; nn <= 3; nn++) {
      long nbs = b->nbsize[nn];
      for (int ip = 0; ip <= 1; ip++) {
        int npc = b->nbc[ip][nn], i = ip * b->ijk[1][nn];
        if (!is_avg(npc)) continue;
        for (int k = 0; k <= b->ijk[3][nn]; k++)
          for (int j = 0; j <= b->ijk[2][nn]; j++) {
            long jk = (long)k * (b->ijk[2][nn] + 1) + j, l = indx3(b, i, j, k, nn);
            double cnt = F(b->rr, np, l, 1) + one;
            F(b->rr, np, l, 1) = cnt;
            double w = one / cnt;
            F(b->rr, np, l, 2) = w;
            for (int q = 1; q <= 5; q++)
              F(b->qa, np, l, q) = w * ((cnt - one) * F(b->qa, np, l, q) + b->drvb[nn][jk + nbs * ((q - 1) + 5 * ip)]);
          }
      }
    }
  }
  return ATI_OK;
}

/* ---- one time step: src/Main3D.f90:552-965 ---------------------------------- */
int orc_step(orc_case *c, int nsteps) {
  if (!c->inited) return ATI_ESTATE;
  for (int s = 0; s < nsteps; s++) {
    orc_filter_step(c);
    for (int nk = 1; nk <= c->cfg.nkrk; nk++) orc_rk_stage(c, nk);
    c->n = c->n + 1;
    c->timo = c->timo + c->dt;
    c->steps_done = c->steps_done + 1;
    if (!isfinite(c->dt)) return ATI_ENONFINITE;
  }
  return ATI_OK;
}

/* ---- clpost: src/rpt.f90:1017-1056 ---------------------------------------- */
int orc_forces(orc_case *c, double out[2]) {
  if (!c->inited) return ATI_ESTATE;
  double span = c->cfg.span;
  double dynp = two / (c->amachoo * c->amachoo * span);
  for (int dir = 1; dir <= 2; dir++) {
    double tot = 0; /* rank 0 (block 0) contributes 0, then the wall blocks in rank order */
    for (int mb = 0; mb < c->nb; mb++) {
      OBlock *b = &c->b[mb];
      if (!b->wflag) continue;
      long np = b->np, nw = b->nwall;
      double clp = 0, clv = 0;
      for (long ll = 0; ll < nw; ll++) clp = clp + (b->p[b->lwall[ll]] * b->wnor[ll + nw * (dir - 1)] * b->area[ll]);
      if (c->cfg.nviscous == 1) {
        for (long ll = 0; ll < nw; ll++) {
          long l = b->lwall[ll];
          const double *t = b->tau;
          double w1 = b->wnor[ll], w2 = b->wnor[ll + nw], w3 = b->wnor[ll + 2 * nw];
          double tw;
          if (dir == 1) tw = F(b->qa, np, l, 1) * (F(t, np, l, TXX) * w1 + F(t, np, l, TXY) * w2 + F(t, np, l, TZX) * w3);
          else tw = F(b->qa, np, l, 1) * (F(t, np, l, TXY) * w1 + F(t, np, l, TYY) * w2 + F(t, np, l, TYZ) * w3);
          clv = clv + tw * b->area[ll];
        }
      }
      tot = tot + (clp + clv) * dynp;
    }
    out[dir - 1] = tot;
  }
  return ATI_OK;
}

/* ---- accessors ------------------------------------------------------------- */
static double *field_ptr(const OBlock *b, int field, int *ncomp) {
  switch (field) {
    case ATI_F_QA: *ncomp = 5; return b->qa;
    case ATI_F_QO: *ncomp = 5; return b->qo;
    case ATI_F_DE: *ncomp = 5; return b->de;
    case ATI_F_RR: *ncomp = 3; return b->rr;
    case ATI_F_SS: *ncomp = 3; return b->ss;
    case ATI_F_XIM: *ncomp = 3; return b->xim;
    case ATI_F_ETM: *ncomp = 3; return b->etm;
    case ATI_F_ZEM: *ncomp = 3; return b->zem;
    case ATI_F_P: *ncomp = 1; return b->p;
    case ATI_F_YACO: *ncomp = 1; return b->yaco;
    case ATI_F_STRESS: *ncomp = 9; return b->tau;
    default: *ncomp = 0; return NULL;
  }
}

int orc_set_state(orc_case *c, int blk, const double *q) { return orc_set_field(c, blk, ATI_F_QA, q); }
int orc_get_state(const orc_case *c, int blk, double *q) { return orc_get_field(c, blk, ATI_F_QA, q); }

int orc_set_field(orc_case *c, int blk, int field, const double *v) {
  if (blk < 0 || blk >= c->nb || !v) return ATI_EINVAL;
  OBlock *b = &c->b[blk];
  if (field == ATI_F_SPONGE) {
    memcpy(b->asz, v, sizeof(double) * b->np);
    memcpy(b->bsz, v + b->np, sizeof(double) * b->np);
    return ATI_OK;
  }
  int nc;
  double *p = field_ptr(b, field, &nc);
  if (!p) return ATI_EINVAL;
  memcpy(p, v, sizeof(double) * nc * b->np);
  return ATI_OK;
}

int orc_get_field(const orc_case *c, int blk, int field, double *v) {
  if (blk < 0 || blk >= c->nb || !v) return ATI_EINVAL;
  const OBlock *b = &c->b[blk];
  if (field == ATI_F_SPONGE) {
    memcpy(v, b->asz, sizeof(double) * b->np);
    memcpy(v + b->np, b->bsz, sizeof(double) * b->np);
    return ATI_OK;
  }
  int nc;
  double *p = field_ptr(b, field, &nc);
  if (!p) return ATI_EINVAL;
  memcpy(v, p, sizeof(double) * nc * b->np);
  return ATI_OK;
}

int orc_get_face(const orc_case *c, int blk, int which, int nn, double *v) {
  if (blk < 0 || blk >= c->nb || nn < 1 || nn > 3 || !v) return ATI_EINVAL;
  const OBlock *b = &c->b[blk];
  long nbs = b->nbsize[nn];
  switch (which) {
    case ATI_FACE_DRVA: memcpy(v, b->drva[nn], sizeof(double) * 10 * nbs); break;
    case ATI_FACE_DRVB: memcpy(v, b->drvb[nn], sizeof(double) * 10 * nbs); break;
    case ATI_FACE_RECV: memcpy(v, b->recv[nn], sizeof(double) * 6 * nbs); break;
    case ATI_FACE_CM: memcpy(v, b->cm[nn], sizeof(double) * 6 * nbs); break;
    default: return ATI_EINVAL;
  }
  return ATI_OK;
}

int orc_get_time(const orc_case *c, ati_time_t *t) {
  t->n = c->n; t->ndt = c->ndt; t->dt = c->dt; t->dts = c->dts; t->dte = c->dte; t->timo = c->timo;
  return ATI_OK;
}

int orc_set_time(orc_case *c, const ati_time_t *t) {
  c->n = t->n; c->ndt = t->ndt; c->dt = t->dt; c->dts = t->dts; c->dte = t->dte; c->timo = t->timo;
  return ATI_OK;
}

int orc_scheme(const orc_case *c, int which, double *out) {
  switch (which) {
    case 0: memcpy(out, c->pbci, sizeof c->pbci); break;
    case 1: memcpy(out, c->pbco, sizeof c->pbco); break;
    case 2: memcpy(out, c->albed, sizeof c->albed); break;
    case 3: memcpy(out, c->albef, sizeof c->albef); break;
    case 4:
      memcpy(out, c->fam, sizeof c->fam); memcpy(out + 3, c->fbm, sizeof c->fbm); memcpy(out + 6, c->fcm, sizeof c->fcm);
      out[9] = c->fa; out[10] = c->fb; out[11] = c->fc; out[12] = c->alphf; out[13] = c->betf;
      break;
    case 5: out[0] = c->sbci[1]; out[1] = c->sbci[2]; out[2] = c->sbci[3]; break;
    case 6:
      for (int r = 0; r < 3; r++)
        for (int q = 0; q < 6; q++) out[q + 6 * r] = c->abc[r][q];
      break;
    case 7: memcpy(out, c->pbcot, sizeof c->pbcot); break;
    default: return ATI_EINVAL;
  }
  return ATI_OK;
}

int orc_factors(const orc_case *c, int blk, int nn, int filter, double *u, double *l) {
  if (blk < 0 || blk >= c->nb || nn < 1 || nn > 3) return ATI_EINVAL;
  const OBlock *b = &c->b[blk];
  int is = line_start(b, nn), len = b->ijk[1][nn] + 1, lim1 = b->lim + 1;
  const double *xu = filter ? b->yu : b->xu, *xl = filter ? b->yl : b->xl;
  for (int q = 0; q < 3; q++) memcpy(u + (size_t)q * len, xu + (size_t)q * lim1 + is, sizeof(double) * len);
  for (int q = 0; q < 2; q++) memcpy(l + (size_t)q * len, xl + (size_t)q * lim1 + is, sizeof(double) * len);
  return ATI_OK;
}

int orc_topology(const orc_case *c, int blk, int32_t nbc[6], int32_t ncd[6]) {
  if (blk < 0 || blk >= c->nb) return ATI_EINVAL;
  const OBlock *b = &c->b[blk];
  for (int ip = 0; ip <= 1; ip++)
    for (int nn = 1; nn <= 3; nn++) {
      nbc[ip * 3 + nn - 1] = b->nbc[ip][nn];
      ncd[ip * 3 + nn - 1] = b->ncd[ip][nn];
    }
  return ATI_OK;
}
