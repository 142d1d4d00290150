// ati_kernels.h — launch interface of the stage engine shared by the C-ABI layer.
//
// The engine is templated on R, the type of the stage intermediates
// (primitives, gradients, stresses, fluxes, right-hand side): double for the
// FP64 path, float for the mixed path.  The conservative state qa/qo and the
// Jacobian used by the RK update are always double.
#pragma once
#include <cuda_runtime.h>

#include "ati_internal.h"
#include "ati_tma.h"

namespace ati {

// scheme coefficients in compute precision T (cast from Scheme on the host)
template <typename T>
struct Coef {
  T abc[3][6];
  T pbci[2][2][12];
  T pbco[2][2][12];
  T pbcot[2][2];
  T fam[3], fbm[3], fcm[3];
  T fa, fb, fc;
  T fex[4], ffx[4];
  T aa, ab, ac;
};

// Device pointers of a handle (one case or a batch) for intermediates of
// type R, passed by value.  Per-case data (sc, scal) is indexed by the case
// of a block (BlockDev::cs) or of a point tile (PTile::cs).
// kinds of pointwise kernel (the PW_ enumeration)
constexpr int PW_KINDS = 7;

// The segmented sweeps' tiles of one direction fall into classes of blocks whose lines have the same segment
// count (a batch mixes line lengths): one launch per class, with the warps and shared memory of the class's
// longest line.  A class is tiles [off, off + n) of lts, lines of up to maxlen points, groups line groups a CTA.
struct SegClass {
  int off, n, maxlen, groups;
};
constexpr int SEG_NCLASS = 8;  // classes per direction (more distinct segment counts share the last class)

template <typename R>
struct Eng {
  const BlockDev *blk;
  const Scheme *sc;     // [ncase]
  const Coef<R> *cf;    // shared: every case of a batch runs the same scheme
  Scalars *scal;        // [ncase]
  int ncase;
  const PTile *pt;      // pointwise work queue
  int npt;
  const LTile *lt[4];   // line-sweep work queue per direction nn = 1..3
  int nlt[4];
  const LTile *lts[4];  // segmented sweeps (mixed path): SEG_LINES x groups lines per tile, per direction, by class
  SegClass segc[4][SEG_NCLASS];
  int nsegc[4];
  const float *segd, *segf;  // their row tables (SEG_RT floats per factor row; derivative, filter)
  const float *dzm;          // dense zeta derivative operators, DENSE_MAX^2 floats per block (k_sweep_dense)
  int dzl;                   // their largest line length (0: the dense zeta sweep is not available)
  bool dense;                // the zeta derivative sweeps take the dense operators (ATI_OPT_DENSE_ZETA)
  const double *facud, *facuf;  // FP64 fast path: scaled-factor row tables (FU_RT per row; derivative, filter)
  int sg_lines[4];      // lines per CTA of the eta (2) and zeta (3) sweeps: the tiles of lt[2], lt[3]
  int maxlen[4];        // longest line per direction
  int64_t N;            // points of all blocks
  // a pointwise kernel's own point tiles, when its timed best differs from pt (index: the PW_ kind; null: pt)
  const PTile *ptk[PW_KINDS];
  int nptk[PW_KINDS];
  double *qa, *qo;      // state (5 planes each), FP64
  const double *yacod;  // Jacobian, FP64 (RK update)
  double *cnt;          // visit counts of the interface averaging (2 planes), FP64
  R *de;                // right-hand side (5 planes)
  R *prim;              // u, v, w, T (4 planes)
  R *mu, *p;            // Sutherland viscosity, pressure
  R *dv;                // d(u,v,w,T)/d(xi,eta,zeta): plane f*3 + (nn-1)
  R *tau;               // txx,tyy,tzz,txy,tyz,tzx,hxx,hyy,hzz
  R *flx;               // fluxes: plane (m-1)*3 + (nn-1)
  R *fw;                // forward-elimination scratch, one plane per field in flight
  int64_t fw_dir;       // offset between the scratch of the three directions (0: one shared scratch)
  const R *xim, *etm, *zem, *yaco;
  const R *asz, *bsz;
  R *drva, *drvb, *recv;
  const R *cm;
  const R *facd, *facf, *sbcc, *rpex;
  int64_t F;            // face index count (face buffers of one field: 6*F for recv)
  // mixed path only (the fluxes there are taken relative to the freestream):
  const R *gm;          // metric divergence sum_d D_d(metric_d) per component (3 planes)
  const R *drvm;        // its line-end values per direction, drva layout (components 0..2)
  // TMA staging of the segmented eta/zeta derivative sweeps (mixed path): tensor maps of the primitive (array 0)
  // and flux (array 1) planes per direction and block, tmaps[(array * 2 + nn - 2) * nblk + b]; tma[nn] when
  // every block's geometry allows them and the option is on
  const TmaMap *tmaps;
  int nblk;
  bool tma[4];
  bool eta_rowtiles;    // the segmented eta tiles hold the lines of one grid row each (built for TMA staging)
  bool pairs;           // segmented derivative sweeps of FP32 arrays solve two line groups a CTA (k_sweep_pair)
};

// The mixed path (R = float) works on deviations from the freestream
// (rho = 1, u = 0, p = 1/gamma): the pressure plane holds p - p_inf, the
// fluxes drop their freestream part, whose divergence is added back from the
// FP64 metric divergence gm.  Constants of that split:
template <typename R>
struct Freestream {
  static constexpr bool on = false;
};
template <>
struct Freestream<float> {
  static constexpr bool on = true;
};

enum { PW_PRIM, PW_CFL, PW_VISC, PW_FLUX, PW_DIV, PW_RK, PW_FLUX_STRESS };
static_assert(PW_FLUX_STRESS + 1 == PW_KINDS, "PW_KINDS counts the pointwise kernels");
enum { FK_GCBC_PREP, FK_GCBC_APPLY, FK_WALL, FK_PACK, FK_AVG };
enum { SC_MOVEF_A, SC_CFL_RESET, SC_DT_NEW, SC_DT, SC_MOVEF_B, SC_ADVANCE, SC_INIT };

// One line sweep over every block: nf fields, field f reads in + f*in_fs and
// writes out + f*out_fs (out2 + f*out_fs too when out2 is set); recv holds the
// closure of field f at recv + f*6*F; a derivative writes its line-end values
// to drva component m0 + f when drva is set.  When the input is wider than the
// compute type, field f is converted as (in - ofs[f]) (a constant the
// operator annihilates, removed before rounding).
template <typename TI, typename TO>
struct SweepIO {
  const TI *in;
  int64_t in_fs;
  TO *out;
  int64_t out_fs;
  TO *out2;
  int nf, m0;
  bool drva;
  TI ofs[5];
};

// lines per work-queue tile of the xi sweeps (shared-memory chunks); the
// eta/zeta sweeps take SG_MIN..SG_MAX lines per CTA and the pointwise kernels
// PT_MIN..PT_MAX points per tile, chosen per handle and pointwise kernel by timing (ati_init)
constexpr int XC_NL = 64;
constexpr int SG_MIN = 32, SG_MAX = 256, SG_DEFAULT = 128;
// (a tile of 256 points is one point per thread: consecutive CTAs then sweep
// consecutive memory, the access order of a plain grid-stride loop)
constexpr int PT_MIN = 256, PT_MAX = 4096, PT_DEFAULT = 256;
// eta/zeta sweeps keep their forward values in shared memory up to this many bytes per CTA
constexpr size_t SG_SMEM_FW = 48 * 1024;

// Segmented line solves of the mixed path: SEG_LINES lines per CTA staged
// whole in shared memory, each line cut into seg_count(L) segments of about
// SEG_ROWS points (one warp per segment).  The segmentation is a function of
// the line length alone, so a block's results do not depend on the other
// blocks or cases of a handle.  Lines up to SEG_LMAX points fit the tile.
constexpr int SEG_LINES = 32, SEG_ROWS = 48, SEG_MAX = 16, SEG_LMAX = 1600;
constexpr size_t SEG_SMEM_MAX = 227 * 1024 - 64;  // (a few bytes of static shared memory per kernel)
__host__ __device__ inline int seg_count(int L) {
  const int s = (L + SEG_ROWS - 1) / SEG_ROWS;
  return s < 1 ? 1 : (s > SEG_MAX ? SEG_MAX : s);
}
// Row table of the segmented sweeps, SEG_RT floats per LU-factor row:
//   [0] l0, [1] l1   forward-elimination factors (zero where the row has none)
//   [4] g, [5] h     the row's forward values from incoming v(s0-2) = 1, v(s0-1) = 1
//   [6] c2, [7] c3   back-substitution factors (c3 zero on the last row)
//   [8] G, [9] H     the row's back-substituted values from b(s1) = 1, b(s1+1) = 1
//   [10] c4          (zero on the last two rows); [2], [3], [11] unused
constexpr int SEG_RT = 12;
// rows of zero padding on each side of a row table (reads ahead of a segment stay in the allocation)
constexpr int SEG_PAD = 8;
// Scaled-factor row table of the FP64 fast path's line solves, FU_RT doubles
// per LU-factor row.  The forward values are carried as u(i) = c2(i) v(i), so
// the back substitution needs no multiply by c2:
//   u(i) = c2(i) r(i) - l0'(i) u(i-2) - l1'(i) u(i-1),  l0' = c2(i) l0 / c2(i-2), l1' = c2(i) l1 / c2(i-1)
//   b(i) = u(i) - c3(i) b(i+1) - c4(i) b(i+2)
// with the interior right-hand side c2(i) r(i) formed from the row's own
// weights A, B, C (c2 times the scheme's three stencil weights):
//   [0] l0', [1] l1' (zero where the row has none), [2] A, [3] B, [4] C,
//   [5] c3, [6] c4 (zero past the line end), [7] c2,
//   [8] D = 2 (A + B + C) (the filter's centre weight: its right-hand side is
//       A (a(i-1) + a(i+1)) + B (a(i-2) + a(i+2)) + C (a(i-3) + a(i+3)) - D a(i)), [9] unused
constexpr int FU_RT = 10;
// first row of segment k of S on a line of L points (the first L % S segments hold one row more)
__host__ __device__ inline int seg_start(int k, int L, int S) {
  const int q = L / S, r = L % S;
  return k * q + (k < r ? k : r);
}
// Lines of one segment leave a CTA of one warp; SEG_GROUPS groups of SEG_LINES lines then share a CTA (one
// warp and one tile each), when every line of a direction is one segment long
constexpr int SEG_GROUPS = 2;
inline int seg_groups(int maxlen) { return seg_count(maxlen) == 1 ? SEG_GROUPS : 1; }
// dynamic shared memory of a segmented sweep over lines of up to maxlen points, in groups line groups
inline size_t seg_smem_bytes(int maxlen, int groups) {
  const int nwarp = groups > 1 ? groups : seg_count(maxlen);
  return (size_t)nwarp * SEG_LINES * 2 * 2 * sizeof(float) + (size_t)groups * maxlen * (SEG_LINES + 1) * sizeof(float);
}
// Dense zeta derivative sweeps (k_sweep_dense): lines of up to DENSE_MAX points, each block's operator an
// L x L matrix in DENSE_MAX x DENSE_MAX storage
constexpr int DENSE_MAX = 64;
// Paired sweeps (k_sweep_pair) take the classes of lines of up to PAIR_MAX_SEG segments
constexpr int PAIR_MAX_SEG = 4;
// ... and of a paired sweep (k_sweep_pair: two line groups, one warp per segment, or one warp when single)
inline size_t pair_smem_bytes(int maxlen, bool single) {
  const int nwarp = single ? 1 : seg_count(maxlen);
  return (size_t)nwarp * SEG_LINES * 2 * 4 * sizeof(float) + (size_t)2 * maxlen * (SEG_LINES + 1) * sizeof(float);
}

// The face lines of a range of face tasks as one index space (fused face chains): tasks t[0..n), cum[q] the
// running count of lines before task q (cum[n] - cum[0] = total).
struct TaskSpan {
  const FaceTask *t;
  const int64_t *cum;
  int n;
  int64_t total;
};
// One fused face chain launch: before the RK update prep = the GCBC faces, dir[d] = the GCBC faces of direction d;
// after it prep = the wall faces, pack = the averaged faces, dir[d] = the averaged faces of direction d, plus the
// junction lines.  bar: the grid-barrier counter (zero at launch), limit: polls a barrier wait may take.
struct FaceChain {
  TaskSpan prep, pack, dir[4];
  const JunctionDev *jn;
  int njct, jnk;
  unsigned *bar;
  unsigned limit;
  int nk;
};

// per-field offsets of a closure (mpigo) over a wider input type
template <typename TI>
struct FieldOfs {
  TI v[5];
};

// Launchers, declared once per arithmetic mode: ati::fast (FMA contraction)
// and ati::strict (every operation rounded, -fmad=false).  Sweep and closure
// launchers exist for (in, out, compute) = (d,d,d), (f,f,f) and (d,d,f).
#define ATI_DECLARE_LAUNCHERS(NS)                                                                                  \
  namespace NS {                                                                                                   \
  void sweep_ddd(const Eng<double> &e, cudaStream_t st, int nn, bool filt, const SweepIO<double, double> &io); \
  void sweep_fff(const Eng<float> &e, cudaStream_t st, int nn, bool filt, const SweepIO<float, float> &io); \
  void sweep_ddf(const Eng<float> &e, cudaStream_t st, int nn, bool filt, const SweepIO<double, double> &io); \
  void mpigo_ddd(const Eng<double> &e, cudaStream_t st, const FaceTask *tasks, int ntask, int maxline, int nt,      \
                 int n45, const double *s1, const double *s2, const double *s3, int64_t fs, int nf);              \
  void mpigo_fff(const Eng<float> &e, cudaStream_t st, const FaceTask *tasks, int ntask, int maxline, int nt,       \
                 int n45, const float *s1, const float *s2, const float *s3, int64_t fs, int nf);                 \
  void mpigo_ddf(const Eng<float> &e, cudaStream_t st, const FaceTask *tasks, int ntask, int maxline, int nt,       \
                 int n45, const double *s1, const double *s2, const double *s3, int64_t fs, int nf,               \
                 const FieldOfs<double> &ofs);                                                                     \
  cudaError_t seg_init();                                                                                          \
  void metric_divergence(const Eng<double> &e, cudaStream_t st, const double *d3, float *gm);                     \
  void pointwise_d(const Eng<double> &e, cudaStream_t st, int which);                                             \
  void pointwise_f(const Eng<float> &e, cudaStream_t st, int which);                                              \
  void face_d(const Eng<double> &e, cudaStream_t st, int which, const FaceTask *tasks, int ntask, int maxline);    \
  void face_f(const Eng<float> &e, cudaStream_t st, int which, const FaceTask *tasks, int ntask, int maxline);     \
  void junction(const Eng<double> &e, cudaStream_t st, const JunctionDev *jn, int njct, int nk);                   \
  void scalar(const Eng<double> &e, cudaStream_t st, int op, int nk);                                             \
  void metrics(const Eng<double> &e, cudaStream_t st, const double *xyz_d);                                       \
  cudaError_t face_pre_d(const Eng<double> &e, cudaStream_t st, const FaceChain &c);                               \
  cudaError_t face_pre_f(const Eng<float> &e, cudaStream_t st, const FaceChain &c);                                \
  cudaError_t face_post(const Eng<double> &e, cudaStream_t st, const FaceChain &c);                                \
  void forces_d(const Eng<double> &e, cudaStream_t st, const FaceTask *tasks, int ntask, const double *area,       \
                const double *wnor, const int64_t *woff, double *out);                                             \
  void forces_f(const Eng<float> &e, cudaStream_t st, const FaceTask *tasks, int ntask, const double *area,        \
                const double *wnor, const int64_t *woff, double *out);                                             \
  }
ATI_DECLARE_LAUNCHERS(fast)
ATI_DECLARE_LAUNCHERS(strict)
#undef ATI_DECLARE_LAUNCHERS

}  // namespace ati
