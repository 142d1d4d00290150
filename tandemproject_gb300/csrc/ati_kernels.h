// ati_kernels.h — kernel launch interface shared by the C-ABI layer.
#pragma once
#include <cuda_runtime.h>

#include "ati_internal.h"

namespace ati {

// Device pointers of one case, passed to every kernel by value.
struct Ctx {
  const BlockDev *blk;
  const Scheme *sc;
  Scalars *scal;
  int64_t N;  // points of all blocks
  double *qa, *qo, *de, *rr, *ss, *xim, *etm, *zem, *p, *yaco, *tau, *asz, *bsz, *fw;
  double *drva, *drvb, *recv, *cm;
  const double *facd, *facf, *sbcc, *rpex;
};

enum { PW_PRIM, PW_CFL, PW_GRAD, PW_STRESS, PW_FLUXPREP, PW_FLUX, PW_DIV, PW_RK, PW_METRICS };
enum { FK_GCBC_PREP, FK_GCBC_APPLY, FK_WALL, FK_PACK, FK_AVG };
enum { SC_MOVEF_A, SC_CFL_RESET, SC_DT_NEW, SC_DT, SC_MOVEF_B, SC_ADVANCE, SC_INIT };

// Launchers, declared once per arithmetic mode: ati::fast (FMA contraction)
// and ati::strict (every operation rounded, -fmad=false).
#define ATI_DECLARE_LAUNCHERS(NS) \
  namespace NS { \
  void launch_sweep(const Ctx &c, cudaStream_t st, int nn, bool filt, const double *in, double *out, int m, int nblocks, \
                    int maxlines); \
  void launch_mpigo(const Ctx &c, cudaStream_t st, const FaceTask *tasks, int ntask, int maxline, int nt, int n45, \
                    const double *s1, const double *s2, const double *s3); \
  void launch_pointwise(const Ctx &c, cudaStream_t st, int which, int m, double *o1, double *o2, double *o3); \
  void launch_face(const Ctx &c, cudaStream_t st, int which, const FaceTask *tasks, int ntask, int maxline); \
  void launch_junction(const Ctx &c, cudaStream_t st, const JunctionDev *jn, int njct, int nk); \
  void launch_scalar(const Ctx &c, cudaStream_t st, int op, int nk); \
  void launch_forces(const Ctx &c, cudaStream_t st, const FaceTask *tasks, int ntask, const double *area, \
                     const double *wnor, const int64_t *woff, double *out); \
  }
ATI_DECLARE_LAUNCHERS(fast)
ATI_DECLARE_LAUNCHERS(strict)
#undef ATI_DECLARE_LAUNCHERS

}  // namespace ati
