// ati_internal.h — device-side data layout of a handle: one case, or a batch
// of independent cases, with every block on one GPU.
//
// Layout in HBM
//  * A batch concatenates its cases' blocks: block b of the handle belongs to
//    case cs_b, and every per-case constant (scheme physics, time scalars)
//    lives in arrays indexed by case.
//  * Every point field is stored as [component][Ntot] doubles, where the
//    points of block b occupy [off_b, off_b + npts_b) of each component plane
//    and, inside a block, l = i + (lxi+1)*(j + (let+1)*k) (xi fastest), the
//    reference's single-rank layout (src/Subroutineso.f90:364-375).  Copying a
//    block's Fortran array f(0:lmx,ncomp) in or out is one strided 2-D copy.
//  * Face buffers (drva, drvb, recv, cm) of block b and direction nn keep the
//    reference's layout buf(0:nbsize-1, ncomp, 0:1) at face offset
//    face_off[b][nn] * ncomp * 2.
//  * LU factors of the pentadiagonal solves are interleaved per line position:
//    fac[(fac_off[b][nn] + i)*5 + {l1,l2,u1,u2,u3}], derivative and filter
//    tables separately.
#pragma once
#include <cstdint>

#include "../../include/ati.h"

namespace ati {

constexpr int LMD = 11;
constexpr int LMF = 8;
constexpr int MBCI = 3;
constexpr int MAXB = 1024;  // blocks per handle (cases x 6)

struct BlockDev {
  int lxi, let, lze;
  int nbc[2][4];   // [ip][nn], nn = 1..3
  int ncd[2][4];   // neighbour block
  int ndf[2][4];   // 1: sub-domain closure (BC 35/40/45), same for derivative and filter
  int nbsize[4];
  int64_t off;         // first point of the block in each component plane
  int64_t npts;
  int64_t face_off[4];  // face index offset (per nn)
  int64_t fac_off[4];   // factor table offset (positions)
  int cs;               // case of the block
  int pad;
};

// Work-queue entries.  Pointwise kernels walk tiles of consecutive points of
// one case; line sweeps walk tiles of consecutive lines of one block.
struct PTile {
  int cs, pad;
  int64_t g0, g1;  // points [g0, g1)
};
struct LTile {
  int b, t0;  // block, first line
};

// Scheme coefficients and physical constants of one case (built on the host
// from the same formulas as src/Main3D.f90:60-73,295-312 and
// src/Subroutineso.f90:15-159).
struct Scheme {
  double abc[3][6];
  double pbci[2][2][12];  // [nt][j][i]
  double pbco[2][2][12];
  double pbcot[2][2];     // [nt][j]
  double fam[3], fbm[3], fcm[3];
  double fa, fb, fc;
  double fex[4], ffx[4];
  double aa, ab, ac;
  // physics
  double gam, gamm1, ham, hamm1, gamm1prndtli, tgamm1prndtli, two_three;
  double srefoo, srefp1dre, rhooo, poo, amachoo, uoo[4];
  double cfl, dto, timf, wtemp, pi;
  double aoa0, aoa1, tps, tp, smago1, smago2;
  int nkrk, nviscous, nsmf, les;
};

// Time-marching scalars on the device.
struct Scalars {
  int64_t n, ndt;
  double dt, dts, dte, timo;
  double umf[4], dudtmf[4];
  double dtk;             // RK update factor of the current stage
  double aoa;
  unsigned long long cflmax[2];  // max reductions (bit patterns of doubles >= 0)
  int flag;               // bits 1, 2, 4: non-finite or non-positive state, CFL maxima or dt; FLAG_TIMEOUT: a bounded
                          // device wait gave up
};

constexpr int FLAG_TIMEOUT = 256;

// One face work item: (block, direction, side).
struct FaceTask {
  int b, nn, ip, bc;
  int nb_b;        // neighbour block (exchange faces)
  int nline;       // nbsize(nn)
  int64_t sbcc_off;  // GCBC weight list offset (4 per line) or -1
  int64_t wall_off;  // wall point list offset (rpex) or -1
};

struct JunctionDev {
  int64_t base[4];  // global point index of k = 0 on the corner line of participant 1..4
  int64_t kstride;  // (lxi+1)(let+1) of each participant (same let/lxi stride per block)
  int64_t kstr[4];
  int nk;           // lze + 1
  int pa, pb;       // participants averaged for velocities (1..4)
};

}  // namespace ati
