// ati_turb.h — synthetic inflow turbulence: mode tables, gust points, launchers.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "ati_internal.h"

namespace ati {

// one point of an inflow sponge zone; entries with g < 0 pad a case's list to
// a multiple of 256 so that every CTA of the evaluation works on one case
struct GustPt {
  int64_t g;          // point index
  float x, y, z, atz;  // coordinates and the streamwise ramp of spongego
  int cs, pad;
};

// the same point in FP64 (coordinates and ramp), for the FP64 synthesis of the strict arithmetic mode
struct GustPt64 {
  double x, y, z, atz;
};

// modes of one case in the concatenated table, and its freestream velocity
struct TurbCase {
  int off, n;
  double u[3];
};

// 8 floats per mode: k_x, k_y, k_z, s_x, s_y, s_z, amplitude a, phase psi
void build_modes(const ati_config_t &cfg, std::vector<float> &out);

void gust_eval(cudaStream_t st, const GustPt *pts, int64_t npts, const TurbCase *tc, const float *modes,
               const Scalars *scal, float *delta, double gam);
void gust_apply_d(cudaStream_t st, const GustPt *pts, int64_t npts, const float *delta, const double *asz,
                  const double *bsz, double *de, int64_t N);
void gust_apply_f(cudaStream_t st, const GustPt *pts, int64_t npts, const float *delta, const double *asz,
                  const double *bsz, float *de, int64_t N);
// the FP64 synthesis (ATI_FP64_STRICT, the parity mode): every operation of the mode sum and of the target
// rounded as written, in the order of the CPU restatement; delta holds 5 doubles per gust point
void gust_eval64(cudaStream_t st, const GustPt *pts, const GustPt64 *p64, int64_t npts, const TurbCase *tc,
                 const float *modes, const Scalars *scal, double *delta, double gam, double gamm1, double hamm1,
                 double ham);
void gust_apply64(cudaStream_t st, const GustPt *pts, int64_t npts, const double *delta, const double *asz,
                  const double *bsz, double *de, int64_t N);
void turb_sample(cudaStream_t st, const TurbCase *tc, int cs, const float *modes, double t, int64_t n,
                 const double *xyz, double *v);

}  // namespace ati
