// ati_scheme.h — host construction of scheme coefficients and LU factors.
#pragma once
#include "ati_internal.h"

namespace ati {

struct SchemeHost {
  Scheme s;
  double albed[2][3][5];  // [ns][row][offset+2]
  double albef[2][3][5];
  double alphf, betf;
  double sbci[MBCI + 1];  // sbci[0] = 1 (boundary point), [1..3] interior weights
};

void build_scheme(const ati_config_t &cfg, SchemeHost &H);
void filter_coeffs(double fltk, double fltr, double &alphz, double &betz, double &za, double &zb, double &zc);
// LU factors of one line of length len: fac[i*5 + {l1, l2, u1, u2*u1, u3*u1}]
void penta_factors(const double albes[3][5], const double albee[3][5], double al, double be, int len, double *fac);

}  // namespace ati
