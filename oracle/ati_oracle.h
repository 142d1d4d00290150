/*
 * ati_oracle.h — CPU restatement of the ATI3D per-RK-stage path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (tandemproject_gb300/,
 * include/) links, loads or calls this code; only tests/, the smoke check in
 * __graft_entry__.py and the CPU-baseline leg of bench.py use it, as the
 * checker.
 *
 * Parity status: the reference (Fortran 90 + MPI) cannot be compiled here or
 * on the GPU machine (no Fortran compiler, no MPI) and ships no tests, golden
 * vectors or recorded outputs, so this restatement is "parity unpinned"
 * against the reference itself.  It is pinned instead by known-answer tests
 * derived from the reference source (tests/test_oracle_kat.py) and by an
 * independent dense-matrix numpy restatement of the line operators
 * (tests/golden/make_golden.py).
 *
 * The entry points mirror include/ati.h one for one (same config struct,
 * same field ids, same selector arguments), so tests drive the oracle and
 * the CUDA path with identical call sequences.
 */
#ifndef ATI_ORACLE_H
#define ATI_ORACLE_H

#include "../include/ati.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_case orc_case;

int orc_create(const ati_config_t *cfg, orc_case **out);
void orc_destroy(orc_case *c);
int orc_nblocks(const orc_case *c);
int orc_block_dims(const orc_case *c, int blk, int32_t dims[3], int64_t *npts);
int orc_set_grid(orc_case *c, int blk, const double *xyz);
int orc_init(orc_case *c);
int orc_set_state(orc_case *c, int blk, const double *q);
int orc_get_state(const orc_case *c, int blk, double *q);
int orc_set_field(orc_case *c, int blk, int field, const double *v);
int orc_get_field(const orc_case *c, int blk, int field, double *v);
int orc_get_face(const orc_case *c, int blk, int which, int nn, double *v);
int orc_get_time(const orc_case *c, ati_time_t *t);
int orc_set_time(orc_case *c, const ati_time_t *t);
int orc_mpigo(orc_case *c, int nt, int nrt, int n45);
int orc_deriv(orc_case *c, int nn, int nz, int m);
int orc_filte(orc_case *c, int nn, int nz);
int orc_filter_step(orc_case *c);
int orc_rk_stage(orc_case *c, int nk);
int orc_step(orc_case *c, int nsteps);
int orc_forces(orc_case *c, double out[2]);
/* Inflow turbulence after orc_init: nmodes Fourier modes, 8 floats each (k_x, k_y, k_z, s_x, s_y, s_z, a, psi, the
 * table ati_turbulence_modes returns), summed in FP64 at the inflow sponge's gust points; 0 modes turn it off. */
int orc_set_turbulence(orc_case *c, const float *modes, int nmodes);
/* The mode table of cfg's inflow turbulence (8 floats per mode; the GPU library's generator restated): returns the
 * mode count, 0 for none; with out == NULL only the count. */
int orc_build_modes(const ati_config_t *cfg, float *out);
void orc_set_threads(int n);
int orc_get_threads(void);

/* Scheme coefficients, for known-answer tests:
 * which = 0 pbci, 1 pbco (each [nt][j][0..11]), 2 albed, 3 albef (each
 * [ns][row][-2..2]), 4 filter rows fam,fbm,fcm,fa,fb,fc,alphf,betf,
 * 5 sbci(1..3), 6 abc(0:5,0:2) column-major, 7 pbcot[nt][j]. */
int orc_scheme(const orc_case *c, int which, double *out);
/* LU factors of one block and direction: xu (len,3), xl (len,2) for the
 * derivative (filter = 0) or yu, yl for the filter (filter = 1). */
int orc_factors(const orc_case *c, int blk, int nn, int filter, double *u, double *l);
/* Boundary codes and neighbour blocks: out[ip*3+nn-1] */
int orc_topology(const orc_case *c, int blk, int32_t nbc[6], int32_t ncd[6]);

#ifdef __cplusplus
}
#endif
#endif
