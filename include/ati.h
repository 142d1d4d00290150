/*
 * ati.h — C ABI of the GB300 per-Runge–Kutta-stage hot path of the ATI3D
 * compressible Navier–Stokes solver (rpt1g12/tandemProject).
 *
 * The reference exposes this path as Fortran module procedures that take only
 * small integer selectors and work on module-global arrays:
 *   mpigo(nt,nrt,n45,itag)   src/Subroutines3D.f90:16-80
 *   deriv(nn,nz,m)           src/Subroutines3D.f90:84-141
 *   filte(nn,nz)             src/Subroutines3D.f90:145-206
 * and as inline code in the time loop of program main3d
 *   per-step filter          src/Main3D.f90:555-561
 *   one RK stage             src/Main3D.f90:567-958
 *   one time step            src/Main3D.f90:552-965
 * Here the globals become a handle that owns every device array of one case
 * (all blocks of the multi-block grid live on one GPU), and each entry point
 * keeps the reference's selector arguments and meaning.
 *
 * Conventions
 *  - Every call returns an int status (ATI_OK == 0); ati_last_error() gives text.
 *  - Host pointers are borrowed for the duration of the call only.
 *  - Arrays cross the boundary in the reference's Fortran layout: a block field
 *    f(0:lmx,ncomp) is ncomp contiguous planes of (lxi+1)(let+1)(lze+1)
 *    doubles, point index l = i + (lxi+1)*(j + (let+1)*k), i = xi fastest
 *    (src/Subroutineso.f90:364-375 indx3, nn=1).
 *  - One CUDA stream per handle; calls on one handle must not run
 *    concurrently; different handles are independent.  Calls are asynchronous
 *    on that stream except the ati_get_* copies, which synchronise.
 *  - No CPU fallback: a handle cannot be created without a CUDA device.
 */
#ifndef ATI_H
#define ATI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ATI_ABI_VERSION 2
#define ATI_MAX_BK 8 /* max blocks per grid direction */

/* ---- status codes ------------------------------------------------------ */
#define ATI_OK 0
#define ATI_EINVAL 1      /* bad argument or configuration                   */
#define ATI_ENOMEM 2      /* device or host allocation failed                */
#define ATI_ECUDA 3       /* CUDA runtime error                              */
#define ATI_ENONFINITE 4  /* NaN/Inf or non-positive rho/p seen on device    */
#define ATI_ETIMEDOUT 5   /* a bounded device or host wait gave up           */
#define ATI_ESTATE 6      /* call out of order (e.g. step before init)       */

/* ---- precision of the fused stage (ati_config_t.precision) -------------- */
#define ATI_FP64 0  /* every array and operation in FP64 (the reference's nr=ieee64) */
#define ATI_MIXED 1 /* line solves, filters, fluxes in FP32; metrics, Jacobian and
                       RK state (qa, qo) in FP64 */
#define ATI_FP64_STRICT 2 /* FP64 with every operation rounded as written (no fused
                             multiply-add contraction): matches the CPU restatement
                             to the last bit except where libm differs */

/* ---- field identifiers (the reference's module arrays) ------------------
 * src/MainVar3D.f90:78-85.  ncomp in brackets. */
#define ATI_F_QA 0    /* qa   [5] conservative state (rho, rho u, rho v, rho w, rho E) */
#define ATI_F_QO 1    /* qo   [5] state at the start of the time step          */
#define ATI_F_DE 2    /* de   [5] primitives / right-hand side                  */
#define ATI_F_RR 3    /* rr   [3] line-sweep work field                          */
#define ATI_F_SS 4    /* ss   [3] work field (grid coordinates at set-up)        */
#define ATI_F_XIM 5   /* xim  [3] d(xi)/dx etc. times J^-1 (non-conservative)    */
#define ATI_F_ETM 6   /* etm  [3]                                                */
#define ATI_F_ZEM 7   /* zem  [3]                                                */
#define ATI_F_P 8     /* p    [1] pressure                                       */
#define ATI_F_YACO 9  /* yaco [1] Jacobian J = 3 / sum(...)                       */
#define ATI_F_STRESS 10 /* [9] txx,tyy,tzz,txy,tyz,tzx,hxx,hyy,hzz              */
#define ATI_F_SPONGE 11 /* [2] dense sponge coefficients asz, bsz (0 outside)    */
#define ATI_F_CP 12   /* [1] derived, ati_get_field only: pressure coefficient of the
                         current qa, (p - p_inf) * 2 / M^2 (getCp, src/rptPost.f90:1456-1465) */
#define ATI_NFIELDS 13

/* ---- face buffers: drva/drvb/recv/cm (src/MainVar3D.f90:96-102) --------
 * Layout as in the reference: buf(0:nbsize(nn)-1, ncomp, 0:1), face index
 * jk = k*(ijk(2,nn)+1) + j (src/Main3D.f90:203-207). */
#define ATI_FACE_DRVA 0 /* [5] boundary derivatives / characteristic R      */
#define ATI_FACE_DRVB 1 /* [5] neighbour's drva (GCIC) / packed qa (averaging) */
#define ATI_FACE_RECV 2 /* [3] sub-domain closure received by mpigo           */
#define ATI_FACE_CM 3   /* [3] unit face normals                              */

/* ---- boundary-condition codes (src/SingleTurbulence3D.f90:121-164) ------ */
#define ATI_BC_INOUT 10    /* non-reflecting inflow/outflow GCBC */
#define ATI_BC_WALL_INV 20 /* inviscid wall                      */
#define ATI_BC_WALL 25     /* isothermal no-slip wall            */
#define ATI_BC_INTER 30    /* characteristic interface (GCIC)    */
#define ATI_BC_AVG 35      /* averaged interface                 */
#define ATI_BC_SPLIT 40    /* internal split                     */
#define ATI_BC_PERIODIC 45 /* periodic (self exchange)           */

/* ---- configuration: the hot-path fields of inputo.dat / inputp.dat ------
 * src/Main3D.f90:34-58 and src/SingleTurbulence3D.f90:39-62.  The block
 * topology is the reference's H-grid (domdcomp, src/SingleTurbulence3D.f90:
 * 121-164) with one sub-block per block (npc = 1): bkx*bky*bkz blocks,
 * block mb = j*bkx + i, spanwise periodic, wall on top of block 1 and under
 * block 4, inflow/outflow on the outer faces, interfaces elsewhere. */
typedef struct ati_config {
  int32_t bkx, bky, bkz;      /* blocks per direction (inputo.dat line 1)      */
  int32_t lxibk[ATI_MAX_BK];  /* last xi index per block column (lxi0-to-bkx)  */
  int32_t letbk[ATI_MAX_BK];  /* last eta index per block row                  */
  int32_t lzebk[ATI_MAX_BK];  /* last zeta index per block plane               */
  int32_t nkrk;               /* RK stages (4)                                 */
  int32_t nviscous;           /* 1: Navier–Stokes, 0: Euler                    */
  int32_t nsmf;               /* 1: frame velocity = freestream at once        */
  int32_t les;                /* 1: Smagorinsky LES branch                     */
  int32_t precision;          /* ATI_FP64 or ATI_MIXED                         */
  int32_t turb_modes;         /* inflow turbulence: Fourier modes (0: none)    */
  int32_t turb_seed;          /* seed of the mode directions and phases        */
  int32_t reserved_i[5];
  double reoo, tempoo;          /* Reynolds number, freestream temperature (K) */
  double amach1, amach2, amach3;/* freestream Mach components                 */
  double wtemp;                 /* wall temperature ratio                      */
  double cfl;                   /* CFL number (used when dto < 0)              */
  double timf;                  /* frame ramp time (nsmf = 0)                  */
  double fltk, fltkbc;          /* filter cut-offs as fractions of pi          */
  double dto;                   /* fixed dt if > 0, CFL mode if < 0            */
  double aoa0, aoa1, tps, tp;   /* pitching (active when tp > 0)               */
  double smago1, smago2;        /* LES constants                               */
  double domlen, span;          /* domain length, span (inputp.dat)            */
  double szth1, szth2, szxt, szco; /* sponge thicknesses and strength         */
  double turb_intensity;        /* inflow turbulence: rms of each velocity
                                   component as a fraction of |U_inf|          */
  double turb_length;           /* von Karman integral length scale            */
  double reserved_d[6];
} ati_config_t;

/* Time-marching scalars (src/MainVar3D.f90:121,141), restart header order
 * of wrRsta (src/rpt.f90:589-600). */
typedef struct ati_time {
  int64_t n, ndt;
  double dt, dts, dte, timo;
} ati_time_t;

typedef struct ati_handle ati_handle_t;

/* ---- lifetime ----------------------------------------------------------- */
/* Allocate all device arrays of one case (src/Main3D.f90:270-291) and build
 * the scheme coefficients (penta, fcbcm, fcint, sbcco: src/Main3D.f90:295-332). */
int ati_create(const ati_config_t *cfg, ati_handle_t **out);
/* A batch: ncase independent cases in one handle (no counterpart in the
 * reference, which runs one case per MPI job).  Their blocks are concatenated
 * (case c owns blocks 6c .. 6c+5), every kernel launch of a step covers all
 * cases through a work queue of (case, block, line tile) and (case, point
 * tile) entries, and one CUDA graph replays a step of the whole batch.  The
 * cases may differ in block sizes and physics (Re, T_inf, Mach, angle of
 * attack, wall temperature, CFL, sponge, span) but share the numerics:
 * nkrk, nviscous, les, precision, fltk and fltkbc.  They step together (one
 * step count n), each with its own dt.  Calls without a case argument refer
 * to case 0, except ati_set_time (every case) and the block-indexed ones. */
int ati_create_batch(const ati_config_t *cfgs, int ncase, ati_handle_t **out);
int ati_case_count(ati_handle_t *h, int *ncase);
int ati_case_blocks(ati_handle_t *h, int cs, int *first_block, int *nblocks);
int ati_case_time(ati_handle_t *h, int cs, ati_time_t *t);
/* t->n must equal the batch's step count when the handle holds several cases. */
int ati_case_set_time(ati_handle_t *h, int cs, const ati_time_t *t);
int ati_case_config(ati_handle_t *h, int cs, ati_config_t *cfg);
int ati_destroy(ati_handle_t *h);
const char *ati_last_error(const ati_handle_t *h);
int ati_abi_version(void);
int ati_synchronize(ati_handle_t *h);

/* Grid coordinates of block blk: xyz(0:lmx,3) = x,y,z planes, as rdGrid
 * leaves them in ss(:,1:3) (src/rpt.f90:673-696). */
int ati_set_grid(ati_handle_t *h, int blk, const double *xyz);

/* After every block's grid is set: metrics and Jacobian on the device
 * (src/Main3D.f90:365-413), face normals (:429-439), GCBC weights
 * (:443-480), sponge (spongeup, src/SingleTurbulence3D.f90:209-249), and
 * the initial condition of initialo (:203) with n = 0, dt = 0. */
int ati_init(ati_handle_t *h);

/* Synthetic inflow turbulence (new: the reference's own inflow-eddy generator
 * is disabled, src/SingleTurbulence3D.f90:260).  With turb_modes > 0 the sponge
 * of spongego (src/SingleTurbulence3D.f90:332-374) drives the points of the
 * inflow sponge zone (x < -0.7 domlen + szth1) towards a turbulent target
 * instead of rest, through the reference's gust form: rho_t = (1 - (gamma-1)/2
 * |v|^2)^(1/(gamma-1)), momentum target atz rho_t v, pressure target
 * rho_t^gamma / gamma, atz = sin^2(min(pi (x + domlen) / szth1, pi/2)).  The
 * velocity is a sum of turb_modes Fourier modes of a von Karman spectrum
 * (E(k) ~ (k/ke)^4 / (1 + (k/ke)^2)^(17/6), ke = 0.747 / turb_length), with
 * directions, polarisations and phases uniform from turb_seed, divergence free,
 * scaled to turb_intensity |U_inf| rms per component and convected with the
 * freestream: v(x, t) = sum_n 2 a_n s_n cos(k_n . (x - U_inf t) + psi_n).  The
 * field is evaluated in FP32 at the start time of the first step and of every
 * step that takes a new dt (n % 10 == 1), and held in between.
 * ati_turbulence_modes copies case cs's table (8 floats per mode: k_x, k_y,
 * k_z, s_x, s_y, s_z, a, psi) and ati_turbulence_sample evaluates v at n given
 * points (xyz: x[n], y[n], z[n]; v likewise) at time t on the device. */
int ati_turbulence_modes(ati_handle_t *h, int cs, float *modes, int32_t *nmodes);
int ati_turbulence_sample(ati_handle_t *h, int cs, double t, int64_t n, const double *xyz, double *v);

/* Grid check after ati_init (no counterpart in the reference): flags[b] for
 * every block b has bit 0 set if some Jacobian J = yaco is positive, bit 1 if
 * some is negative, bit 2 if some is zero or not finite.  A block whose J
 * changes sign (flags 3) folds under the compact-derivative metrics, and the
 * reference's scheme diverges on it within a few dozen steps. */
int ati_jacobian_sign(ati_handle_t *h, int32_t *flags);

/* State and field copies (block blk, Fortran layout, all components). */
int ati_set_state(ati_handle_t *h, int blk, const double *q);
int ati_get_state(ati_handle_t *h, int blk, double *q);
/* The whole state of a handle in one transfer per direction (no counterpart in
 * the reference, where each MPI rank holds one block): q[c * n + g] for
 * component c = 0..4 and point g of all blocks in handle order (block b's
 * points at g = off_b .. off_b + npts_b - 1, off_b the sum of the earlier
 * blocks' npts), n = ati_points_total.  With pinned host memory each call is
 * one DMA copy; ati_get_state_all waits for it. */
int ati_set_state_all(ati_handle_t *h, const double *q);
int ati_get_state_all(ati_handle_t *h, double *q);
int ati_points_total(ati_handle_t *h, int64_t *n);
int ati_set_field(ati_handle_t *h, int blk, int field, const double *v);
int ati_get_field(ati_handle_t *h, int blk, int field, double *v);
int ati_get_face(ati_handle_t *h, int blk, int which, int nn, double *v);
int ati_get_time(ati_handle_t *h, ati_time_t *t);
int ati_set_time(ati_handle_t *h, const ati_time_t *t);
/* Sizes: npts of block blk, and nbsize(nn) of its faces. */
int ati_block_dims(ati_handle_t *h, int blk, int32_t dims[3], int64_t *npts);

/* ---- granular calls, one per reference procedure, over all blocks ------- */
/* mpigo(nt,nrt,n45,itag), src/Subroutines3D.f90:16-80: closure values of the
 * faces with ndf = 1, exchanged on the device (BC 45: the line's other end). */
int ati_mpigo(ati_handle_t *h, int nt, int nrt, int n45);
/* deriv(nn,nz,m), src/Subroutines3D.f90:84-141: rr(:,nn) = d rr(:,nz) / d
 * xi_nn on every line; boundary values to drva_nn(:,m,0:1). */
int ati_deriv(ati_handle_t *h, int nn, int nz, int m);
/* filte(nn,nz), src/Subroutines3D.f90:145-206: rr(:,nz) += filter correction. */
int ati_filte(ati_handle_t *h, int nn, int nz);

/* ---- fused calls -------------------------------------------------------- */
/* Per-step filter of the five conservative variables, then qo = qa
 * (src/Main3D.f90:555-561). */
int ati_filter_step(ati_handle_t *h);
/* One RK stage nk = 1..nkrk (src/Main3D.f90:567-958). */
int ati_rk_stage(ati_handle_t *h, int nk);
/* nsteps full time steps: filter, nkrk stages, n += 1, timo += dt
 * (src/Main3D.f90:552-965).  Returns ATI_ENONFINITE if the state blew up. */
int ati_step(ati_handle_t *h, int nsteps);
/* For a host that drives many handles at once (no counterpart in the
 * reference): ati_step_async issues the steps and returns without waiting;
 * ati_query sets *idle = 1 once the handle's stream has finished its work;
 * ati_check waits for it and returns ati_step's status (ATI_ENONFINITE if
 * the state blew up). */
int ati_step_async(ati_handle_t *h, int nsteps);
int ati_query(ati_handle_t *h, int *idle);
int ati_check(ati_handle_t *h);
/* Failure detection (the reference's only check is the dt = 0 "Overflow."
 * stop, src/Main3D.f90:1086-1090).  Every case of a handle has its own device
 * flag, set by the primitives kernel for a NaN/Inf or non-positive density or
 * pressure, by the CFL maxima or by a non-finite dt; it stays set until
 * ati_init.  Cases of a batch share no data on the device, so a case that
 * fails keeps stepping (its state stays non-finite) while the others go on
 * unchanged: ati_step and ati_check name the first failed case, and
 * ati_case_check returns ATI_ENONFINITE for case cs alone if it failed. */
int ati_case_check(ati_handle_t *h, int cs);
/* Bounded host waits (no counterpart in the reference): with seconds > 0,
 * ati_synchronize, ati_step, ati_check and ati_case_check poll the handle's
 * stream and give up after that long with ATI_ETIMEDOUT, the work still in
 * flight (a later wait picks it up); 0 (the default) waits without limit.
 * The ati_get_* copies always wait without limit. */
int ati_set_wait_timeout(ati_handle_t *h, double seconds);

/* ---- instrumentation (no counterpart in the reference) ------------------
 * With profiling enabled every kernel launch of the handle is bracketed by
 * CUDA events on the handle's stream and its device time is summed per
 * kernel class (ATI_K_*); ati_profile_read synchronises and returns the sums
 * in milliseconds with the launch counts.  ati_launch_count counts every
 * kernel launch since creation, profiled or not. */
#define ATI_K_DERIV_XI 0
#define ATI_K_DERIV_ETA 1
#define ATI_K_DERIV_ZETA 2
#define ATI_K_FILTER_XI 3
#define ATI_K_FILTER_ETA 4
#define ATI_K_FILTER_ZETA 5
#define ATI_K_MPIGO 6
#define ATI_K_PRIM 7
#define ATI_K_CFL 8
#define ATI_K_VISC 9
#define ATI_K_FLUX 10
#define ATI_K_DIV 11
#define ATI_K_RK 12
#define ATI_K_GCBC 13
#define ATI_K_WALL_JUNCTION 14
#define ATI_K_AVERAGE 15
#define ATI_K_SCALAR 16
#define ATI_K_NSLOTS 17
/* Profiling replaces the CUDA-graph replay of ati_step by eager launches. */
int ati_profile_enable(ati_handle_t *h, int enable);
int ati_profile_read(ati_handle_t *h, int nslots, double *ms, int64_t *launches);
int ati_launch_count(ati_handle_t *h, int64_t *count);
/* Work-queue tile shapes in use: out[0] xi lines per CTA, out[1] eta and
 * out[2] zeta lines per CTA, out[3] points per tile of the flux kernel.
 * ati_init picks out[1..2] and, per pointwise kernel, the points per tile by
 * timing candidates on the handle's own grid (results do not depend on them:
 * every line and point is computed the same way). */
int ati_tiles(ati_handle_t *h, int32_t out[4]);
/* Pins the tile shapes (same meaning as ati_tiles; 0 keeps the current value;
 * in[3] then applies to every pointwise kernel): in[0] must be 0 or the fixed
 * xi tile, in[1] and in[2] multiples of 32 in [32, 256], in[3] a multiple of
 * 256 in [256, 4096].  Waits for the steps in flight and re-captures the step
 * graphs at the next step. */
int ati_set_tiles(ati_handle_t *h, const int32_t in[4]);
/* The whole tile choice of a handle, to reuse it on a handle of the same
 * block shapes without timing candidates again (a host that starts many
 * similar cases; results do not depend on tiles): plan[0..3] as ati_tiles,
 * plan[4 + k] the points per tile of pointwise kernel k (0: the shared queue
 * of plan[3]; otherwise one of the sizes ati_init times).  ati_set_tuning(h, 0)
 * before ati_init skips the timing (the handle then runs on the default tiles
 * until ati_set_tile_plan); ati_set_tile_plan waits for the steps in flight and
 * re-captures the step graphs at the next step. */
#define ATI_TILE_PLAN 11
int ati_set_tuning(ati_handle_t *h, int enable);
int ati_get_tile_plan(ati_handle_t *h, int32_t plan[ATI_TILE_PLAN]);
int ati_set_tile_plan(ati_handle_t *h, const int32_t plan[ATI_TILE_PLAN]);
/* Kernel options (no counterpart in the reference; results do not depend on
 * them, only timings do, except ATI_OPT_DENSE_ZETA's by FP32 rounding).
 * ATI_OPT_TMA, ATI_OPT_PAIRED_LINES and ATI_OPT_STRESS_AT_POINT are on by
 * default, ATI_OPT_FUSED_FACES (measured slower inside the step graphs) and
 * ATI_OPT_DENSE_ZETA off.
 *  ATI_OPT_TMA: the mixed path's segmented eta and zeta derivative sweeps
 *    stage each tile of 32 lines into shared memory with one tensor copy
 *    (TMA, cp.async.bulk.tensor) on every direction whose blocks' FP32 planes
 *    a tensor map can describe (plane bases and row or plane sizes multiples
 *    of 16 bytes, lines of at most 256 points); off, or elsewhere, with
 *    per-thread asynchronous copies.
 *  ATI_OPT_FUSED_FACES: the face and scalar work around the RK update of a
 *    stage (src/Main3D.f90:780-952) runs as two cooperative launches whose
 *    phases are ordered by grid barriers with bounded waits (see
 *    ati_set_spin_limit), instead of one launch per face kind and direction.
 *  ATI_OPT_PAIRED_LINES: the mixed path's segmented derivative sweeps solve
 *    two groups of 32 lines per CTA, each lane two lines, on lines of up to
 *    four segments (192 points; longer ones one group per CTA).
 *  ATI_OPT_DENSE_ZETA (off by default; its results differ from the
 *    recurrence's by FP32 rounding): the mixed path's zeta derivatives as
 *    one dense L x L product per line, the operator of each block built once
 *    from the line algorithm in FP64, where every zeta face is periodic onto
 *    its own block and lines have 13 to 64 points (else it has no effect).
 *  ATI_OPT_STRESS_AT_POINT: the ATI_FP64 path's viscous fluxes take the
 *    stresses at the point inside the flux kernel instead of writing and
 *    reading nine stress planes (no effect in the strict mode, the mixed path
 *    or with the LES term; the stress output and the forces rebuild the planes
 *    on demand).
 * *active (may be NULL) gets the options in effect, plus ATI_OPT_TMA_ETA and
 * ATI_OPT_TMA_ZETA for the directions staged by TMA.  Waits for the steps in
 * flight; the step graphs are captured again. */
#define ATI_OPT_TMA 1
#define ATI_OPT_FUSED_FACES 2
#define ATI_OPT_TMA_ETA 4
#define ATI_OPT_TMA_ZETA 8
#define ATI_OPT_PAIRED_LINES 16
#define ATI_OPT_STRESS_AT_POINT 32
#define ATI_OPT_DENSE_ZETA 64
int ati_set_options(ati_handle_t *h, int flags, int32_t *active);
/* The dense zeta operator ATI_OPT_DENSE_ZETA applies (no counterpart in the
 * reference; host only, needs no device): M (*L x *L, row-major, FP64, room
 * for 64 x 64 doubles) with d = M f the zeta derivative of a zeta line f of
 * block blk, src/Subroutines3D.f90:84-141 with the periodic closure of
 * src/Subroutines3D.f90:16-80 (n45 = 0) folded in.  The device takes M
 * rounded to FP32.  ATI_EINVAL where the case's zeta lines do not qualify
 * (see ATI_OPT_DENSE_ZETA). */
int ati_dense_zeta_operator(const ati_config_t *cfg, int blk, double *M, int32_t *L);
/* Device-side waits are bounded (no counterpart in the reference): a grid
 * barrier of the fused face chains gives up after this many polls (0 = the
 * default, 2^24, seconds), marks every case of the handle, and the next
 * ati_step / ati_check / ati_case_check returns ATI_ETIMEDOUT.  The state is
 * then not valid: set it (or call ati_init) before stepping on.  The TMA tile
 * waits of the segmented sweeps have their own fixed bound and report the
 * same way. */
int ati_set_spin_limit(ati_handle_t *h, int64_t polls);
/* The handle's CUDA stream (a cudaStream_t), for callers that order their
 * own work or events against the solver's. */
void *ati_stream(ati_handle_t *h);
/* FMA throughput of the current device (independent FMA chains, no memory
 * traffic) in TFLOP/s, FP64 when fp64 != 0 else FP32: the compute roofline
 * denominator of the FP64 path. */
int ati_probe_fma_tflops(int fp64, double *tflops);
/* The mixed path widens FP32 to FP64 with integer and bit operations (the
 * FP64 pipe that runs the conversion instruction is GB300's slowest); this
 * runs both forms on n device-generated bit patterns covering every exponent,
 * zeros, subnormals, infinities and NaNs, and returns how many results differ
 * (0 expected). */
int ati_check_conversions(int64_t n, int64_t *mismatches);
/* The FP64 fast build's primitives take 1/a and 1/sqrt(a) from hardware
 * approximations refined by two Newton-Raphson steps; this evaluates both on
 * n device-generated positive normal arguments (2^-200..2^200) and returns in
 * worst[0] and worst[1] their largest relative differences from the IEEE
 * division and square root (a few 2^-53 expected). */
int ati_check_recip(int64_t n, double worst[2]);

/* ---- allocation-free derivative (no counterpart in the reference) -------
 * For callers that must not allocate GPU memory when they call in: codes
 * that give all device memory to their own pool at start-up, or time loops
 * that may not allocate once running (an allocation can stall the whole
 * device or fail late).  Computes the compact first derivative of nlines
 * contiguous lines of len points each, in -> out (both caller-owned device
 * arrays, line t at offset t*len), with the one-sided boundary rows at both
 * ends -- the result ati_deriv gives along xi on blocks whose two xi faces
 * have ndf = 0 (boundary codes 10, 20, 25 and 30), bit for bit; faces with
 * codes 35, 40 or 45 (ndf = 1) take closure rows instead and differ --
 * asynchronously on `stream` (a cudaStream_t; NULL = the legacy default
 * stream).
 *  - Allocates and frees nothing.  Its scratch (LU factors and the
 *    forward-elimination values) is one static device array of
 *    5*ATI_NOALLOC_MAX_LEN + ATI_NOALLOC_MAX_POINTS doubles (about 16 MB)
 *    per GPU, held until the process exits.
 *  - The first call on each device (and again after a device reset, which
 *    gives the context a new array) looks up the array's device address with
 *    cudaGetSymbolAddress, that device current.  Under CUDA's default lazy
 *    module loading that look-up is also when the driver loads the module and
 *    reserves the 16 MB, so the first call can fail with ATI_ECUDA on a device
 *    with no room left: make one call (nlines may be 1) before a memory pool
 *    takes the device's memory and before any stream capture, or set
 *    CUDA_MODULE_LOADING=EAGER so that the array is reserved when the context
 *    is created.
 *  - Rejects len outside 7..ATI_NOALLOC_MAX_LEN and nlines*len above
 *    ATI_NOALLOC_MAX_POINTS with ATI_EINVAL (text in ati_last_error(NULL)),
 *    and, without launching anything, a CUDA error already pending from
 *    earlier work with ATI_ECUDA (that error is left pending).
 *  - All calls share the one scratch array and it keeps the previous call's
 *    contents: the LU factors depend only on len and are refactored when len
 *    differs from the previous call's, and every other value a call reads it
 *    wrote itself, so nothing needs clearing.  Calls must therefore be
 *    ordered on the GPU: calls that overlap (different streams, no ordering
 *    between them) race on the array and must not be issued. */
#define ATI_NOALLOC_MAX_POINTS 2000000
#define ATI_NOALLOC_MAX_LEN 4096
int ati_deriv_lines_noalloc(const double *in, double *out, int64_t nlines, int32_t len, void *stream);

/* Lift and drag of the wall blocks as clpost computes them
 * (src/rpt.f90:1017-1056), from the p and stresses of the last stage:
 * out[0] = force coefficient along x, out[1] = along y. */
int ati_forces(ati_handle_t *h, double out[2]);
int ati_case_forces(ati_handle_t *h, int cs, double out[2]);

/* ---- outputs and on-disk formats ---------------------------------------- */
/* The configuration the handle was created with. */
int ati_get_config(ati_handle_t *h, ati_config_t *cfg);
/* Moving-frame velocity umf(1:3) and angle of attack aoa (degrees) of the
 * current time (movef / pitch, src/Subroutineso.f90:192-259). */
int ati_get_frame(ati_handle_t *h, double umf[3], double *aoa);
int ati_case_frame(ati_handle_t *h, int cs, double umf[3], double *aoa);

/* Surface-pressure recorder (no counterpart in the reference, which writes
 * whole fields at intervals): with capacity > 0, every time step ends with one
 * record of the static pressure, from the new qa in FP64, on the mid-span line
 * (k = lze/2, i = 0..lxi) of every wall face (BC 20/25, the order of
 * ati_forces), into a device ring buffer of `capacity` records; capacity 0
 * turns it off.  ati_wall_probe_read copies the last min(steps, capacity)
 * records, oldest first: p[r*npts + i] and the time t[r] of record r; with
 * p == NULL it only returns nrec and npts. */
int ati_wall_probe_enable(ati_handle_t *h, int capacity);
int ati_wall_probe_read(ati_handle_t *h, double *p, double *t, int64_t *nrec, int64_t *npts);

/* Restart file of block blk in the layout of wrRsta (src/rpt.f90:555-621,
 * one block per file, npc = 1): six 8-byte header slots -- n and ndt as int32
 * in the first 4 bytes of their slot, then dt, dts, dte, timo as float64 --
 * followed by qa(0:lmx,1:5) as float64, native byte order. */
int ati_write_restart(ati_handle_t *h, int blk, const char *path);
/* rdRsta (src/rpt.f90:626-668): the header sets the time scalars, the body
 * the state of block blk. */
int ati_read_restart(ati_handle_t *h, int blk, const char *path);
/* Plot3D multi-block files as wrP3dG and wrP3dS write them with mblk = 1
 * (src/rpt.f90:246-330 and 115-241): int32 block count, int32
 * (IMax, JMax, KMax) per block, then per block x, y, z as float32 (grid), or
 * Mach, AoA, Re, time followed by rho, u, v, w, p as float32 (solution; the
 * velocities rho u / rho + umf, p the pressure of the last stage).  A batch
 * writes every block of every case, each with its own case's header values. */
int ati_write_plot3d_grid(ati_handle_t *h, const char *path);
int ati_write_plot3d_solution(ati_handle_t *h, const char *path);

#ifdef __cplusplus
}
#endif
#endif /* ATI_H */
