/*
 * les_ref.h -- C interface of the CPU oracle for the MPI-LES per-timestep solver.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker: a loop-by-loop
 * C++ restatement of the reference's Fortran subroutines (src/velnw.f95,
 * src/bondv1.f95, src/velFG.f95, src/vel2.f95, src/feedbf.f95, src/les.f95,
 * src/boundsm.f95, src/adam.f95, src/press.f95, src/bondFG.f95, src/boundp.f95 and,
 * for the inputs, src/grid.f95, src/init.f95, src/feedbfm.f95, src/set.f95).
 * Only tests, the smoke check and the benchmark's CPU-baseline leg load it; the
 * GPU product never links or calls it.
 *
 * PARITY UNPINNED: the reference is Fortran, this image has no Fortran compiler, and
 * the reference ships no golden vectors for the solver, so the restatement cannot be
 * checked against the reference's own outputs.  It is held to the reference by its
 * loop-by-loop citations, the FP32-vs-FP64 drift bound and equation-derived checks.
 *
 * The oracle is instantiated in FP32 (prec = 4, the reference's real(kind=4)) and
 * in FP64 (prec = 8, the equivalent of compiling the reference with
 * -freal-4-real-8).  Field ids are the same numbers as the LES_FIELD_* ids of the
 * product's C-ABI; a CPU test checks that they agree.
 */
#ifndef LES_REF_H
#define LES_REF_H

#ifdef __cplusplus
extern "C" {
#endif

/* option slots of ref_create's opts[] */
enum {
  REF_OPT_NMAXP = 0,      /* SOR iteration cap (press.f95:44, 50)                     */
  REF_OPT_SOR_FIXED = 1,  /* 1: no early exit on sor < pjuge (press.f95:119)           */
  REF_OPT_RED64 = 2,      /* 1: FP64 accumulation of rhsav/area/sor/pav/pco            */
  REF_OPT_SQRT_HALF = 3,  /* 1: x**0.5 as sqrt (0: powf(x,0.5) as gfortran emits)      */
  REF_OPT_DZ_LAW = 4,     /* 0: grid.f95 piecewise law; 1: geometric dz0*ratio^(k-1)   */
  REF_OPT_COUNT = 5
};

/* constant slots of ref_create's consts[] */
enum {
  REF_C_DT = 0, REF_C_RO, REF_C_VN, REF_C_ALPHA, REF_C_BETA, REF_C_OMEGA, REF_C_PJUGE,
  REF_C_DX, REF_C_DY, REF_C_DZ0, REF_C_DZRATIO, REF_C_COUNT
};

/* stage ids of ref_stage */
enum {
  REF_STEP = 0, REF_VELNW = 1, REF_BONDV1 = 2, REF_VELFG = 3, REF_FEEDBF = 4,
  REF_LES = 5, REF_ADAM = 6, REF_PRESS = 7, REF_BOUNDP1 = 8, REF_BOUNDP2 = 9,
  REF_BONDFG = 10
};

/* zbm: im*jm heights (i fastest); uin/vin/win: jm*km inflow planes (j fastest). */
void *ref_create(int prec, int im, int jm, int km, const double *consts, const int *opts,
                 const float *zbm, const float *uin, const float *vin, const float *win);
void ref_destroy(void *h);
int ref_stage(void *h, int stage, int n, int nmax);
/* aveflow.f95:5-200 at step n with averaging from step n1 to nmax (the time averages,
 * fields 100..110, exist after the first call) */
int ref_aveflow(void *h, int n, int n1, int nmax);
/* copy a field (Fortran extents lb..ub, i fastest) out of / into the oracle */
int ref_get(void *h, int field, double *out, const int *lb, const int *ub);
int ref_set(void *h, int field, const double *in, const int *lb, const int *ub);
/* declared extents of a field in the reference (main.f95:63-159) */
int ref_extents(void *h, int field, int *lb, int *ub);
/* diagnostics of the last step: [iters, sor, uout, rhsav, pav, area, pco] */
void ref_diag(void *h, double *out);
/* 1 if built with array bounds checks (mirrors gfortran -fbounds-check) */
int ref_bounds_checked(void);
const char *ref_last_error(void);
/* The configs' seeded synthetic scenario (heightmap zbm(1:im,1:jm), inflow planes
 * (1:jm,1:km)), restated so that the checker and the CPU baseline need nothing from the
 * product.  fl[10] = {dz0, dz_ratio, coverage, h_min, h_max, u_ref, z_ref, pl_exp,
 * direction_deg, noise}; in[4] = {dz_law, fp_min, fp_max, inflow_law}. */
int ref_scenario(int im, int jm, int km, const float *fl, const int *in, unsigned long long seed, float *zbm,
                 float *uin, float *vin, float *win);
/* threads of the fast build's parallel loops from now on (n > 0), for the calling
 * thread; returns the number its next loops will use (1 in the serial builds) */
int ref_set_threads(int n);
/* on != 0: a later velfg stops with an error (status -3, ref_last_error) where a wall
 * speed is zero, the 0/0 of vel2.f95:138,173, instead of producing its NaN */
int ref_trap_wall(void *h, int on);

#ifdef __cplusplus
}
#endif
#endif
