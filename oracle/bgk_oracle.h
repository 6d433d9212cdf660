/*
 * bgk_oracle.h -- CPU oracle for the BGK2D D2Q9 time step (TEST INFRASTRUCTURE).
 *
 * This library is the checker used by tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py.  It is never linked into, called by, or used as a
 * fallback for the product library (libbgk2d_gb300.so).
 *
 * It restates, in plain C, the reference's serial semantics of
 *   SRC/init.F90, SRC/hencol.F90, SRC/build.bcond.F90, SRC/build.obs.F90,
 *   SRC/bcond.driven.F90, SRC/bcond.periodic.F90, SRC/bcond.channel.F90,
 *   SRC/bcond.inflow.F90, SRC/bcond.couette.F90, SRC/bcond.step.F90,
 *   SRC/bcond.obs.F90, SRC/movef.F90, SRC/col.F90, SRC/col_MC.F90,
 *   SRC/diagno.F90, SRC/draglift.F90, SRC/probe.F90, SRC/prof_j.F90
 * keeping the reference's parenthesisation, mixed-kind promotions and loop order.
 * It must be compiled with -ffp-contract=off (no FMA contraction) so that each
 * Fortran operation is one IEEE operation.
 *
 * Arrays use the reference layout: population q is a column-major array
 * (0:l+1, 0:m+1), i fastest (SRC/alloca.F90:113-121, ipad=jpad=0), and the
 * direction order is 01,03,05,08,10,12,14,17,19 (SRC/bgk2d.F90:29-39).
 */
#ifndef BGK_ORACLE_H
#define BGK_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* precision: SRC/precision.F90:13-47 */
enum { ORC_SINGLE = 0, ORC_DOUBLE = 1, ORC_MIXED2 = 2 };
/* test case (compile-time -D flag in the reference, SRC/Makefile:155-187) */
enum { ORC_LDC = 0, ORC_TGV = 1, ORC_POF = 2, ORC_VKS = 3, ORC_COU = 4, ORC_BFS = 5,
       ORC_MYV = 6 /* -DMYVERSION: periodic boundaries with the CHANNEL volume force
                    * (SRC/boundaries.F90:46-48, SRC/build.bcond.F90:39-41) */ };
/* obstacle shapes: SRC/build.obs.F90 (default circle, SQUARE, HALF_CIRCLE) */
enum { ORC_OBS_NONE = 0, ORC_OBS_CIRCLE = 1, ORC_OBS_SQUARE = 2, ORC_OBS_HALF_CIRCLE = 3 };
/* order of the racy in-place obstacle loop (SRC/bcond.obs.F90:59-71):
 * SERIAL = the serial build's j-outer/i-inner order, SNAPSHOT = every read before any write */
enum { ORC_OBS_SERIAL = 0, ORC_OBS_SNAPSHOT = 1 };

typedef struct orc_state orc_state;

typedef struct {
    int l, m;
    int prec;          /* ORC_SINGLE / ORC_DOUBLE / ORC_MIXED2 */
    int tcase;         /* ORC_LDC ... */
    int fused;         /* 1: col_MC + pointer swap, 0: movef + col */
    int obstacle;      /* ORC_OBS_* shape, 0 = none */
    int obs_order;     /* ORC_OBS_SERIAL / ORC_OBS_SNAPSHOT */
    int radius;        /* namelist radius (SRC/input.F90:61) */
    int obs_icoord;    /* obstacle centre; <0 selects 2*l/5 (SRC/build.obs.F90:174) */
    int obs_jcoord;    /* <0 selects m/2 (SRC/build.obs.F90:175) */
    int init_v;        /* 0 rest flow; TGV cases use the periodic init */
    double svisc;      /* namelist svisc, rounded to mykind */
    double u0;         /* namelist u0, rounded to mykind */
    int les;           /* 1: Smagorinsky eddy viscosity (-DLES, SRC/col_MC.F90:178-264) */
    double cte_s;      /* namelist cteS (SRC/input.F90:55), rounded to mykind */
    int trick1;        /* 1: the merged lid-cavity boundary loop of -DTRICK1 (SRC/bcond.driven.F90:43-81);
                        * LDC on a square box only (SRC/check_case.F90:173-178) */
    int noshift;       /* 1: -DNOSHIFT, the populations f themselves are stored instead of f - w
                        * (cte1/cte0 of SRC/col_MC.F90:70-75, SRC/init.F90:73-77, ...) */
    int force_y;       /* 1: -DFORCING_Y, the volume force of CHANNEL / MYVERSION acts along y
                        * (forcey = fgrad*rho, SRC/col_MC.F90:268-282, SRC/col.F90:212-226) */
} orc_params;

orc_state *orc_create(const orc_params *p);
void orc_destroy(orc_state *s);
/* one full time step = boundaries + propagation + collision (SRC/bgk2d.F90:100-102) */
void orc_step(orc_state *s, int nsteps);
/* same step, OpenMP-parallel over rows (fused col_MC only); used as the timed CPU baseline */
void orc_step_omp(orc_state *s, int nsteps, int nthreads);

/* populations of the current "a" arrays, (l+2)*(m+2) doubles per direction, 9 directions */
void orc_get_pops(const orc_state *s, double *out);
void orc_set_pops(orc_state *s, const double *in);
/* raw storage bytes of the current "a" arrays (float or double, 9 planes back to back) */
void orc_get_raw(const orc_state *s, void *out);
void orc_set_raw(orc_state *s, const void *in);
int  orc_storage_bytes(const orc_state *s);

/* obstacle mask obs(1:l,1:m) (column-major, i fastest) and bbox/nobs */
void orc_get_obs(const orc_state *s, int32_t *mask, int32_t bbox[5]);
/* standalone mask builder, same arithmetic as build_obs; bbox = imin,imax,jmin,jmax,nobs */
void orc_build_obs(int l, int m, int shape, int radius, int icoord, int jcoord, int prec,
                   int32_t *mask, int32_t bbox[5]);

/* scalars set up by hencol/build_bcond, returned in double */
void orc_get_scalars(const orc_state *s, double out[4]); /* omega, fgrad, u00, u0 */

/* diagnostics.  mode 0: reference diagno (mykind, sequential j/i order);
 * mode 1: same per-cell arithmetic, FP64 accumulation; mode 2: FP64, fluid cells only */
void orc_diagno(const orc_state *s, int mode, double out[4]);  /* <u>,<v>,<rho>,<|u|^2> */
/* drag/lift (SRC/draglift.F90); mode 0 mykind sums, 1 FP64 sums; out = Fx*norm, Fy*norm */
void orc_draglift(const orc_state *s, int mode, double out[2]);
/* centre-line profile at column icoord (SRC/prof_j.F90:47-67), m values each */
void orc_prof_j(const orc_state *s, int icoord, double *u, double *v, double *den);
/* macroscopic fields over the interior, l*m each, i fastest (diagno's per-cell arithmetic) */
void orc_fields(const orc_state *s, double *rho, double *u, double *v);
/* the VTK writers' single-precision fields (SRC/vtk_xy.binary.F90, SRC/vtk_om.binary.F90): u, w,
 * rho over 1..l x 1..m (l*m each); vorticity and stream function over 2..l-1 x 2..m-1
 * ((l-2)*(m-2) each); i fastest.  from_ghost_row = 1 integrates the stream function from ghost
 * row 0 as the reference does, 0 from row 1 */
void orc_vtk(const orc_state *s, int from_ghost_row, float *u, float *w, float *rho, float *vort, float *stream);

#ifdef __cplusplus
}
#endif
#endif
