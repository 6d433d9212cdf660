/*
 * bgk_oracle.c -- CPU oracle for the BGK2D D2Q9 time step (TEST INFRASTRUCTURE ONLY).
 *
 * Used by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / --impl reference
 * leg as the checker and the timed CPU baseline.  The product library never links it.
 * See bgk_oracle.h for the list of reference routines restated here.
 *
 * Build: gcc -O3 -fPIC -shared -fopenmp -ffp-contract=off -fno-fast-math (oracle/Makefile).
 */
#include "bgk_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>

#if defined(__FAST_MATH__)
#error "the oracle must be built without -ffast-math"
#endif

struct orc_state {
    orc_params p;
    int l, m, ld;
    size_t n;           /* (l+2)*(m+2) elements per plane */
    int ssize;          /* bytes per stored element */
    void *A[9];         /* current populations a01..a19 */
    void *B[9];         /* second buffer b01..b19 */
    int32_t *obs;       /* obs(1:l,1:m), i fastest */
    int imin, imax, jmin, jmax, nobs;
    int icoord, jcoord;
    int stepx, stepy;   /* input.F90:74-75 */
    double omega, fgrad, u00, u0;  /* mykind values, stored exactly in double */
};

/* SINGLE: mystorage = mykind = REAL(4) */
#define S float
#define K float
#define FN(x) x##_ss
#define SIN sinf
#define SQRT sqrtf
#define COS cosf
#include "bgk_oracle_body.h"
#undef S
#undef K
#undef FN
#undef SIN
#undef SQRT
#undef COS

/* DOUBLE: mystorage = mykind = REAL(8) */
#define S double
#define K double
#define FN(x) x##_dd
#define SIN sin
#define SQRT sqrt
#define COS cos
#include "bgk_oracle_body.h"
#undef S
#undef K
#undef FN
#undef SIN
#undef SQRT
#undef COS

/* MIXED2: mystorage = REAL(4), mykind = REAL(8) */
#define S float
#define K double
#define FN(x) x##_sd
#define SIN sin
#define SQRT sqrt
#define COS cos
#include "bgk_oracle_body.h"
#undef S
#undef K
#undef FN
#undef SIN
#undef SQRT
#undef COS

#define DISPATCH(s, fn, args)                              \
    do {                                                   \
        switch ((s)->p.prec) {                             \
        case ORC_DOUBLE: fn##_dd args; break;              \
        case ORC_MIXED2: fn##_sd args; break;              \
        default: fn##_ss args; break;                      \
        }                                                  \
    } while (0)

orc_state *orc_create(const orc_params *p)
{
    if (p->l < 2 || p->m < 2) return NULL;
    if (p->trick1 && (p->tcase != ORC_LDC || p->l != p->m)) return NULL;
    orc_state *s = (orc_state *)calloc(1, sizeof(orc_state));
    s->p = *p;
    s->l = p->l; s->m = p->m; s->ld = p->l + 2;
    s->n = (size_t)(p->l + 2) * (size_t)(p->m + 2);
    s->ssize = (p->prec == ORC_DOUBLE) ? 8 : 4;
    s->stepy = p->m / 2;
    s->stepx = p->l / 20;
    for (int q = 0; q < 9; ++q) {
        s->A[q] = malloc(s->n * (size_t)s->ssize);
        s->B[q] = malloc(s->n * (size_t)s->ssize);
        /* alloca.F90:133-151 poisons every array with huge(mykind) */
        for (size_t k = 0; k < s->n; ++k) {
            if (s->ssize == 8) { ((double *)s->A[q])[k] = DBL_MAX; ((double *)s->B[q])[k] = DBL_MAX; }
            else { ((float *)s->A[q])[k] = FLT_MAX; ((float *)s->B[q])[k] = FLT_MAX; }
        }
    }
    s->obs = (int32_t *)calloc((size_t)p->l * (size_t)p->m, sizeof(int32_t));
    s->icoord = p->obs_icoord >= 0 ? p->obs_icoord : 2 * p->l / 5;
    s->jcoord = p->obs_jcoord >= 0 ? p->obs_jcoord : p->m / 2;
    s->imin = p->l; s->jmin = p->m; s->imax = 0; s->jmax = 0; s->nobs = 0;
    if (p->obstacle) {
        int32_t bb[5];
        orc_build_obs(p->l, p->m, p->obstacle, p->radius, s->icoord, s->jcoord, p->prec, s->obs, bb);
        s->imin = bb[0]; s->imax = bb[1]; s->jmin = bb[2]; s->jmax = bb[3]; s->nobs = bb[4];
    }
    DISPATCH(s, setup_scalars, (s));
    DISPATCH(s, init, (s));
    return s;
}

void orc_destroy(orc_state *s)
{
    if (!s) return;
    for (int q = 0; q < 9; ++q) { free(s->A[q]); free(s->B[q]); }
    free(s->obs);
    free(s);
}

void orc_build_obs(int l, int m, int shape, int radius, int icoord, int jcoord, int prec,
                   int32_t *mask, int32_t bbox[5])
{
    if (prec == ORC_SINGLE) build_obs_ss(l, m, shape, radius, icoord, jcoord, mask, bbox);
    else build_obs_dd(l, m, shape, radius, icoord, jcoord, mask, bbox);
}

void orc_step(orc_state *s, int nsteps) { DISPATCH(s, step, (s, nsteps, 1)); }

void orc_step_omp(orc_state *s, int nsteps, int nthreads) { DISPATCH(s, step, (s, nsteps, nthreads)); }

void orc_get_pops(const orc_state *s, double *out) { DISPATCH(s, get_pops, (s, out)); }
void orc_set_pops(orc_state *s, const double *in) { DISPATCH(s, set_pops, (s, in)); }

int orc_storage_bytes(const orc_state *s) { return s->ssize; }

void orc_get_raw(const orc_state *s, void *out)
{
    size_t pb = s->n * (size_t)s->ssize;
    for (int q = 0; q < 9; ++q) memcpy((char *)out + (size_t)q * pb, s->A[q], pb);
}

void orc_set_raw(orc_state *s, const void *in)
{
    size_t pb = s->n * (size_t)s->ssize;
    for (int q = 0; q < 9; ++q) memcpy(s->A[q], (const char *)in + (size_t)q * pb, pb);
}

void orc_get_obs(const orc_state *s, int32_t *mask, int32_t bbox[5])
{
    if (mask) memcpy(mask, s->obs, sizeof(int32_t) * (size_t)s->l * (size_t)s->m);
    bbox[0] = s->imin; bbox[1] = s->imax; bbox[2] = s->jmin; bbox[3] = s->jmax; bbox[4] = s->nobs;
}

void orc_get_scalars(const orc_state *s, double out[4])
{
    out[0] = s->omega; out[1] = s->fgrad; out[2] = s->u00; out[3] = s->u0;
}

void orc_diagno(const orc_state *s, int mode, double out[4]) { DISPATCH(s, diagno, (s, mode, out)); }
void orc_draglift(const orc_state *s, int mode, double out[2]) { DISPATCH(s, draglift, (s, mode, out)); }
void orc_prof_j(const orc_state *s, int icoord, double *u, double *v, double *den)
{
    DISPATCH(s, prof_j, (s, icoord, u, v, den));
}
void orc_fields(const orc_state *s, double *rho, double *u, double *v) { DISPATCH(s, fields, (s, rho, u, v)); }
void orc_vtk(const orc_state *s, int from_ghost_row, float *u, float *w, float *rho, float *vort, float *stream)
{
    DISPATCH(s, vtk, (s, from_ghost_row, u, w, rho, vort, stream));
}
