/*
 * bgk_oracle_body.h -- precision-generic body of the CPU oracle (TEST INFRASTRUCTURE).
 *
 * Included three times by bgk_oracle.c with
 *   S  = storage kind (the reference's `mystorage`),
 *   K  = compute kind (the reference's `mykind`),
 *   FN(x) = x##_<suffix>,
 *   SIN/COS = the libm functions of kind K.
 * Every expression keeps the reference's parenthesisation; where a Fortran expression
 * mixes kinds (e.g. a `3.d0` literal in a single-precision build) the promotion to
 * double is written out explicitly.
 */

#define A_(q, i, j) (((S *)s->A[q])[(size_t)(i) + (size_t)(j) * (size_t)s->ld])
#define B_(q, i, j) (((S *)s->B[q])[(size_t)(i) + (size_t)(j) * (size_t)s->ld])
#define RA(q, i, j) ((K)A_(q, i, j))
#define RB(q, i, j) ((K)B_(q, i, j))

/* storage.F90:130-138 -- constants cast to mykind */
#define UNO ((K)1)
#define ZERO ((K)0)
#define TRE ((K)3)
#define RF ((K)3)
#define QF ((K)1.5)
#define P0 ((K)(4.0 / 9.0))
#define P1 ((K)(1.0 / 9.0))
#define P2 ((K)(1.0 / 36.0))

/* init.F90:33-137 (cte1 = 0, or 1 under NOSHIFT: init.F90:73-77; rest flow, or the periodic
 * vortex under PERIODIC) */
static void FN(init)(orc_state *s)
{
    const int l = s->l, m = s->m;
    /* parameter(pi=3.1415...) is a default-real literal: it is rounded to REAL(4) */
    const K pi = (K)3.14159265358979323846f;
    const K crho = (K)1;
    const K cte1 = s->p.noshift ? UNO : ZERO;
    K xj = (K)0, yj = (K)0;
    for (int j = 0; j <= m + 1; ++j) {
        K y = (K)(((double)(K)j - 0.5) / (double)(K)m);
        for (int i = 0; i <= l + 1; ++i) {
            if (s->p.tcase == ORC_TGV) {
                K x = (K)(((double)(K)i - 0.5) / (double)(K)l);
                xj = (K)((0.1 * (double)SIN((K)2 * pi * x)) * (double)COS((K)2 * pi * y));
                yj = (K)(-((0.1 * (double)COS((K)2 * pi * x)) * (double)SIN((K)2 * pi * y)));
            }
            K cvsq = xj * xj + yj * yj;
            double dc = (double)cvsq;
            K cx01 = (K)((double)(RF * (xj - yj)) + (double)QF * ((3.0 * (double)(xj - yj)) * (double)(xj - yj) - dc));
            K cx03 = (K)((double)(RF * (xj + yj)) + (double)QF * ((3.0 * (double)(xj + yj)) * (double)(xj + yj) - dc));
            K cx05 = (K)((double)(RF * (xj)) + (double)QF * ((3.0 * (double)(xj)) * (double)(xj) - dc));
            K cx08 = (K)((double)(RF * (yj)) + (double)QF * ((3.0 * (double)(yj)) * (double)(yj) - dc));
            K cx10 = (K)((double)(RF * (-xj - yj)) + (double)QF * ((3.0 * (double)(xj + yj)) * (double)(xj + yj) - dc));
            K cx12 = (K)((double)(RF * (-xj + yj)) + (double)QF * ((3.0 * (double)(xj - yj)) * (double)(xj - yj) - dc));
            K cx14 = (K)((double)(RF * (-xj)) + (double)QF * ((3.0 * (double)(xj)) * (double)(xj) - dc));
            K cx17 = (K)((double)(RF * (-yj)) + (double)QF * ((3.0 * (double)(yj)) * (double)(yj) - dc));
            K cx19 = (K)((double)RF * 0.0 + (double)QF * ((3.0 * 0.0) * 0.0 - dc));
            A_(0, i, j) = (S)((crho * P2) * (cte1 + cx01));
            A_(1, i, j) = (S)((crho * P2) * (cte1 + cx03));
            A_(2, i, j) = (S)((crho * P1) * (cte1 + cx05));
            A_(3, i, j) = (S)((crho * P1) * (cte1 + cx08));
            A_(4, i, j) = (S)((crho * P2) * (cte1 + cx10));
            A_(5, i, j) = (S)((crho * P2) * (cte1 + cx12));
            A_(6, i, j) = (S)((crho * P1) * (cte1 + cx14));
            A_(7, i, j) = (S)((crho * P1) * (cte1 + cx17));
            A_(8, i, j) = (S)((crho * P0) * (cte1 + cx19));
        }
    }
}

/* build.bcond.F90:47-56 and hencol.F90:30-50 */
static void FN(setup_scalars)(orc_state *s)
{
    K u0 = (K)s->p.u0;
    K svisc = (K)s->p.svisc;
    K u00;
    if (s->p.tcase == ORC_POF || s->p.tcase == ORC_MYV) { u00 = (K)0; }  /* CHANNEL, MYVERSION: volume force */
    else { u00 = u0; u0 = (K)0; }                     /* wall-driven */
    K omega = (UNO + UNO) / (((K)6 * svisc) + (K)1);
    K fgrad = (((K)4 * u0) * svisc) / (((K)3 * (K)s->m) * (K)s->m);
    s->omega = (double)omega;
    s->fgrad = (double)fgrad;
    s->u00 = (double)u00;
    s->u0 = (double)u0;
}

/* build.obs.F90:38-205 (circle by default, SQUARE, HALF_CIRCLE); d2 and R are mykind.  Inline:
 * not every precision instance calls it. */
static inline void FN(build_obs)(int l, int m, int shape, int radius, int icoord, int jcoord,
                                 int32_t *obs, int32_t *bbox)
{
    int imin = l, jmin = m, imax = 0, jmax = 0, nobs = 0;
    for (size_t k = 0; k < (size_t)l * (size_t)m; ++k) obs[k] = 0;
#define OBS_SET(i, j)                                                    \
    do {                                                                 \
        obs[(size_t)((i) - 1) + (size_t)((j) - 1) * (size_t)l] = 1;     \
        nobs += 1;                                                       \
        if ((i) < imin) imin = (i);                                      \
        if ((j) < jmin) jmin = (j);                                      \
        if ((i) > imax) imax = (i);                                      \
        if ((j) > jmax) jmax = (j);                                      \
    } while (0)
    if (shape == ORC_OBS_SQUARE) {
        K hsize = (K)radius;
        for (int j = 1; j <= m; ++j) {
            if (((K)j >= ((K)jcoord - hsize)) && ((K)j <= ((K)jcoord + hsize))) {
                for (int i = 1; i <= l; ++i) {
                    if (((K)i >= ((K)icoord - hsize)) && ((K)i <= ((K)icoord + hsize))) OBS_SET(i, j);
                }
            }
        }
    } else if (shape == ORC_OBS_CIRCLE || shape == ORC_OBS_HALF_CIRCLE) {
        K R = (K)radius * UNO;
        int j0 = (shape == ORC_OBS_HALF_CIRCLE) ? m / 2 : 1;
        for (int j = j0; j <= m; ++j) {
            for (int i = 1; i <= l; ++i) {
                K d2 = (K)((icoord - i) * (icoord - i) + (jcoord - j) * (jcoord - j));
                if (d2 <= R * R) OBS_SET(i, j);
            }
        }
    }
#undef OBS_SET
    bbox[0] = imin; bbox[1] = imax; bbox[2] = jmin; bbox[3] = jmax; bbox[4] = nobs;
}

/* bcond.driven.F90:85-153 (default, TRICK1 off): x-walls first, then y-walls with the lid */
static void FN(bcond_driven)(orc_state *s)
{
    const int l = s->l, m = s->m, l1 = l + 1, m1 = m + 1;
    const K force = (K)s->u00 / (K)6.0;
    for (int j = 1; j <= m; ++j) {
        A_(5, l1, j - 1) = A_(0, l, j);   /* a12(l1,j-1) = a01(l,j) */
        A_(4, l1, j + 1) = A_(1, l, j);   /* a10(l1,j+1) = a03(l,j) */
        A_(6, l1, j) = A_(2, l, j);       /* a14(l1,j)   = a05(l,j) */
        A_(1, 0, j - 1) = A_(4, 1, j);    /* a03(0,j-1)  = a10(1,j) */
        A_(0, 0, j + 1) = A_(5, 1, j);    /* a01(0,j+1)  = a12(1,j) */
        A_(2, 0, j) = A_(6, 1, j);        /* a05(0,j)    = a14(1,j) */
    }
    for (int i = 1; i <= l; ++i) {
        A_(3, i, 0) = A_(7, i, 1);                       /* a08(i,0)    = a17(i,1) */
        A_(5, i + 1, 0) = A_(0, i, 1);                   /* a12(i+1,0)  = a01(i,1) */
        A_(1, i - 1, 0) = A_(4, i, 1);                   /* a03(i-1,0)  = a10(i,1) */
        A_(4, i + 1, m1) = (S)(RA(1, i, m) - force);     /* a10(i+1,m1) = a03(i,m) - force */
        A_(7, i, m1) = A_(3, i, m);                      /* a17(i,m1)   = a08(i,m) */
        A_(0, i - 1, m1) = (S)(RA(5, i, m) + force);     /* a01(i-1,m1) = a12(i,m) + force */
    }
}

/* bcond.driven.F90:43-81 (-DTRICK1, square box): one loop over j = 1..m that writes, in this
 * order, the lid (y = m), the x = l wall, the x = 0 wall and the y = 0 wall of index j.  In the
 * serial order the x-wall statements of j = m overwrite the lid's two upper corner ghosts, so
 * a01(0,m1) and a10(l1,m1) carry no lid term; every other ghost equals the default order's. */
static void FN(bcond_driven_trick1)(orc_state *s)
{
    const int l = s->l, m = s->m, l1 = l + 1, m1 = m + 1;
    const K force = (K)s->u00 / (K)6.0;
    for (int j = 1; j <= m; ++j) {
        A_(0, j - 1, m1) = (S)(RA(5, j, m) + force);     /* a01(j-1,m1) = a12(j,m) + force */
        A_(7, j, m1) = A_(3, j, m);                      /* a17(j,m1)   = a08(j,m) */
        A_(4, j + 1, m1) = (S)(RA(1, j, m) - force);     /* a10(j+1,m1) = a03(j,m) - force */
        A_(5, l1, j - 1) = A_(0, l, j);                  /* a12(l1,j-1) = a01(l,j) */
        A_(4, l1, j + 1) = A_(1, l, j);                  /* a10(l1,j+1) = a03(l,j) */
        A_(6, l1, j) = A_(2, l, j);                      /* a14(l1,j)   = a05(l,j) */
        A_(1, 0, j - 1) = A_(4, 1, j);                   /* a03(0,j-1)  = a10(1,j) */
        A_(0, 0, j + 1) = A_(5, 1, j);                   /* a01(0,j+1)  = a12(1,j) */
        A_(2, 0, j) = A_(6, 1, j);                       /* a05(0,j)    = a14(1,j) */
        A_(1, j - 1, 0) = A_(4, j, 1);                   /* a03(j-1,0)  = a10(j,1) */
        A_(3, j, 0) = A_(7, j, 1);                       /* a08(j,0)    = a17(j,1) */
        A_(5, j + 1, 0) = A_(0, j, 1);                   /* a12(j+1,0)  = a01(j,1) */
    }
}

/* bcond.periodic.F90:45-114 */
static void FN(bcond_periodic)(orc_state *s)
{
    const int l = s->l, m = s->m, l1 = l + 1, m1 = m + 1;
    for (int j = 0; j <= m + 1; ++j) {
        A_(0, 0, j) = A_(0, l, j);
        A_(1, 0, j) = A_(1, l, j);
        A_(2, 0, j) = A_(2, l, j);
        A_(4, l1, j) = A_(4, 1, j);
        A_(5, l1, j) = A_(5, 1, j);
        A_(6, l1, j) = A_(6, 1, j);
    }
    for (int i = 0; i <= l + 1; ++i) {
        A_(7, i, m1) = A_(7, i, 1);
        A_(0, i, m1) = A_(0, i, 1);
        A_(4, i, m1) = A_(4, i, 1);
        A_(1, i, 0) = A_(1, i, m);
        A_(3, i, 0) = A_(3, i, m);
        A_(5, i, 0) = A_(5, i, m);
    }
}

/* bcond.channel.F90:56-133: periodic x, no-slip walls in y */
static void FN(bcond_channel)(orc_state *s)
{
    const int l = s->l, m = s->m, l1 = l + 1, m1 = m + 1;
    for (int j = 0; j <= m + 1; ++j) {
        A_(4, l1, j) = A_(4, 1, j);
        A_(5, l1, j) = A_(5, 1, j);
        A_(6, l1, j) = A_(6, 1, j);
        A_(0, 0, j) = A_(0, l, j);
        A_(1, 0, j) = A_(1, l, j);
        A_(2, 0, j) = A_(2, l, j);
    }
    for (int i = 0; i <= l + 1; ++i) {
        A_(3, i, 0) = A_(7, i, 1);
        if (i + 1 <= l + 1) A_(5, i + 1, 0) = A_(0, i, 1);
        if (i - 1 >= 0) A_(1, i - 1, 0) = A_(4, i, 1);
        if (i + 1 <= l + 1) A_(4, i + 1, m1) = A_(1, i, m);
        A_(7, i, m1) = A_(3, i, m);
        if (i - 1 >= 0) A_(0, i - 1, m1) = A_(5, i, m);
    }
}

/* outflow equilibrium shared by bcond.inflow.F90:80-99 and bcond.step.F90:82-101 */
static void FN(outflow_col)(orc_state *s, int j)
{
    const int l = s->l, l1 = l + 1;
    const K crho = UNO, rhoinv = UNO, cte1 = s->p.noshift ? UNO : ZERO;  /* bcond.inflow.F90:48-52 */
    K xj = (((RA(1, l, j) - RA(5, l, j)) + (RA(0, l, j) - RA(4, l, j))) + (RA(2, l, j) - RA(6, l, j))) * rhoinv;
    K yj = (((RA(1, l, j) - RA(0, l, j)) + (RA(5, l, j) - RA(4, l, j))) + (RA(3, l, j) - RA(7, l, j))) * rhoinv;
    K cvsq = xj * xj + yj * yj;
    K cx10 = RF * (-xj - yj) + QF * (((K)3.0 * (xj + yj)) * (xj + yj) - cvsq);
    K cx12 = RF * (-xj + yj) + QF * (((K)3.0 * (xj - yj)) * (xj - yj) - cvsq);
    K cx14 = RF * (-xj) + QF * (((K)3.0 * (xj)) * (xj) - cvsq);
    A_(4, l1, j) = (S)((crho * P2) * (cte1 + cx10));
    A_(5, l1, j) = (S)((crho * P2) * (cte1 + cx12));
    A_(6, l1, j) = (S)((crho * P1) * (cte1 + cx14));
}

/* inflow equilibrium at velocity (xj, 0): bcond.inflow.F90:101-113, bcond.step.F90:135-150 */
static void FN(inflow_cell)(orc_state *s, int j, K xj)
{
    const K crho = UNO, cte1 = s->p.noshift ? UNO : ZERO;
    K yj = ZERO;
    K cvsq = xj * xj + yj * yj;
    double dc = (double)cvsq;
    K cx01 = (K)((double)(RF * (xj - yj)) + (double)QF * ((3.0 * (double)(xj - yj)) * (double)(xj - yj) - dc));
    K cx03 = (K)((double)(RF * (xj + yj)) + (double)QF * ((3.0 * (double)(xj + yj)) * (double)(xj + yj) - dc));
    K cx05 = (K)((double)(RF * (xj)) + (double)QF * ((3.0 * (double)(xj)) * (double)(xj) - dc));
    A_(0, 0, j) = (S)((crho * P2) * (cte1 + cx01));
    A_(1, 0, j) = (S)((crho * P2) * (cte1 + cx03));
    A_(2, 0, j) = (S)((crho * P1) * (cte1 + cx05));
}

/* bcond.inflow.F90:59-154: outflow (x=l+1), inflow u=0.1 (x=0), periodic y */
static void FN(bcond_inflow)(orc_state *s)
{
    const int l = s->l, m = s->m, m1 = m + 1;
    const K u_inflow = (K)0.1f;   /* u_inflow=0.1 is a default-real literal */
    for (int j = 0; j <= m + 1; ++j) {
        FN(outflow_col)(s, j);
        FN(inflow_cell)(s, j, u_inflow);
    }
    for (int i = 0; i <= l + 1; ++i) {
        A_(7, i, m1) = A_(7, i, 1);
        A_(0, i, m1) = A_(0, i, 1);
        A_(4, i, m1) = A_(4, i, 1);
        A_(1, i, 0) = A_(1, i, m);
        A_(3, i, 0) = A_(3, i, m);
        A_(5, i, 0) = A_(5, i, m);
    }
}

/* bcond.couette.F90:41-104: periodic x (j=1..m), wall y=0, moving wall y=m+1 */
static void FN(bcond_couette)(orc_state *s)
{
    const int l = s->l, m = s->m, l1 = l + 1, m1 = m + 1;
    const K force = (K)s->u00 / (K)6.0;
    for (int j = 1; j <= m; ++j) {
        A_(0, 0, j) = A_(0, l, j);
        A_(1, 0, j) = A_(1, l, j);
        A_(2, 0, j) = A_(2, l, j);
        A_(4, l1, j) = A_(4, 1, j);
        A_(5, l1, j) = A_(5, 1, j);
        A_(6, l1, j) = A_(6, 1, j);
    }
    for (int i = 1; i <= l; ++i) {
        A_(3, i, 0) = A_(7, i, 1);
        A_(5, i + 1, 0) = A_(0, i, 1);
        A_(1, i - 1, 0) = A_(4, i, 1);
        A_(4, i + 1, m1) = (S)(RA(1, i, m) - force);
        A_(7, i, m1) = A_(3, i, m);
        A_(0, i - 1, m1) = (S)(RA(5, i, m) + force);
    }
}

/* bcond.step.F90:55-255 (serial build: the wall loop runs i=1..l) */
static void FN(bcond_step)(orc_state *s)
{
    const int l = s->l, m = s->m, m1 = m + 1;
    const int stepx = s->stepx, stepy = s->stepy;
    const K u_inflow = (K)0.1f;
    for (int j = 0; j <= m + 1; ++j) FN(outflow_col)(s, j);
    for (int j = stepy; j <= m + 1; ++j) {
        /* xj = u_inflow*float(j-stepy)*float(m-j)/float((m-stepy)*(m-stepy)/4) */
        K xj = ((u_inflow * (K)(float)(j - stepy)) * (K)(float)(m - j)) /
               (K)(float)(((m - stepy) * (m - stepy)) / 4);
        FN(inflow_cell)(s, j, xj);
    }
    for (int i = 1; i <= l; ++i) {
        A_(3, i, 0) = A_(7, i, 1);
        A_(5, i + 1, 0) = A_(0, i, 1);
        A_(1, i - 1, 0) = A_(4, i, 1);
        A_(4, i + 1, m1) = A_(1, i, m);
        A_(7, i, m1) = A_(3, i, m);
        A_(0, i - 1, m1) = A_(5, i, m);
    }
    for (int i = 1; i <= stepx; ++i) {
        A_(3, i, stepy - 1) = A_(7, i, stepy);
        A_(5, i + 1, stepy - 1) = A_(0, i, stepy);
        A_(1, i - 1, stepy - 1) = A_(4, i, stepy);
    }
    for (int j = 1; j <= stepy; ++j) {
        A_(1, stepx - 1, j - 1) = A_(4, stepx, j);
        A_(0, stepx - 1, j + 1) = A_(5, stepx, j);
        A_(2, stepx - 1, j) = A_(6, stepx, j);
    }
}

/* bcond.obs.F90:59-71: obstacle cells take the opposite population of their neighbour */
static void FN(bcond_obs)(orc_state *s)
{
    const int l = s->l;
    if (s->nobs <= 0) return;
    if (s->p.obs_order == ORC_OBS_SERIAL) {
        for (int j = s->jmin; j <= s->jmax; ++j) {
            for (int i = s->imin; i <= s->imax; ++i) {
                if (s->obs[(size_t)(i - 1) + (size_t)(j - 1) * (size_t)l] == 1) {
                    A_(0, i, j) = A_(5, i + 1, j - 1);
                    A_(1, i, j) = A_(4, i + 1, j + 1);
                    A_(2, i, j) = A_(6, i + 1, j);
                    A_(3, i, j) = A_(7, i, j + 1);
                    A_(4, i, j) = A_(1, i - 1, j - 1);
                    A_(5, i, j) = A_(0, i - 1, j + 1);
                    A_(6, i, j) = A_(2, i - 1, j);
                    A_(7, i, j) = A_(3, i, j - 1);
                }
            }
        }
    } else {
        /* all reads from a snapshot taken before any write */
        const int ni = s->imax - s->imin + 1, nj = s->jmax - s->jmin + 1;
        S *tmp = (S *)malloc(sizeof(S) * 8 * (size_t)ni * (size_t)nj);
        for (int j = s->jmin; j <= s->jmax; ++j) {
            for (int i = s->imin; i <= s->imax; ++i) {
                S *t = tmp + 8 * ((size_t)(i - s->imin) + (size_t)(j - s->jmin) * (size_t)ni);
                t[0] = A_(5, i + 1, j - 1); t[1] = A_(4, i + 1, j + 1);
                t[2] = A_(6, i + 1, j);     t[3] = A_(7, i, j + 1);
                t[4] = A_(1, i - 1, j - 1); t[5] = A_(0, i - 1, j + 1);
                t[6] = A_(2, i - 1, j);     t[7] = A_(3, i, j - 1);
            }
        }
        for (int j = s->jmin; j <= s->jmax; ++j) {
            for (int i = s->imin; i <= s->imax; ++i) {
                if (s->obs[(size_t)(i - 1) + (size_t)(j - 1) * (size_t)l] == 1) {
                    S *t = tmp + 8 * ((size_t)(i - s->imin) + (size_t)(j - s->jmin) * (size_t)ni);
                    for (int q = 0; q < 8; ++q) A_(q, i, j) = t[q];
                }
            }
        }
        free(tmp);
    }
}

/* boundaries.F90:31-56 */
static void FN(boundaries)(orc_state *s)
{
    switch (s->p.tcase) {
    case ORC_TGV: case ORC_MYV: FN(bcond_periodic)(s); break;
    case ORC_POF: FN(bcond_channel)(s); break;
    case ORC_VKS: FN(bcond_inflow)(s); break;
    case ORC_COU: FN(bcond_couette)(s); break;
    case ORC_BFS: FN(bcond_step)(s); break;
    default: if (s->p.trick1) FN(bcond_driven_trick1)(s); else FN(bcond_driven)(s); break;
    }
    if (s->p.obstacle) FN(bcond_obs)(s);
}

/* col_MC.F90:114-176 / col.F90:90-152 (equilibrium) and :285-293 / :229-237 (relaxation);
 * x[] holds x01..x19, out[] receives the nine post-collision values in mykind.  cte1 = 1, or 0
 * under NOSHIFT (col_MC.F90:70-75, col.F90:61-66), and cte0 = 1 - cte1 */
static inline void FN(collide)(const K *x, K omega, K fgrad, int forced, int les, K cte_s, int noshift, K *out)
{
    const K cte1 = noshift ? ZERO : UNO, cte0 = UNO - cte1;
    K x01 = x[0], x03 = x[1], x05 = x[2], x08 = x[3], x10 = x[4];
    K x12 = x[5], x14 = x[6], x17 = x[7], x19 = x[8];
    K rho = ((((x01 + x03) + x10) + x12) + (((x05 + x08) + x14) + x17) + x19) + cte1;
    K rhoinv = UNO / rho;
    K vx = (((x03 - x12) + (x01 - x10)) + (x05 - x14)) * rhoinv;
    K vy = (((x03 - x01) + (x12 - x10)) + (x08 - x17)) * rhoinv;
    K vx2 = vx * vx;
    K vy2 = vy * vy;
    K vsq = vx2 + vy2;
    K vxpy = vx + vy;
    K vxmy = vx - vy;
    K qxpy = cte0 + QF * ((TRE * vxpy) * vxpy - vsq);
    K qxmy = cte0 + QF * ((TRE * vxmy) * vxmy - vsq);
    K qx = cte0 + QF * (TRE * vx2 - vsq);
    K qy = cte0 + QF * (TRE * vy2 - vsq);
    K q0 = cte0 + QF * (-vsq);
    vx = RF * vx;
    vy = RF * vy;
    vxpy = RF * vxpy;
    vxmy = RF * vxmy;
    K rp0 = rho * P0;
    K rp1 = rho * P1;
    K rp2 = rho * P2;
    K e01 = rp2 * (+vxmy + qxmy) + cte1 * (rp2 - P2);
    K e03 = rp2 * (+vxpy + qxpy) + cte1 * (rp2 - P2);
    K e05 = rp1 * (+vx + qx) + cte1 * (rp1 - P1);
    K e08 = rp1 * (+vy + qy) + cte1 * (rp1 - P1);
    K e10 = rp2 * (-vxpy + qxpy) + cte1 * (rp2 - P2);
    K e12 = rp2 * (-vxmy + qxmy) + cte1 * (rp2 - P2);
    K e14 = rp1 * (-vx + qx) + cte1 * (rp1 - P1);
    K e17 = rp1 * (-vy + qy) + cte1 * (rp1 - P1);
    K e19 = rp0 * (+q0) + cte1 * (rp0 - P0);
    if (les) {
        /* col_MC.F90:178-248: non-equilibrium stress, then omega = 1/Ts with the Smagorinsky
         * eddy viscosity; omega1 is the molecular rate (hencol.F90:31, equal to omega).
         * `18.0` and `1.0` are default-real literals, exact in either kind. */
        const K omega1 = omega;
        K n01 = x01 - e01, n03 = x03 - e03, n05 = x05 - e05, n08 = x08 - e08;
        K n10 = x10 - e10, n12 = x12 - e12, n14 = x14 - e14, n17 = x17 - e17;
        K pxx = ((((n01 + n03) + n05) + n10) + n12) + n14;
        K pyy = ((((n01 + n03) + n08) + n10) + n12) + n17;
        K pxy = (((-n01) + n03) + n10) - n12;
        K pyx = pxy;
        K ptotal = SQRT(((pxx * pxx) + (((K)2 * pxy) * pyx)) + (pyy * pyy));
        K r = UNO / omega1;
        K ts = UNO / ((K)2 * omega1) + SQRT((((K)18 * (cte_s * cte_s)) * ptotal) + (r * r)) / (K)2;
        omega = UNO / ts;
    }
    K forcex = ZERO, forcey = ZERO;
    if (forced == 2) forcey = fgrad * rho;  /* FORCING_Y */
    else if (forced) forcex = fgrad * rho;
    out[0] = (x01 - omega * (x01 - e01)) + (forcex - forcey);
    out[1] = (x03 - omega * (x03 - e03)) + (forcex + forcey);
    out[2] = (x05 - omega * (x05 - e05)) + (forcex);
    out[3] = (x08 - omega * (x08 - e08)) + (forcey);
    out[4] = (x10 - omega * (x10 - e10)) + ((-forcex) - forcey);
    out[5] = (x12 - omega * (x12 - e12)) + ((-forcex) + forcey);
    out[6] = (x14 - omega * (x14 - e14)) + (-forcex);
    out[7] = (x17 - omega * (x17 - e17)) + (-forcey);
    out[8] = x19 - omega * (x19 - e19);
}

/* col_MC.F90:97-293 for rows j0..j1 without LES or forcing: the same per-cell operations as the
 * general loop below, over restrict row pointers with the flags constant, so that the compiler
 * runs several cells per SIMD instruction (each cell's IEEE operations are unchanged) */
static void FN(col_MC_rows_plain)(orc_state *s, int j0, int j1)
{
    const int l = s->l, noshift = s->p.noshift;
    const size_t ld = (size_t)s->ld;
    const K omega = (K)s->omega;
    for (int j = j0; j <= j1; ++j) {
        const size_t jm = (size_t)(j - 1) * ld, j0r = (size_t)j * ld, jp = (size_t)(j + 1) * ld;
        const S *restrict p01 = (const S *)s->A[0] + jp - 1;  /* (i-1, j+1) */
        const S *restrict p03 = (const S *)s->A[1] + jm - 1;  /* (i-1, j-1) */
        const S *restrict p05 = (const S *)s->A[2] + j0r - 1; /* (i-1, j)   */
        const S *restrict p08 = (const S *)s->A[3] + jm;      /* (i, j-1)   */
        const S *restrict p10 = (const S *)s->A[4] + jp + 1;  /* (i+1, j+1) */
        const S *restrict p12 = (const S *)s->A[5] + jm + 1;  /* (i+1, j-1) */
        const S *restrict p14 = (const S *)s->A[6] + j0r + 1; /* (i+1, j)   */
        const S *restrict p17 = (const S *)s->A[7] + jp;      /* (i, j+1)   */
        S *restrict p19 = (S *)s->A[8] + j0r;                 /* in place   */
        S *restrict b01 = (S *)s->B[0] + j0r, *restrict b03 = (S *)s->B[1] + j0r;
        S *restrict b05 = (S *)s->B[2] + j0r, *restrict b08 = (S *)s->B[3] + j0r;
        S *restrict b10 = (S *)s->B[4] + j0r, *restrict b12 = (S *)s->B[5] + j0r;
        S *restrict b14 = (S *)s->B[6] + j0r, *restrict b17 = (S *)s->B[7] + j0r;
        /* the eighteen row streams never overlap: the a planes are read, the b planes and the
         * rest population (read and written at the same index) are written */
#pragma GCC ivdep
        for (int i = 1; i <= l; ++i) {
            K x[9], o[9];
            x[0] = (K)p01[i]; x[1] = (K)p03[i]; x[2] = (K)p05[i]; x[3] = (K)p08[i]; x[4] = (K)p10[i];
            x[5] = (K)p12[i]; x[6] = (K)p14[i]; x[7] = (K)p17[i]; x[8] = (K)p19[i];
            FN(collide)(x, omega, ZERO, 0, 0, ZERO, noshift, o);
            b01[i] = (S)o[0]; b03[i] = (S)o[1]; b05[i] = (S)o[2]; b08[i] = (S)o[3];
            b10[i] = (S)o[4]; b12[i] = (S)o[5]; b14[i] = (S)o[6]; b17[i] = (S)o[7];
            p19[i] = (S)o[8];
        }
    }
}

/* col_MC.F90:97-293 for rows j0..j1, then (by the caller) the pointer swap :311-341 */
static void FN(col_MC_rows)(orc_state *s, int j0, int j1)
{
    if (s->p.tcase != ORC_POF && s->p.tcase != ORC_MYV && !s->p.les) {
        FN(col_MC_rows_plain)(s, j0, j1);
        return;
    }
    const int l = s->l;
    const K omega = (K)s->omega, fgrad = (K)s->fgrad, cte_s = (K)s->p.cte_s;
    const int forced = (s->p.tcase == ORC_POF || s->p.tcase == ORC_MYV) ? (s->p.force_y ? 2 : 1) : 0, les = s->p.les;
    K x[9], o[9];
    for (int j = j0; j <= j1; ++j) {
        for (int i = 1; i <= l; ++i) {
            x[0] = RA(0, i - 1, j + 1);
            x[1] = RA(1, i - 1, j - 1);
            x[2] = RA(2, i - 1, j);
            x[3] = RA(3, i, j - 1);
            x[4] = RA(4, i + 1, j + 1);
            x[5] = RA(5, i + 1, j - 1);
            x[6] = RA(6, i + 1, j);
            x[7] = RA(7, i, j + 1);
            x[8] = RA(8, i, j);
            FN(collide)(x, omega, fgrad, forced, les, cte_s, s->p.noshift, o);
            for (int q = 0; q < 8; ++q) B_(q, i, j) = (S)o[q];
            A_(8, i, j) = (S)o[8];
        }
    }
}

static void FN(swap)(orc_state *s)
{
    for (int q = 0; q < 8; ++q) { void *t = s->A[q]; s->A[q] = s->B[q]; s->B[q] = t; }
}

/* movef.F90:46-53 followed by col.F90:87-237 */
static void FN(movef_col)(orc_state *s)
{
    const int l = s->l, m = s->m;
    const K omega = (K)s->omega, fgrad = (K)s->fgrad, cte_s = (K)s->p.cte_s;
    const int forced = (s->p.tcase == ORC_POF || s->p.tcase == ORC_MYV) ? (s->p.force_y ? 2 : 1) : 0, les = s->p.les;
    for (int j = 1; j <= m; ++j) {
        for (int i = 1; i <= l; ++i) {
            B_(0, i, j) = A_(0, i - 1, j + 1);
            B_(1, i, j) = A_(1, i - 1, j - 1);
            B_(2, i, j) = A_(2, i - 1, j);
            B_(3, i, j) = A_(3, i, j - 1);
            B_(4, i, j) = A_(4, i + 1, j + 1);
            B_(5, i, j) = A_(5, i + 1, j - 1);
            B_(6, i, j) = A_(6, i + 1, j);
            B_(7, i, j) = A_(7, i, j + 1);
        }
    }
    K x[9], o[9];
    for (int j = 1; j <= m; ++j) {
        for (int i = 1; i <= l; ++i) {
            for (int q = 0; q < 8; ++q) x[q] = RB(q, i, j);
            x[8] = RA(8, i, j);
            FN(collide)(x, omega, fgrad, forced, les, cte_s, s->p.noshift, o);
            for (int q = 0; q < 9; ++q) A_(q, i, j) = (S)o[q];
        }
    }
}

static void FN(step)(orc_state *s, int nsteps, int nthreads)
{
    for (int it = 0; it < nsteps; ++it) {
        FN(boundaries)(s);
        if (s->p.fused) {
            if (nthreads > 1) {
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
                for (int j = 1; j <= s->m; ++j) FN(col_MC_rows)(s, j, j);
            } else {
                FN(col_MC_rows)(s, 1, s->m);
            }
            FN(swap)(s);
        } else {
            FN(movef_col)(s);
        }
    }
}

/* per-cell moments exactly as diagno.F90:82-93 */
static inline void FN(moments)(const orc_state *s, int i, int j, K *rho_o, K *xj_o, K *yj_o)
{
    const K cte1 = s->p.noshift ? ZERO : UNO;  /* diagno.F90:42-46 */
    K x01 = RA(0, i, j), x03 = RA(1, i, j), x05 = RA(2, i, j), x08 = RA(3, i, j);
    K x10 = RA(4, i, j), x12 = RA(5, i, j), x14 = RA(6, i, j), x17 = RA(7, i, j);
    K x19 = RA(8, i, j);
    K rho = ((((x01 + x03) + x10) + x12) + (((x05 + x08) + x14) + x17) + x19) + cte1;
    K rhoinv = UNO / rho;
    *xj_o = (((x03 - x12) + (x01 - x10)) + (x05 - x14)) * rhoinv;
    *yj_o = (((x03 - x01) + (x12 - x10)) + (x08 - x17)) * rhoinv;
    *rho_o = rho;
}

/* diagno.F90:63-101 */
static void FN(diagno)(const orc_state *s, int mode, double *out)
{
    const int l = s->l, m = s->m;
    if (mode == 0) {
        K rtot = ZERO, xtot = ZERO, ytot = ZERO, stot = ZERO;
        for (int j = 1; j <= m; ++j) {
            for (int i = 1; i <= l; ++i) {
                K rho, xj, yj;
                FN(moments)(s, i, j, &rho, &xj, &yj);
                rtot = rtot + rho;
                xtot = xtot + xj;
                ytot = ytot + yj;
                stot = stot + (xj * xj + yj * yj);
            }
        }
        rtot = (rtot / (K)(float)l) / (K)(float)m;
        xtot = (xtot / (K)(float)l) / (K)(float)m;
        ytot = (ytot / (K)(float)l) / (K)(float)m;
        stot = (stot / (K)(float)l) / (K)(float)m;
        out[0] = (double)xtot; out[1] = (double)ytot; out[2] = (double)rtot; out[3] = (double)stot;
    } else {
        double rtot = 0, xtot = 0, ytot = 0, stot = 0;
        for (int j = 1; j <= m; ++j) {
            for (int i = 1; i <= l; ++i) {
                if (mode == 2 && s->obs[(size_t)(i - 1) + (size_t)(j - 1) * (size_t)l]) continue;
                K rho, xj, yj;
                FN(moments)(s, i, j, &rho, &xj, &yj);
                rtot += (double)rho;
                xtot += (double)xj;
                ytot += (double)yj;
                stot += (double)(xj * xj + yj * yj);
            }
        }
        double n = (double)l * (double)m;
        out[0] = xtot / n; out[1] = ytot / n; out[2] = rtot / n; out[3] = stot / n;
    }
}

/* draglift.F90:41-100 (box around the obstacle centre, border 3) */
static void FN(draglift)(const orc_state *s, int mode, double *out)
{
    static const int icx[8] = {1, 1, 1, 0, -1, -1, -1, 0};
    static const int icy[8] = {-1, 1, 0, 1, -1, 1, 0, -1};
    const int l = s->l, m = s->m;
    const int icoord = s->icoord, jcoord = s->jcoord, radius = s->p.radius, delta = 3;
    const int istart = icoord - radius - delta, istop = icoord + radius + delta;
    const int jstart = jcoord - radius - delta, jstop = jcoord + radius + delta;
    const K u_inflow = (K)0.1f;
#define OBSAT(i, j) (((i) >= 1 && (i) <= l && (j) >= 1 && (j) <= m) ? s->obs[(size_t)((i) - 1) + (size_t)((j) - 1) * (size_t)l] : 0)
    K fK[2] = {ZERO, ZERO};
    double fD[2] = {0.0, 0.0};
    for (int comp = 0; comp < 2; ++comp) {
        for (int j = jstart; j <= jstop; ++j) {
            for (int i = istart; i <= istop; ++i) {
                if (OBSAT(i, j) != 0) continue;
                if (i < 0 || i > l + 1 || j < 0 || j > m + 1) continue;
                K f[8];
                for (int q = 0; q < 8; ++q) {
                    K c = (K)(comp == 0 ? icx[q] : icy[q]);
                    f[q] = (((K)2.0 * c) * RA(q, i, j)) * (K)OBSAT(i + icx[q], j + icy[q]);
                }
                K sum = ((((((f[0] + f[1]) + f[2]) + f[3]) + f[4]) + f[5]) + f[6]) + f[7];
                if (mode == 0) fK[comp] = fK[comp] + sum;
                else fD[comp] += (double)sum;
            }
        }
    }
#undef OBSAT
    K norm = UNO / ((u_inflow * u_inflow) * (K)radius);
    if (mode == 0) { out[0] = (double)(fK[0] * norm); out[1] = (double)(fK[1] * norm); }
    else { out[0] = fD[0] * (double)norm; out[1] = fD[1] * (double)norm; }
}

/* prof_j.F90:47-67.  The a?? arrays are read directly, so their sums run in the storage kind S
 * (real(sp) in MIXED2); adding cte1 (mykind) and the divisions by den (mykind) run in K. */
static void FN(prof_j)(const orc_state *s, int icoord, double *u, double *v, double *den)
{
    const K cte1 = s->p.noshift ? ZERO : UNO;  /* prof_j.F90:40-44 */
    for (int j = 1; j <= s->m; ++j) {
        int i = icoord;
        S t = ((((((((A_(0, i, j) + A_(1, i, j)) + A_(2, i, j)) + A_(3, i, j)) + A_(4, i, j)) + A_(5, i, j)) + A_(6, i, j)) + A_(7, i, j)) + A_(8, i, j));
        K d = (K)t + cte1;
        S nu = ((A_(0, i, j) - A_(4, i, j)) + (A_(1, i, j) - A_(5, i, j))) + (A_(2, i, j) - A_(6, i, j));
        S nv = ((A_(1, i, j) - A_(0, i, j)) + (A_(3, i, j) - A_(7, i, j))) + (A_(5, i, j) - A_(4, i, j));
        K uu = (K)nu / d;
        K vv = (K)nv / d;
        den[j - 1] = (double)d; u[j - 1] = (double)uu; v[j - 1] = (double)vv;
    }
}

/* SRC/vtk_xy.binary.F90:75-140 and SRC/vtk_om.binary.F90:61-155: the VTK writers' fields in
 * real(sp).  Sums of stored values run in the storage kind S (mystorage, not mykind: float in
 * MIXED2) and are then rounded to sp; the
 * vorticity's quotients divide a storage-kind numerator by an sp denominator in the wider kind. */
static inline float FN(vtk_den)(const orc_state *s, int i, int j)
{
    S t = ((((((((A_(0, i, j) + A_(1, i, j)) + A_(2, i, j)) + A_(3, i, j)) + A_(4, i, j)) + A_(5, i, j)) + A_(6, i, j)) +
            A_(7, i, j)) + A_(8, i, j));
    return (float)(t + (S)(s->p.noshift ? 0.0f : 1.0f));  /* cte1: vtk_xy.binary.F90:46-50 */
}
static inline S FN(vtk_u)(const orc_state *s, int i, int j)
{
    return ((((A_(0, i, j) + A_(1, i, j)) + A_(2, i, j)) - A_(4, i, j)) - A_(5, i, j)) - A_(6, i, j);
}
static inline S FN(vtk_v)(const orc_state *s, int i, int j)
{
    return ((((A_(1, i, j) + A_(3, i, j)) + A_(5, i, j)) - A_(0, i, j)) - A_(4, i, j)) - A_(7, i, j);
}
static void FN(vtk)(const orc_state *s, int from_ghost_row, float *u, float *w, float *rho, float *vort, float *stream)
{
    const int l = s->l, m = s->m;
    for (int j = 1; j <= m; ++j)
        for (int i = 1; i <= l; ++i) {
            const size_t k = (size_t)(i - 1) + (size_t)(j - 1) * (size_t)l;
            const float den = FN(vtk_den)(s, i, j);
            u[k] = (float)FN(vtk_u)(s, i, j) / den;
            w[k] = (float)FN(vtk_v)(s, i, j) / den;
            rho[k] = den;
        }
    float *phi = (float *)malloc(sizeof(float) * (size_t)(m + 2));
    float prev = 0.0f;
    phi[0] = 0.0f;
    for (int j = from_ghost_row ? 0 : 1; j <= m; ++j) {  /* column integral of u at i = 1 */
        const float den = FN(vtk_den)(s, 1, j);
        const float uv = (float)FN(vtk_u)(s, 1, j);
        phi[j] = prev + uv / den;
        prev = phi[j];
    }
    for (int j = 2; j <= m - 1; ++j)
        for (int i = 2; i <= l - 1; ++i) {
            const size_t k = (size_t)(i - 2) + (size_t)(j - 2) * (size_t)(l - 2);
            const float d_up = FN(vtk_den)(s, i, j + 1), d_down = FN(vtk_den)(s, i, j - 1);
            const float d_left = FN(vtk_den)(s, i - 1, j), d_right = FN(vtk_den)(s, i + 1, j);
            const float up1 = (float)(FN(vtk_u)(s, i, j + 1) / (S)d_up);
            const float down1 = (float)(FN(vtk_u)(s, i, j - 1) / (S)d_down);
            const float left1 = (float)(FN(vtk_v)(s, i - 1, j) / (S)d_left);
            const float right1 = (float)(FN(vtk_v)(s, i + 1, j) / (S)d_right);
            vort[k] = 0.5f * (up1 - down1) - 0.5f * (right1 - left1);
            const float den = FN(vtk_den)(s, i, j);
            const float vv = (float)FN(vtk_v)(s, i, j);
            phi[j] = phi[j] - vv / den;
            stream[k] = phi[j];
        }
    free(phi);
}

static void FN(fields)(const orc_state *s, double *rho, double *u, double *v)
{
    for (int j = 1; j <= s->m; ++j) {
        for (int i = 1; i <= s->l; ++i) {
            K r, x, y;
            FN(moments)(s, i, j, &r, &x, &y);
            size_t k = (size_t)(i - 1) + (size_t)(j - 1) * (size_t)s->l;
            rho[k] = (double)r; u[k] = (double)x; v[k] = (double)y;
        }
    }
}

static void FN(get_pops)(const orc_state *s, double *out)
{
    for (int q = 0; q < 9; ++q)
        for (size_t k = 0; k < s->n; ++k) out[(size_t)q * s->n + k] = (double)((S *)s->A[q])[k];
}

static void FN(set_pops)(orc_state *s, const double *in)
{
    for (int q = 0; q < 9; ++q)
        for (size_t k = 0; k < s->n; ++k) ((S *)s->A[q])[k] = (S)in[(size_t)q * s->n + k];
}

#undef A_
#undef B_
#undef RA
#undef RB
#undef UNO
#undef ZERO
#undef TRE
#undef RF
#undef QF
#undef P0
#undef P1
#undef P2
