// bgk_setup.h -- host-side set-up of one case: the reference's build_bcond, hencol, build_obs
// and init semantics, evaluated in the compute kind K (templates), producing the scalars,
// face rules, obstacle mask and initial populations the device lattice needs.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/bgk2d_gb300.h"
#include "bgk_common.cuh"

namespace bgk {

struct CaseSetup {
    int faces[4];
    double wt[4][9];
    double omega, fgrad, u00, u0;   // values of the compute kind
    int forced;
    int bfs = 0;                    // backward-facing step (solid block, inflow above it, outflow)
    int stepx = 0, stepy = 0;       // step corner (SRC/input.F90:74-75)
    int inflow_y0 = 0;              // first row of the x_lo inflow (the step's wall below it)
    int corner_x = 0;               // the x-wall rule sets the corner ghosts (-DTRICK1)
    int noshift = 0;                // populations stored whole, not as deviations (-DNOSHIFT)
    int les;                        // Smagorinsky eddy viscosity on
    double cte_s;                   // Smagorinsky constant (compute kind)
    double u_inflow;                // compute-kind inflow speed (peak for the parabolic profile)
    std::vector<double> inflow;     // [3][ly+2] equilibrium deviations of 01,03,05 at x_lo
    std::vector<int32_t> obs;       // obs(1:lx,1:ly), i fastest
    int bbox[5];                    // imin, imax, jmin, jmax, nobs
    int icoord, jcoord, radius;
    bool has_obs;
};

// equilibrium deviation of an inflow ghost at velocity (xj, 0) with rho = 1
// (SRC/bcond.inflow.F90:101-113), or the equilibrium itself for populations stored whole
// (cte1 = 1, SRC/bcond.inflow.F90:48-52).  The `3.d0` literal promotes that sub-expression to
// double even in a single-precision build, which is kept here.
template <typename K>
inline void inflow_eq(K xj, K out[3], bool noshift = false)
{
    const K rf = (K)3, qf = (K)1.5, crho = (K)1, cte1 = noshift ? (K)1 : (K)0;
    const K p1 = (K)(1.0 / 9.0), p2 = (K)(1.0 / 36.0);
    const K yj = (K)0;
    const K cvsq = xj * xj + yj * yj;
    const double dc = (double)cvsq;
    const K a = xj - yj, b = xj + yj, c = xj;
    K cx01 = (K)((double)(rf * a) + (double)qf * ((3.0 * (double)a) * (double)a - dc));
    K cx03 = (K)((double)(rf * b) + (double)qf * ((3.0 * (double)b) * (double)b - dc));
    K cx05 = (K)((double)(rf * c) + (double)qf * ((3.0 * (double)c) * (double)c - dc));
    out[0] = (crho * p2) * (cte1 + cx01);
    out[1] = (crho * p2) * (cte1 + cx03);
    out[2] = (crho * p1) * (cte1 + cx05);
}

// obstacle mask as SRC/build.obs.F90:49-205 (circle by default, SQUARE, HALF_CIRCLE)
template <typename K>
inline void build_obs(int l, int m, int shape, int radius, int icoord, int jcoord, std::vector<int32_t> &obs, int bbox[5])
{
    obs.assign((size_t)l * (size_t)m, 0);
    int imin = l, jmin = m, imax = 0, jmax = 0, nobs = 0;
    auto set = [&](int i, int j) {
        obs[(size_t)(i - 1) + (size_t)(j - 1) * (size_t)l] = 1;
        ++nobs;
        imin = std::min(imin, i); jmin = std::min(jmin, j);
        imax = std::max(imax, i); jmax = std::max(jmax, j);
    };
    if (shape == BGK_OBS_SQUARE) {
        const K hsize = (K)radius;
        for (int j = 1; j <= m; ++j)
            if ((K)j >= ((K)jcoord - hsize) && (K)j <= ((K)jcoord + hsize))
                for (int i = 1; i <= l; ++i)
                    if ((K)i >= ((K)icoord - hsize) && (K)i <= ((K)icoord + hsize)) set(i, j);
    } else if (shape == BGK_OBS_CIRCLE || shape == BGK_OBS_HALF_CIRCLE) {
        const K R = (K)radius * (K)1;
        const int j0 = shape == BGK_OBS_HALF_CIRCLE ? m / 2 : 1;
        for (int j = j0; j <= m; ++j)
            for (int i = 1; i <= l; ++i) {
                const K d2 = (K)((icoord - i) * (icoord - i) + (jcoord - j) * (jcoord - j));
                if (d2 <= R * R) set(i, j);
            }
    }
    bbox[0] = imin; bbox[1] = imax; bbox[2] = jmin; bbox[3] = jmax; bbox[4] = nobs;
}

// initial populations (host kind H, reference layout (0:l+1, 0:m+1) per direction)
// BGK_INIT_REST / BGK_INIT_TGV_REF: SRC/init.F90:83-137 in kind K; cte1 = 1 for populations
// stored whole (SRC/init.F90:73-77).
template <typename K, typename H>
inline void init_reference(int l, int m, bool vortex, std::vector<H> &out, bool noshift = false)
{
    const size_t n = (size_t)(l + 2) * (size_t)(m + 2);
    out.assign(9 * n, (H)0);
    const K pi = (K)3.14159265358979323846f;  // default-real literal in init.F90:63
    const K rf = (K)3, qf = (K)1.5, crho = (K)1, cte1 = noshift ? (K)1 : (K)0;
    const K p0 = (K)(4.0 / 9.0), p1 = (K)(1.0 / 9.0), p2 = (K)(1.0 / 36.0);
    for (int j = 0; j <= m + 1; ++j) {
        const K y = (K)(((double)(K)j - 0.5) / (double)(K)m);
        for (int i = 0; i <= l + 1; ++i) {
            K xj = (K)0, yj = (K)0;
            if (vortex) {
                const K x = (K)(((double)(K)i - 0.5) / (double)(K)l);
                const K ax = (K)2 * pi * x, ay = (K)2 * pi * y;
                xj = (K)((0.1 * (double)std::sin(ax)) * (double)std::cos(ay));
                yj = (K)(-((0.1 * (double)std::cos(ax)) * (double)std::sin(ay)));
            }
            const K cvsq = xj * xj + yj * yj;
            const double dc = (double)cvsq;
            auto cx = [&](K lin, K d) -> K {
                return (K)((double)(rf * lin) + (double)qf * ((3.0 * (double)d) * (double)d - dc));
            };
            const K dm = xj - yj, dp = xj + yj;
            K c[9];
            c[0] = cx(xj - yj, dm);
            c[1] = cx(xj + yj, dp);
            c[2] = cx(xj, xj);
            c[3] = cx(yj, yj);
            c[4] = cx(-xj - yj, dp);
            c[5] = cx(-xj + yj, dm);
            c[6] = cx(-xj, xj);
            c[7] = cx(-yj, yj);
            c[8] = (K)((double)rf * 0.0 + (double)qf * ((3.0 * 0.0) * 0.0 - dc));
            const K w[9] = {p2, p2, p1, p1, p2, p2, p1, p1, p0};
            const size_t k = (size_t)i + (size_t)j * (size_t)(l + 2);
            for (int q = 0; q < 9; ++q) out[(size_t)q * n + k] = (H)((crho * w[q]) * (cte1 + c[q]));
        }
    }
}

// build_bcond + hencol (SRC/build.bcond.F90:47-56, SRC/hencol.F90:30-50) and the face rules of
// the reference's boundary routines, in compute kind K.  Returns an empty string on success.
template <typename K>
inline std::string setup_case(const bgk_case_desc &d, CaseSetup &cs)
{
    const int l = d.lx, m = d.ly;
    K u0 = (K)d.u0, svisc = (K)d.svisc, u00;
    const bool force_case = d.tcase == BGK_CASE_POF || d.tcase == BGK_CASE_MYV || d.tcase == BGK_CASE_CUSTOM;
    if (force_case) { u00 = (K)0; }
    else { u00 = u0; u0 = (K)0; }
    K omega = ((K)1 + (K)1) / (((K)6 * svisc) + (K)1);
    if (d.omega > 0) omega = (K)d.omega;
    const K fgrad = (((K)4 * u0) * svisc) / (((K)3 * (K)m) * (K)m);
    cs.omega = (double)omega;
    cs.les = d.les != 0;
    cs.cte_s = (double)(K)d.cte_s;  // namelist value read in mykind
    cs.fgrad = (double)fgrad;
    cs.u00 = (double)u00;
    cs.u0 = (double)u0;
    // 1: the body force along x (SRC/col_MC.F90:268-274), 2: along y (-DFORCING_Y)
    cs.forced = (force_case && fgrad != (K)0) ? (d.force_y ? 2 : 1) : 0;
    if (d.force_y && !force_case) return "force_y: a body-forced case only (POF, MYV or CUSTOM)";
    for (int f = 0; f < 4; ++f)
        for (int q = 0; q < 9; ++q) cs.wt[f][q] = 0.0;
    const K force = u00 / (K)6.0;  // SRC/bcond.driven.F90:41
    switch (d.tcase) {
    case BGK_CASE_LDC:
        cs.faces[XLO] = cs.faces[XHI] = cs.faces[YLO] = cs.faces[YHI] = FK_WALL;
        cs.wt[YHI][D01] = (double)force;      // a01(i-1,m1) = a12(i,m) + force
        cs.wt[YHI][D10] = (double)(-force);   // a10(i+1,m1) = a03(i,m) - force
        break;
    case BGK_CASE_TGV:
        cs.faces[XLO] = cs.faces[XHI] = cs.faces[YLO] = cs.faces[YHI] = FK_PERIODIC;
        break;
    case BGK_CASE_POF:
        cs.faces[XLO] = cs.faces[XHI] = FK_PERIODIC;
        cs.faces[YLO] = cs.faces[YHI] = FK_WALL;
        break;
    case BGK_CASE_MYV:  // SRC/boundaries.F90:46-48: bcond_periodic, with the volume force
        cs.faces[XLO] = cs.faces[XHI] = cs.faces[YLO] = cs.faces[YHI] = FK_PERIODIC;
        break;
    case BGK_CASE_VKS:
        cs.faces[XLO] = FK_INFLOW;
        cs.faces[XHI] = FK_OUTFLOW_EQ;
        cs.faces[YLO] = cs.faces[YHI] = FK_PERIODIC;
        break;
    case BGK_CASE_COU:
        cs.faces[XLO] = cs.faces[XHI] = FK_PERIODIC;
        cs.faces[YLO] = cs.faces[YHI] = FK_WALL;
        cs.wt[YHI][D01] = (double)force;
        cs.wt[YHI][D10] = (double)(-force);
        break;
    case BGK_CASE_BFS:
        // SRC/bcond.step.F90 as face and obstacle rules: the equilibrium outflow at x_hi
        // (:66-101), the parabolic inflow at x_lo from row stepy up (:118-151) with the step's
        // wall below it, no-slip walls at y (:168-190), and the block x < stepx, y < stepy as
        // obstacle cells, whose faces (:207-255) are the obstacle bounce-back except at the
        // step's corner (step_bounce)
        cs.faces[XLO] = FK_INFLOW;
        cs.faces[XHI] = FK_OUTFLOW_EQ;
        cs.faces[YLO] = cs.faces[YHI] = FK_WALL;
        cs.bfs = 1;
        cs.stepx = l / 20;
        cs.stepy = m / 2;
        cs.inflow_y0 = cs.stepy;
        if (cs.stepx < 2 || m < 4) return "backward-facing step needs lx >= 40 and ly >= 4";
        break;
    case BGK_CASE_CUSTOM:
        for (int f = 0; f < 4; ++f) cs.faces[f] = d.faces[f];
        for (int f = 0; f < 4; ++f) {
            for (int q = 0; q < 8; ++q) {
                const K cu = (K)cx_of(q) * (K)d.wall_u[f][0] + (K)cy_of(q) * (K)d.wall_u[f][1];
                const bool diag = cx_of(q) != 0 && cy_of(q) != 0;
                cs.wt[f][q] = diag ? (double)(cu / (K)6) : (double)((cu * (K)2) / (K)3);
            }
        }
        break;
    default:
        return "unknown test case";
    }
    if (d.noshift) {
        // SRC/precision.F90: the reference stores half-precision populations as deviations only
        if (d.storage != BGK_STORE_F32 && d.storage != BGK_STORE_F64) return "noshift: FP32 or FP64 storage only";
        cs.noshift = 1;
    }
    if (d.trick1) {
        // the merged loop of SRC/bcond.driven.F90:43-81 indexes the lid by the wall index j = 1..m
        if (d.tcase != BGK_CASE_LDC) return "trick1: lid-driven cavity only";
        if (l != m) return "trick1: square box mandatory (SRC/check_case.F90:173-178)";
        cs.corner_x = 1;
    }
    for (int f = 0; f < 4; ++f)
        if (cs.faces[f] < FK_WALL || cs.faces[f] > FK_OUTFLOW_ZG) return "unknown face kind";
    if ((cs.faces[XLO] == FK_PERIODIC) != (cs.faces[XHI] == FK_PERIODIC)) return "x faces: periodic must pair";
    if ((cs.faces[YLO] == FK_PERIODIC) != (cs.faces[YHI] == FK_PERIODIC)) return "y faces: periodic must pair";
    if (cs.faces[XHI] == FK_INFLOW) return "inflow is supported on the x_lo face only";
    if (cs.faces[XLO] == FK_OUTFLOW_EQ || cs.faces[XLO] == FK_OUTFLOW_ZG) return "outflow is supported on the x_hi face only";
    for (int f = YLO; f <= YHI; ++f)
        if (cs.faces[f] != FK_WALL && cs.faces[f] != FK_PERIODIC) return "y faces must be walls or periodic";

    // inflow table (u_inflow=0.1 is a default-real literal in SRC/bcond.inflow.F90:59)
    const K uin = d.u_inflow > 0 ? (K)d.u_inflow : (K)0.1f;
    cs.u_inflow = (double)uin;
    cs.inflow.assign(3 * (size_t)(m + 2), 0.0);
    if (cs.bfs) {
        // parabolic inflow above the step, u = 0.1 (j-stepy)(m-j) / ((m-stepy)^2/4) with the
        // reference's float() conversions and integer division (SRC/bcond.step.F90:133-136)
        const int sy = cs.stepy;
        for (int j = sy; j <= m + 1; ++j) {
            const K xj = ((uin * (K)(float)(j - sy)) * (K)(float)(m - j)) / (K)(float)(((m - sy) * (m - sy)) / 4);
            K e[3];
            inflow_eq<K>(xj, e, d.noshift != 0);
            for (int t = 0; t < 3; ++t) cs.inflow[(size_t)t * (m + 2) + j] = (double)e[t];
        }
    } else if (cs.faces[XLO] == FK_INFLOW) {
        for (int j = 0; j <= m + 1; ++j) {
            K u = uin;
            if (d.inflow_profile == 1) {
                const double yy = j - 0.5;
                u = (K)(4.0 * (double)uin * yy * ((double)m - yy) / ((double)m * (double)m));
            }
            K e[3];
            inflow_eq<K>(u, e, d.noshift != 0);
            for (int t = 0; t < 3; ++t) cs.inflow[(size_t)t * (m + 2) + j] = (double)e[t];
        }
    }

    // obstacle (SRC/build.obs.F90; VKS always has one, SRC/Makefile:176)
    int shape = d.obstacle;
    if (d.tcase == BGK_CASE_VKS && shape == BGK_OBS_NONE) shape = BGK_OBS_CIRCLE;
    if (cs.bfs && shape != BGK_OBS_NONE) return "backward-facing step: no obstacle besides the step";
    cs.radius = d.radius;
    cs.icoord = d.obs_icoord >= 0 ? d.obs_icoord : 2 * l / 5;
    cs.jcoord = d.obs_jcoord >= 0 ? d.obs_jcoord : m / 2;
    cs.has_obs = false;
    cs.bbox[0] = l; cs.bbox[1] = 0; cs.bbox[2] = m; cs.bbox[3] = 0; cs.bbox[4] = 0;
    if (shape == BGK_OBS_MASK) {
        if (!d.obs_mask) return "obstacle mask pointer is NULL";
        cs.obs.assign(d.obs_mask, d.obs_mask + (size_t)l * (size_t)m);
        int imin = l, jmin = m, imax = 0, jmax = 0, nobs = 0;
        for (int j = 1; j <= m; ++j)
            for (int i = 1; i <= l; ++i)
                if (cs.obs[(size_t)(i - 1) + (size_t)(j - 1) * l] == 1) {
                    ++nobs;
                    imin = std::min(imin, i); jmin = std::min(jmin, j);
                    imax = std::max(imax, i); jmax = std::max(jmax, j);
                }
        cs.bbox[0] = imin; cs.bbox[1] = imax; cs.bbox[2] = jmin; cs.bbox[3] = jmax; cs.bbox[4] = nobs;
    } else if (shape != BGK_OBS_NONE) {
        if (shape < BGK_OBS_CIRCLE || shape > BGK_OBS_HALF_CIRCLE) return "unknown obstacle shape";
        if (d.radius > m - 2) return "radius too big";  // SRC/input.F90:83-86
        build_obs<K>(l, m, shape, d.radius, cs.icoord, cs.jcoord, cs.obs, cs.bbox);
    } else if (cs.bfs) {
        // the solid block x = 1..stepx-1, y = 1..stepy-1 of the step; it touches the x_lo and
        // y_lo faces, whose rules never reach into it from a fluid cell
        cs.obs.assign((size_t)l * (size_t)m, 0);
        for (int j = 1; j < cs.stepy; ++j)
            for (int i = 1; i < cs.stepx; ++i) cs.obs[(size_t)(i - 1) + (size_t)(j - 1) * l] = 1;
        cs.bbox[0] = 1; cs.bbox[1] = cs.stepx - 1; cs.bbox[2] = 1; cs.bbox[3] = cs.stepy - 1;
        cs.bbox[4] = (cs.stepx - 1) * (cs.stepy - 1);
    } else {
        cs.obs.assign((size_t)l * (size_t)m, 0);
    }
    if (cs.bbox[4] > 0) {
        cs.has_obs = true;
        if (!cs.bfs && (cs.bbox[0] < 2 || cs.bbox[1] > l - 1 || cs.bbox[2] < 2 || cs.bbox[3] > m - 1))
            return "obstacle must not touch the domain boundary";
    }
    return "";
}

}  // namespace bgk
