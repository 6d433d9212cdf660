// bgk_kernels.cuh -- fused stream + collide kernels for one lattice (templated bodies).
//
// Ping-pong (PP): the pull form of SRC/col_MC.F90:97-293.  Cell (x,y) reads population q from
// (x - c_q) in the source buffer, relaxes, and writes the destination buffer at (x,y) (the rest
// population too, where col_MC.F90:293 updates a19 in place).  The ghost-frame fills of
// SRC/bcond.*.F90 are folded into the pull: a source outside the interior is replaced by the
// value the reference's boundary routine would have written there, and an obstacle source by
// the value SRC/bcond.obs.F90:59-71 would have written (the pulling cell's own opposite
// population).
//
// AA: one buffer.  Phase 0 holds post-collision values in swapped slots (plane opp(q) at x holds
// f*_q(x)); the "P" step pulls from the neighbours' swapped slots, relaxes and pushes to
// (x + c_q) in plane q (phase 1: streamed, pre-collision values); the "L" step is purely local
// and returns to phase 0.  Every cell reads and writes the same nine slots, so the update is
// in place.  Boundary rules are applied in the P step when pulling and when pushing.
//
// Two-pass (ORIGINAL, SRC/movef.F90 + SRC/col.F90): the ping-pong kernel without its collision
// streams into the second buffer, and col_kernel relaxes that buffer in place.
//
// Each thread updates N consecutive cells of a row with 8- or 16-byte vector accesses; the +-x
// neighbours come from adjacent lanes.  A block may first ask for an L2 prefetch of the rows of
// the block a set distance ahead in launch order (prefetch_tile).  The collision with the
// Smagorinsky eddy viscosity and whole-population storage are template parameters (the
// collision variant CV: CV_LES, CV_NOSHIFT), instantiated separately.
//
// All arithmetic is one IEEE operation per reference operation: this file is compiled with
// -fmad=false for the FP32/FP64 kinds so that results are bit-identical to the reference's
// serial arithmetic; the 16-bit storage kernels are compiled with contraction enabled.
#pragma once

#include "bgk_common.cuh"

namespace bgk {

// Collision variants (bits of the template parameter CV of the step kernels):
// CV_LES      the Smagorinsky eddy viscosity of -DLES (SRC/col_MC.F90:178-248);
// CV_NOSHIFT  the planes hold the populations f themselves, not f - w (-DNOSHIFT,
//             SRC/col_MC.F90:70-75): cte1 = 0 and cte0 = 1 in the collision.  FP32/FP64 kinds only.
constexpr int CV_LES = 1, CV_NOSHIFT = 2;

// ---------------------------------------------------------------------------------------------
// collision: SRC/col_MC.F90:128-176 (equilibrium) and :285-293 (relaxation + body force)
// ---------------------------------------------------------------------------------------------
// Smagorinsky eddy viscosity (SRC/col_MC.F90:178-248): the relaxation rate from the
// non-equilibrium momentum flux n_q = x_q - e_q; the molecular rate omega1 equals omega
// (hencol.F90:30-31).
template <typename K>
__device__ __forceinline__ K les_omega(K n01, K n03, K n05, K n08, K n10, K n12, K n14, K n17, K omega1, K cte_s)
{
    const K uno = (K)1;
    const K pxx = ((((n01 + n03) + n05) + n10) + n12) + n14;
    const K pyy = ((((n01 + n03) + n08) + n10) + n12) + n17;
    const K pxy = (((-n01) + n03) + n10) - n12;
    const K ptotal = sqrt(((pxx * pxx) + (((K)2 * pxy) * pxy)) + (pyy * pyy));
    const K r = uno / omega1;
    const K ts = uno / ((K)2 * omega1) + sqrt((((K)18 * (cte_s * cte_s)) * ptotal) + (r * r)) / (K)2;
    return uno / ts;
}

// +0 + y as the IEEE add gives it (y, except that -0 becomes +0).  The reference adds zeros:
// cte0 = 1 - 1, and the force terms of an unforced case.  On GB300 an FP64 add costs scarce FP64
// throughput, so the FP64 kind makes the same value by an integer select; the FP32 kind keeps
// the add (its step is bound by memory, and the selects cost it registers).  y + (-0) is y.
template <typename K>
__device__ __forceinline__ K add_zero(K y)
{
    if constexpr (sizeof(K) == 8) {
        const long long b = __double_as_longlong(y);
        return __longlong_as_double(b == (long long)0x8000000000000000ull ? 0ll : b);
    } else {
        return (K)0 + y;
    }
}

// x + 0 * d as the IEEE operations give it: 0 * d is +0 for d >= +0 and -0 for d <= -0, and adding
// -0 changes nothing.  The FP64 kind selects on the sign bits, the FP32 kind keeps the operations.
template <typename K>
__device__ __forceinline__ K add_zero_times(K x, K d)
{
    if constexpr (sizeof(K) == 8) return (__double_as_longlong(d) < 0) ? x : add_zero(x);
    else return x + (K)0 * d;
}

template <typename K, int CV = 0>
__device__ __forceinline__ void collide(K (&x)[9], K omega, K fgrad, int forced, K cte_s = (K)0)
{
    constexpr bool NS = (CV & CV_NOSHIFT) != 0;
    const K uno = (K)1, cte1 = (K)1;  // cte0 = uno - cte1 = +0: cte0 + z is add_zero(z)
    const K tre = (K)3, qf = (K)1.5, rf = (K)3;
    const K p0 = (K)(4.0 / 9.0), p1 = (K)(1.0 / 9.0), p2 = (K)(1.0 / 36.0);
    K x01 = x[0], x03 = x[1], x05 = x[2], x08 = x[3], x10 = x[4];
    K x12 = x[5], x14 = x[6], x17 = x[7], x19 = x[8];
    const K sum = (((x01 + x03) + x10) + x12) + (((x05 + x08) + x14) + x17) + x19;
    K rho = NS ? add_zero(sum) : sum + cte1;  // NOSHIFT: cte1 = 0
    K rhoinv = uno / rho;
    K vx = (((x03 - x12) + (x01 - x10)) + (x05 - x14)) * rhoinv;
    K vy = (((x03 - x01) + (x12 - x10)) + (x08 - x17)) * rhoinv;
    K vx2 = vx * vx;
    K vy2 = vy * vy;
    K vsq = vx2 + vy2;
    K vxpy = vx + vy;
    K vxmy = vx - vy;
    // cte0 + z: cte0 = +0 (add_zero), or 1 under NOSHIFT
    auto cte0_plus = [&](K z) -> K { return NS ? uno + z : add_zero(z); };
    K qxpy = cte0_plus(qf * ((tre * vxpy) * vxpy - vsq));
    K qxmy = cte0_plus(qf * ((tre * vxmy) * vxmy - vsq));
    K qx = cte0_plus(qf * (tre * vx2 - vsq));
    K qy = cte0_plus(qf * (tre * vy2 - vsq));
    K q0 = cte0_plus(qf * (-vsq));
    vx = rf * vx;
    vy = rf * vy;
    vxpy = rf * vxpy;
    vxmy = rf * vxmy;
    K rp0 = rho * p0;
    K rp1 = rho * p1;
    K rp2 = rho * p2;
    // + cte1 * (rp - p): cte1 = 1, or 0 under NOSHIFT
    auto eq = [&](K z, K d) -> K { return NS ? add_zero_times(z, d) : z + cte1 * d; };
    K e01 = eq(rp2 * (vxmy + qxmy), rp2 - p2);
    K e03 = eq(rp2 * (vxpy + qxpy), rp2 - p2);
    K e05 = eq(rp1 * (vx + qx), rp1 - p1);
    K e08 = eq(rp1 * (vy + qy), rp1 - p1);
    K e10 = eq(rp2 * (-vxpy + qxpy), rp2 - p2);
    K e12 = eq(rp2 * (-vxmy + qxmy), rp2 - p2);
    K e14 = eq(rp1 * (-vx + qx), rp1 - p1);
    K e17 = eq(rp1 * (-vy + qy), rp1 - p1);
    K e19 = eq(rp0 * (q0), rp0 - p0);
    if constexpr ((CV & CV_LES) != 0) omega = les_omega<K>(x01 - e01, x03 - e03, x05 - e05, x08 - e08, x10 - e10, x12 - e12, x14 - e14,
                                  x17 - e17, omega, cte_s);
    if (forced || sizeof(K) == 4) {
        // forced: 1 along x (forcex = fgrad*rho), 2 along y (forcey, -DFORCING_Y); the other is +0
        const K f = forced ? fgrad * rho : (K)0;
        const K fx = forced == 2 ? (K)0 : f, fy = forced == 2 ? f : (K)0;
        x[0] = (x01 - omega * (x01 - e01)) + (fx - fy);
        x[1] = (x03 - omega * (x03 - e03)) + (fx + fy);
        x[2] = (x05 - omega * (x05 - e05)) + (fx);
        x[3] = (x08 - omega * (x08 - e08)) + (fy);
        x[4] = (x10 - omega * (x10 - e10)) + ((-fx) - fy);
        x[5] = (x12 - omega * (x12 - e12)) + ((-fx) + fy);
        x[6] = (x14 - omega * (x14 - e14)) + (-fx);
        x[7] = (x17 - omega * (x17 - e17)) + (-fy);
    } else {
        // fx = fy = +0: the force terms are +0 for 01, 03, 05, 08, 12 and -0 for 10, 14, 17
        x[0] = add_zero(x01 - omega * (x01 - e01));
        x[1] = add_zero(x03 - omega * (x03 - e03));
        x[2] = add_zero(x05 - omega * (x05 - e05));
        x[3] = add_zero(x08 - omega * (x08 - e08));
        x[4] = x10 - omega * (x10 - e10);
        x[5] = add_zero(x12 - omega * (x12 - e12));
        x[6] = x14 - omega * (x14 - e14);
        x[7] = x17 - omega * (x17 - e17);
    }
    x[8] = x19 - omega * (x19 - e19);
}

// Exact IEEE operations for the 16-bit kinds' collision, on one value (float) or on the values
// of two cells at once (F2: the packed FP32 pair instructions add/sub/mul/fma .f32x2 of sm_100 and
// later, one instruction for both cells).  The intrinsics are never contracted, so the scalar
// and the packed collision round identically and give the same bits for the same inputs.
struct F2 {
    unsigned long long v;
};
__device__ __forceinline__ F2 f2_pack(float lo, float hi)
{
    F2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void f2_unpack(F2 a, float &lo, float &hi)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(a.v));
}
__device__ __forceinline__ float op_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float op_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float op_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float op_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float op_rcp(float a) { return __fdividef(1.0f, a); }
__device__ __forceinline__ F2 op_add(F2 a, F2 b)
{
    F2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ F2 op_sub(F2 a, F2 b)
{
    F2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ F2 op_mul(F2 a, F2 b)
{
    F2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ F2 op_fma(F2 a, F2 b, F2 c)
{
    F2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
    return r;
}
__device__ __forceinline__ F2 op_rcp(F2 a)
{
    float lo, hi;
    f2_unpack(a, lo, hi);
    return f2_pack(__fdividef(1.0f, lo), __fdividef(1.0f, hi));
}
template <typename T> __device__ __forceinline__ T splat(float a);
template <> __device__ __forceinline__ float splat<float>(float a) { return a; }
template <> __device__ __forceinline__ F2 splat<F2>(float a) { return f2_pack(a, a); }

// Collision of the 16-bit storage kernels, on scaled deviations D_q = s_q (f_q - w_q) in FP32.
// Same BGK relaxation as collide<K> rewritten for throughput: with j = rho u and
// A = (rho - 1) - 1.5 j.u, the equilibrium deviation is w_q (A + 3 c.j + 4.5 (c.j)(c.u)); the
// scales satisfy s_q w_q = 8/9 for every q, so D_q' = (1 - omega) D_q + (8/9) omega (...).
// T = float: one cell; T = F2: two cells.  LES: the Smagorinsky rate of each cell replaces omega
// (les_scaled below).
template <typename T> __device__ __forceinline__ T les_rate(T p2, float omega, float cte_s);

// Body force on scaled deviations (SRC/col_MC.F90:285-291): along x (forced = 1) +F on 01, 03, 05
// and -F on 10, 12, 14; along y (forced = 2, -DFORCING_Y) -F on 01, 10, 17 and +F on 03, 08, 12.
// In scaled units F is 32 F on the diagonals and 8 F on the axes, both exact.
template <typename T>
__device__ __forceinline__ void force_scaled(T (&D)[9], T rho, float fgrad, int forced)
{
    const T F = op_mul(splat<T>(fgrad), rho);
    const T F32 = op_mul(splat<T>(32.0f), F), F8 = op_mul(splat<T>(8.0f), F);
    if (forced == 2) {
        D[D01] = op_sub(D[D01], F32); D[D03] = op_add(D[D03], F32); D[D08] = op_add(D[D08], F8);
        D[D10] = op_sub(D[D10], F32); D[D12] = op_add(D[D12], F32); D[D17] = op_sub(D[D17], F8);
    } else {
        D[D01] = op_add(D[D01], F32); D[D03] = op_add(D[D03], F32); D[D05] = op_add(D[D05], F8);
        D[D10] = op_sub(D[D10], F32); D[D12] = op_sub(D[D12], F32); D[D14] = op_sub(D[D14], F8);
    }
}

template <typename T, bool LES = false>
__device__ __forceinline__ void collide_scaled(T (&D)[9], float omega, float fgrad, int forced, float cte_s = 0.0f)
{
    const T i32 = splat<T>(1.0f / 32.0f), i8 = splat<T>(1.0f / 8.0f);
    const T sd = op_add(op_add(D[D01], D[D03]), op_add(D[D10], D[D12]));
    const T sa = op_add(op_add(D[D05], D[D08]), op_add(D[D14], D[D17]));
    const T rho1 = op_fma(sd, i32, op_fma(sa, i8, op_mul(D[D19], splat<T>(0.5f))));
    const T rho = op_add(splat<T>(1.0f), rho1);
    const T dpp = op_sub(D[D03], D[D10]);  // c = (1, 1)
    const T dpm = op_sub(D[D01], D[D12]);  // c = (1,-1)
    const T jx = op_fma(op_add(dpp, dpm), i32, op_mul(op_sub(D[D05], D[D14]), i8));
    const T jy = op_fma(op_sub(dpp, dpm), i32, op_mul(op_sub(D[D08], D[D17]), i8));
    const T rinv = op_rcp(rho);
    const T ux = op_mul(jx, rinv), uy = op_mul(jy, rinv);
    const T A = op_fma(splat<T>(-1.5f), op_fma(jx, ux, op_mul(jy, uy)), rho1);
    if constexpr (LES) {
        // Equilibrium deviations in scaled units, E = (8/9) (A + (c.j)(4.5 c.u) +- 3 c.j), and the
        // non-equilibrium parts N = D - E (N_q / s_q is the reference's x_q - e_q).  The momentum
        // flux P of the non-equilibrium parts sets the eddy viscosity (SRC/col_MC.F90:178-248):
        // D' = D - omega_eff N.
        const T c89 = splat<T>(8.0f / 9.0f);
        const T ux45 = op_mul(splat<T>(4.5f), ux), uy45 = op_mul(splat<T>(4.5f), uy);
        T E[9];
        auto eq = [&](int qp, int qm, T cj, T cu45) {
            const T t = op_fma(cj, cu45, A);
            E[qp] = op_mul(c89, op_fma(splat<T>(3.0f), cj, t));
            E[qm] = op_mul(c89, op_fma(splat<T>(-3.0f), cj, t));
        };
        eq(D05, D14, jx, ux45);
        eq(D08, D17, jy, uy45);
        eq(D03, D10, op_add(jx, jy), op_add(ux45, uy45));
        eq(D01, D12, op_sub(jx, jy), op_sub(ux45, uy45));
        E[D19] = op_mul(c89, A);
        T N[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) N[q] = op_sub(D[q], E[q]);
        const T nd = op_add(op_add(N[D01], N[D03]), op_add(N[D10], N[D12]));
        const T pxx = op_fma(nd, i32, op_mul(op_add(N[D05], N[D14]), i8));
        const T pyy = op_fma(nd, i32, op_mul(op_add(N[D08], N[D17]), i8));
        const T pxy = op_mul(op_sub(op_add(N[D03], N[D10]), op_add(N[D01], N[D12])), i32);
        const T p2 = op_fma(pxx, pxx, op_fma(op_add(pxy, pxy), pxy, op_mul(pyy, pyy)));
        const T w = les_rate<T>(p2, omega, cte_s);
#pragma unroll
        for (int q = 0; q < 9; ++q) D[q] = op_sub(D[q], op_mul(w, N[q]));
        if (forced) force_scaled(D, rho, fgrad, forced);
        return;
    }
    const T omc = splat<T>(__fsub_rn(1.0f, omega)), k = splat<T>(__fmul_rn(omega, 8.0f / 9.0f));
    // k folded into A and j, 4.5 into u: per direction pair (q, opp q) with kcj = k c.j and
    // cu45 = 4.5 c.u,  D' = (1 - omega) D + kA + kcj cu45 +- 3 kcj
    const T kA = op_mul(k, A), kjx = op_mul(k, jx), kjy = op_mul(k, jy);
    const T ux45 = op_mul(splat<T>(4.5f), ux), uy45 = op_mul(splat<T>(4.5f), uy);
    auto pair = [&](int qp, int qm, T kcj, T cu45) {
        const T t = op_fma(kcj, cu45, kA);
        D[qp] = op_fma(omc, D[qp], op_fma(splat<T>(3.0f), kcj, t));
        D[qm] = op_fma(omc, D[qm], op_fma(splat<T>(-3.0f), kcj, t));
    };
    pair(D05, D14, kjx, ux45);
    pair(D08, D17, kjy, uy45);
    pair(D03, D10, op_add(kjx, kjy), op_add(ux45, uy45));
    pair(D01, D12, op_sub(kjx, kjy), op_sub(ux45, uy45));
    D[D19] = op_fma(omc, D[D19], kA);
    if (forced) force_scaled(D, rho, fgrad, forced);
}

// Smagorinsky rate of one cell from p2 = |P|^2 (SRC/col_MC.F90:178-248, as les_omega):
// 1 / (1 / (2 omega) + sqrt(18 cte_s^2 |P| + 1 / omega^2) / 2)
// The square roots come from the hardware reciprocal square root (about one ulp): the 16-bit
// kinds store to three or four decimal digits.
__device__ __forceinline__ float les_sqrt(float x) { return x > 0.0f ? __fmul_rn(x, rsqrtf(x)) : 0.0f; }
__device__ __forceinline__ float les_rate1(float p2, float omega, float cte_s)
{
    const float r = __fdividef(1.0f, omega);
    const float a = __fmul_rn(__fmul_rn(18.0f, __fmul_rn(cte_s, cte_s)), les_sqrt(p2));
    const float ts = __fmaf_rn(0.5f, r, __fmul_rn(0.5f, les_sqrt(__fmaf_rn(r, r, a))));
    return __fdividef(1.0f, ts);
}
template <> __device__ __forceinline__ float les_rate<float>(float p2, float omega, float cte_s)
{
    return les_rate1(p2, omega, cte_s);
}
template <> __device__ __forceinline__ F2 les_rate<F2>(F2 p2, float omega, float cte_s)
{
    float lo, hi;
    f2_unpack(p2, lo, hi);
    return f2_pack(les_rate1(lo, omega, cte_s), les_rate1(hi, omega, cte_s));
}

// collision on unscaled deviations in compute kind K, for any storage kind
template <typename S, typename K, int CV = 0>
__device__ __forceinline__ void collide_stored(K (&v)[9], K omega, K fgrad, int forced, K cte_s)
{
    if constexpr (Is16<S>::value) {
        static_assert((CV & CV_NOSHIFT) == 0, "the 16-bit kinds store scaled deviations only");
        float D[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) D[q] = (float)v[q] * scale_of(q);  // exact: powers of two
        collide_scaled<float, (CV & CV_LES) != 0>(D, (float)omega, (float)fgrad, forced, (float)cte_s);
#pragma unroll
        for (int q = 0; q < 9; ++q) v[q] = (K)(D[q] * (1.0f / scale_of(q)));
    } else {
        collide<K, CV>(v, omega, fgrad, forced, cte_s);
    }
}

// equilibrium deviation of the outflow ghost (rho = 1, local u): bcond.inflow.F90:80-99; the
// equilibrium itself (cte1 = 1, bcond.inflow.F90:48-52) for populations stored whole
template <typename K>
__device__ __forceinline__ K outflow_eq(int q, K a01, K a03, K a05, K a08, K a10, K a12, K a14, K a17, bool noshift)
{
    const K rhoinv = (K)1, crho = (K)1, cte1 = noshift ? (K)1 : (K)0, rf = (K)3, qf = (K)1.5;
    const K p1 = (K)(1.0 / 9.0), p2 = (K)(1.0 / 36.0);
    K xj = (((a03 - a12) + (a01 - a10)) + (a05 - a14)) * rhoinv;
    K yj = (((a03 - a01) + (a12 - a10)) + (a08 - a17)) * rhoinv;
    K cvsq = xj * xj + yj * yj;
    if (q == D10) {
        K c = rf * (-xj - yj) + qf * (((K)3 * (xj + yj)) * (xj + yj) - cvsq);
        return (crho * p2) * (cte1 + c);
    } else if (q == D12) {
        K c = rf * (-xj + yj) + qf * (((K)3 * (xj - yj)) * (xj - yj) - cvsq);
        return (crho * p2) * (cte1 + c);
    } else {
        K c = rf * (-xj) + qf * (((K)3 * (xj)) * (xj) - cvsq);
        return (crho * p1) * (cte1 + c);
    }
}

// value rounded through the storage kind of plane q (a ghost value lives in storage)
template <typename S, typename K>
__device__ __forceinline__ K rnd(int q, K v)
{
    if constexpr (Is16<S>::value) return (K)(Store<S>::raw_get(S((float)v * scale_of(q))) * (1.0f / scale_of(q)));
    else return Store<S>::template getq<K>(Store<S>::template putq<K>(v, q), q);
}

template <typename S, typename K>
__device__ __forceinline__ K ldq(const S *plane, int64_t i, int q) { return Store<S>::template getq<K>(plane[i], q); }

// 16-byte vector access
template <typename S> union V16 {
    uint4 u;
    S s[16 / sizeof(S)];
};

template <typename S>
__device__ __forceinline__ void ldv(const S *p, S (&o)[16 / sizeof(S)])
{
    V16<S> t;
    t.u = __ldg(reinterpret_cast<const uint4 *>(p));
#pragma unroll
    for (int c = 0; c < 16 / (int)sizeof(S); ++c) o[c] = t.s[c];
}
template <typename S>
__device__ __forceinline__ void stv(S *p, const S (&v)[16 / sizeof(S)])
{
    V16<S> t;
#pragma unroll
    for (int c = 0; c < 16 / (int)sizeof(S); ++c) t.s[c] = v[c];
    *reinterpret_cast<uint4 *>(p) = t.u;
}

// N consecutive elements, N * sizeof(S) = 8 or 16 bytes
template <typename S, int N> struct VecT;
template <typename S> struct VecT<S, 16 / sizeof(S)> {
    using U = uint4;
};
template <typename S> struct VecT<S, 8 / sizeof(S)> {
    using U = uint2;
};
template <typename S, int N>
__device__ __forceinline__ void ldn(const S *p, S (&o)[N])
{
    using U = typename VecT<S, N>::U;
    union { U u; S s[N]; } t;
    t.u = __ldg(reinterpret_cast<const U *>(p));
#pragma unroll
    for (int c = 0; c < N; ++c) o[c] = t.s[c];
}
template <typename S, int N>
__device__ __forceinline__ void stn(S *p, const S (&v)[N])
{
    using U = typename VecT<S, N>::U;
    union { U u; S s[N]; } t;
#pragma unroll
    for (int c = 0; c < N; ++c) t.s[c] = v[c];
    *reinterpret_cast<U *>(p) = t.u;
}

template <typename K>
__device__ __forceinline__ K shfl_up(K v, int w) { return __shfl_up_sync(0xffffffffu, v, 1, w); }
template <typename K>
__device__ __forceinline__ K shfl_down(K v, int w) { return __shfl_down_sync(0xffffffffu, v, 1, w); }

// Load N consecutive values of direction q pulled from (x - c_q): an aligned 8- or 16-byte load
// of row y - cy at the thread's own columns; for a +-1 column shift, one scalar load of the
// element beside the vector (it sits in the neighbouring lane's vector, so it comes from L1).
template <typename S, typename K, int q, bool RAW = false, int N = vec_of<S>()>
__device__ __forceinline__ void pull_vec(const Lattice &L, const S *plane, int xv, int y, bool loads,
                                         K (&out)[N])
{
    auto cvt = [](S v) -> K {
        if constexpr (RAW) return (K)Store<S>::raw_get(v);
        else return Store<S>::template get<K, q>(v);
    };
    constexpr int sx = -cx_of(q), sy = -cy_of(q);
    const int64_t idx = cell_index<S>(L, xv, y + sy);
    S v[N];
    if (loads) ldn<S, N>(plane + idx, v);
    else {
#pragma unroll
        for (int c = 0; c < N; ++c) v[c] = S(0.0f);
    }
    K kv[N];
#pragma unroll
    for (int c = 0; c < N; ++c) kv[c] = cvt(v[c]);
    if (sx == 0) {
#pragma unroll
        for (int c = 0; c < N; ++c) out[c] = kv[c];
    } else if (sx == -1) {
        out[0] = loads ? cvt(plane[idx - 1]) : K(0);
#pragma unroll
        for (int c = 1; c < N; ++c) out[c] = kv[c - 1];
    } else {
#pragma unroll
        for (int c = 0; c < N - 1; ++c) out[c] = kv[c + 1];
        out[N - 1] = loads ? cvt(plane[idx + N]) : K(0);
    }
}

// ---------------------------------------------------------------------------------------------
// Boundary rules for one pulled value.  (sx, sy) is the source of direction q for cell (x, y).
// The y-face rule is applied first and wins at corners, as the reference's y-loop runs after
// its x-loop (e.g. SRC/bcond.driven.F90:100-108 then :136-143).  With L.corner_x (the merged
// loop of SRC/bcond.driven.F90:43-81, whose x-wall statements of j = m come last at the two
// upper corners) the x-face rule wins instead; both faces are walls there.
//   plane_of(q, cx, cy): element holding the value of direction q "at" (cx, cy) in the
//   current state; own(q): the pulling cell's own post-collision value of direction q.
// ---------------------------------------------------------------------------------------------
template <typename S, typename K, bool HAS_OBS, typename PlaneAt, typename Own, typename Ghost>
__device__ __forceinline__ K pull_rule(const Lattice &L, int q, int x, int y, PlaneAt plane_at, Own own,
                                       Ghost ghost_xhi)
{
    int sx = x - cx_of(q), sy = y - cy_of(q);
    const int l = L.lx, m = L.ly;
    const int oq = opp_of(q);
    if (HAS_OBS && step_bounce(L, x, y, q)) return own(oq);
    if ((sy < 1 || sy > m) && !(L.corner_x && (sx < 1 || sx > l))) {
        const int f = sy < 1 ? YLO : YHI;
        if (L.faces[f] == FK_PERIODIC) {
            sy = (sy < 1) ? m : 1;
        } else {
            K v = own(oq);
            const K wt = (K)L.wt[f][q];
            return wt != (K)0 ? rnd<S, K>(q, v + wt) : v;
        }
    }
    if (sx < 1 || sx > l) {
        const int f = sx < 1 ? XLO : XHI;
        const int kind = L.faces[f];
        if (kind == FK_PERIODIC) {
            sx = (sx < 1) ? l : 1;
        } else if (kind == FK_WALL || (HAS_OBS && kind == FK_INFLOW && sy < L.inflow_y0)) {
            // below the inflow rows of a backward-facing step (a case with obstacle cells, the
            // step's block) the x_lo face is the step's wall
            K v = own(oq);
            const K wt = (K)L.wt[f][q];
            return wt != (K)0 ? rnd<S, K>(q, v + wt) : v;
        } else if (kind == FK_INFLOW) {
            // directions 01, 03, 05 enter through x_lo
            const int t = (q == D01) ? 0 : (q == D03) ? 1 : 2;
            return rnd<S, K>(q, (K)L.inflow[(int64_t)t * (m + 2) + sy]);
        } else {
            return ghost_xhi(q, sy);
        }
    }
    if (HAS_OBS) {
        if (obs_bit(L, sx, sy)) return own(oq);
    }
    return plane_at(q, sx, sy);
}

// relax N cells in place: x[q][c] holds direction q of cell c (scaled 16-bit units when RAW)
template <typename S, typename K, bool RAW, int N = vec_of<S>(), int CV = 0>
__device__ __forceinline__ void relax_vec(K (&x)[9][N], K omega, K fgrad, int forced, K cte_s)
{
    if constexpr (RAW) {
        // two cells per packed FP32 instruction
        static_assert(N % 2 == 0, "16-bit vectors hold an even number of cells");
        static_assert((CV & CV_NOSHIFT) == 0, "the 16-bit kinds store scaled deviations only");
#pragma unroll
        for (int c = 0; c < N; c += 2) {
            F2 v[9];
#pragma unroll
            for (int q = 0; q < 9; ++q) v[q] = f2_pack(x[q][c], x[q][c + 1]);
            collide_scaled<F2, (CV & CV_LES) != 0>(v, (float)omega, (float)fgrad, forced, (float)cte_s);
#pragma unroll
            for (int q = 0; q < 9; ++q) f2_unpack(v[q], x[q][c], x[q][c + 1]);
        }
    } else {
#pragma unroll
        for (int c = 0; c < N; ++c) {
            K v[9];
#pragma unroll
            for (int q = 0; q < 9; ++q) v[q] = x[q][c];
            collide<K, CV>(v, omega, fgrad, forced, cte_s);
#pragma unroll
            for (int q = 0; q < 9; ++q) x[q][c] = v[q];
        }
    }
}

// store N values of direction q as one 8- or 16-byte vector
template <typename S, typename K, int q, bool RAW, int N = vec_of<S>()>
__device__ __forceinline__ void store_vec(S *p, const K (&v)[N], const uint32_t (&rh)[npair<N>()])
{
    if constexpr (RAW) {
        // stochastic rounding of each pair of cells with a direction-dependent rotation of the
        // pair's hash word rh[j]
        if constexpr (N == 8) {
            uint4 u;
            u.x = Store<S>::pack2_rs((float)v[0], (float)v[1], pair_bits<q>(rh[0]));
            u.y = Store<S>::pack2_rs((float)v[2], (float)v[3], pair_bits<q>(rh[1]));
            u.z = Store<S>::pack2_rs((float)v[4], (float)v[5], pair_bits<q>(rh[2]));
            u.w = Store<S>::pack2_rs((float)v[6], (float)v[7], pair_bits<q>(rh[3]));
            *reinterpret_cast<uint4 *>(p) = u;
        } else {
            uint2 u;
            u.x = Store<S>::pack2_rs((float)v[0], (float)v[1], pair_bits<q>(rh[0]));
            u.y = Store<S>::pack2_rs((float)v[2], (float)v[3], pair_bits<q>(rh[1]));
            *reinterpret_cast<uint2 *>(p) = u;
        }
    } else {
        S o[N];
#pragma unroll
        for (int c = 0; c < N; ++c) o[c] = Store<S>::template put<K, q>(v[c]);
        stn<S, N>(p, o);
    }
}

// ---------------------------------------------------------------------------------------------
// Ping-pong kernel
// ---------------------------------------------------------------------------------------------
// Cell whose pull crosses the domain boundary or touches an obstacle: the boundary rules decide
// at least one of its nine inputs.
template <bool HAS_OBS>
__device__ __forceinline__ bool needs_rule(const Lattice &L, int x, int y)
{
    if (x == 1 || x == L.lx || y == 1 || y == L.ly) return true;
    if (HAS_OBS) {
        // the corner of a backward-facing step and its neighbours: step_bounce pulls and pushes
        if (L.step_x > 0 && abs(x - L.step_x) <= 1 && abs(y - L.step_y) <= 1) return true;
        if (y >= L.ob_y0 && y <= L.ob_y1 && x >= L.ob_x0 && x <= L.ob_x1) {
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx)
                    if ((dx | dy) != 0 && obs_bit(L, x + dx, y + dy)) return true;
        }
    }
    return false;
}

// one cell with the boundary rules: reads the source buffer only, writes the destination
template <typename S, typename K, bool HAS_OBS, int CV = 0, bool COLLIDE = true>
__device__ void pp_cell_slow(const Lattice &L, const S *src, S *dst, int x, int y)
{
    const int64_t pe = L.plane_elems;
    const int64_t me = cell_index<S>(L, x, y);
    auto plane_at = [&](int q, int sx, int sy) -> K { return ldq<S, K>(src + q * pe, cell_index<S>(L, sx, sy), q); };
    auto own = [&](int q) -> K { return ldq<S, K>(src + q * pe, me, q); };
    auto ghost_xhi = [&](int q, int sy) -> K {
        const int l = L.lx;
        if (L.faces[XHI] == FK_OUTFLOW_ZG) return plane_at(q, l, sy);
        const int64_t i = cell_index<S>(L, l, sy);
        K a[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = ldq<S, K>(src + k * pe, i, k);
        return rnd<S, K>(q, outflow_eq<K>(q, a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], L.noshift != 0));
    };
    K v[9];
#pragma unroll 1
    for (int q = 0; q < 8; ++q) v[q] = pull_rule<S, K, HAS_OBS>(L, q, x, y, plane_at, own, ghost_xhi);
    v[8] = ldq<S, K>(src + D19 * pe, me, D19);
    if constexpr (COLLIDE) collide_stored<S, K, CV>(v, lat_omega<K>(L), lat_fgrad<K>(L), L.forced, lat_cte_s<K>(L));
#pragma unroll
    for (int q = 0; q < 9; ++q) dst[q * pe + me] = Store<S>::template putq<K>(v[q], q);
}

// First (x = 1, LOW) or last (x = lx) cell of a row in rows 2..ly-1 away from obstacles: only the
// three inputs that come from the x ghost column need the boundary rules; they replace the
// vector-loaded values in place (position C of the thread's N cells, scaled when RAW).
template <typename S, typename K, bool HAS_OBS, bool RAW, bool LOW, int N>
__device__ __forceinline__ void pp_edge_pull(const Lattice &L, const S *src, int x, int y, int C, K (&v)[9][N])
{
    const int64_t pe = L.plane_elems;
    const int64_t me = cell_index<S>(L, x, y);
    auto plane_at = [&](int q, int sx, int sy) -> K { return ldq<S, K>(src + q * pe, cell_index<S>(L, sx, sy), q); };
    auto own = [&](int q) -> K { return ldq<S, K>(src + q * pe, me, q); };
    auto ghost_xhi = [&](int q, int sy) -> K {
        const int l = L.lx;
        if (L.faces[XHI] == FK_OUTFLOW_ZG) return plane_at(q, l, sy);
        const int64_t i = cell_index<S>(L, l, sy);
        K a[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = ldq<S, K>(src + k * pe, i, k);
        return rnd<S, K>(q, outflow_eq<K>(q, a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], L.noshift != 0));
    };
    constexpr int q0 = LOW ? D01 : D10, q1 = LOW ? D03 : D12, q2 = LOW ? D05 : D14;
    const K a = pull_rule<S, K, HAS_OBS>(L, q0, x, y, plane_at, own, ghost_xhi);
    const K b = pull_rule<S, K, HAS_OBS>(L, q1, x, y, plane_at, own, ghost_xhi);
    const K c = pull_rule<S, K, HAS_OBS>(L, q2, x, y, plane_at, own, ghost_xhi);
    const K as = RAW ? (K)((float)a * scale_of(q0)) : a;
    const K bs = RAW ? (K)((float)b * scale_of(q1)) : b;
    const K cs = RAW ? (K)((float)c * scale_of(q2)) : c;
#pragma unroll
    for (int i = 0; i < N; ++i) {  // a select per position, so v stays in registers
        if (i == C) {
            v[q0][i] = as;
            v[q1][i] = bs;
            v[q2][i] = cs;
        }
    }
}

// Edge cells of a row that take the in-place rules of pp_edge_pull: x = 1 and x = lx of rows
// 2..ly-1 outside the obstacle zone, whatever the vector width, so that every tile shape
// computes and rounds them alike.  Returns whether cell x qualifies.
template <bool HAS_OBS>
__device__ __forceinline__ bool edge_cell(const Lattice &L, int x, int y)
{
    if (y == 1 || y == L.ly) return false;
    if (HAS_OBS && y >= L.ob_y0 && y <= L.ob_y1 && x >= L.ob_x0 && x <= L.ob_x1) return false;
    return true;
}

// one tile of TXV*VEC x TY cells at tile coordinates (bx, by) of lattice L.  Every lane takes the
// vector path; cells whose inputs come from the boundary rules are then recomputed one by one
// and overwritten (the source buffer is read-only during the step, so the recompute sees the
// same inputs).
template <typename S, typename K, int TXV, int TY, bool HAS_OBS, int N = vec_of<S>(), int CV = 0,
          bool COLLIDE = true>
__device__ __forceinline__ void pp_tile(const Lattice &L, const int bx, const int by, const int parity)
{
    const int nv = (L.lx + N - 1) / N;
    const int tx = threadIdx.x;
    const int k = bx * TXV + tx;
    const int y = by * TY + threadIdx.y + 1;
    static_assert(TXV % 32 == 0, "a warp covers one row segment");
    constexpr bool RAW = Is16<S>::value;
    const bool in_rows = y <= L.ly;
    // 16-bit kinds: whole warps past the last row leave, and lanes past the row end load the
    // last vector (their values are not used) instead of predicating the loads
    if (RAW && !in_rows) return;
    const bool loads = RAW || (in_rows && k <= nv);
    const bool active = in_rows && k < nv;
    const int xv = 1 + k * N;
    const int xl = RAW ? 1 + min(k, nv) * N : xv;
    const int64_t pe = L.plane_elems;
    S *base = reinterpret_cast<S *>(L.planes);
    const S *src = base + (parity ? 9 : 0) * pe;
    S *dst = base + (parity ? 0 : 9) * pe;

    K x[9][N];
    pull_vec<S, K, D01, RAW, N>(L, src + D01 * pe, xl, y, loads, x[D01]);
    pull_vec<S, K, D03, RAW, N>(L, src + D03 * pe, xl, y, loads, x[D03]);
    pull_vec<S, K, D05, RAW, N>(L, src + D05 * pe, xl, y, loads, x[D05]);
    pull_vec<S, K, D08, RAW, N>(L, src + D08 * pe, xl, y, loads, x[D08]);
    pull_vec<S, K, D10, RAW, N>(L, src + D10 * pe, xl, y, loads, x[D10]);
    pull_vec<S, K, D12, RAW, N>(L, src + D12 * pe, xl, y, loads, x[D12]);
    pull_vec<S, K, D14, RAW, N>(L, src + D14 * pe, xl, y, loads, x[D14]);
    pull_vec<S, K, D17, RAW, N>(L, src + D17 * pe, xl, y, loads, x[D17]);
    pull_vec<S, K, D19, RAW, N>(L, src + D19 * pe, xl, y, loads, x[D19]);
    if (!active) return;

    const bool rowb = (y == 1) || (y == L.ly);
    bool obsz = false;
    if (HAS_OBS) obsz = y >= L.ob_y0 && y <= L.ob_y1 && xv + N - 1 >= L.ob_x0 && xv <= L.ob_x1;
    // 16-bit kinds: the row's end cell at any position of the last vector (edge_cell), so that
    // every tile shape rounds it alike; the exact kinds give the same result either way and keep
    // the in-place rules to a last vector that ends at lx.
    const bool left_cell = RAW ? k == 0 && edge_cell<HAS_OBS>(L, 1, y) : !rowb && !obsz && k == 0 && nv > 1;
    const bool right_cell = RAW ? k == nv - 1 && edge_cell<HAS_OBS>(L, L.lx, y)
                                : !rowb && !obsz && k == nv - 1 && nv > 1 && (L.lx % N) == 0;
    if (left_cell) pp_edge_pull<S, K, HAS_OBS, RAW, true, N>(L, src, xv, y, 0, x);
    if (right_cell)
        pp_edge_pull<S, K, HAS_OBS, RAW, false, N>(L, src, RAW ? L.lx : xv + N - 1, y, RAW ? L.lx - xv : N - 1, x);

    if constexpr (COLLIDE) relax_vec<S, K, RAW, N, CV>(x, lat_omega<K>(L), lat_fgrad<K>(L), L.forced, lat_cte_s<K>(L));
    const int64_t me = cell_index<S>(L, xv, y);
    uint32_t rh[npair<N>()] = {};
#pragma unroll
    for (int j = 0; j < N / 2; ++j)
        rh[j] = RAW ? cell_hash((uint32_t)me + 2 * j, (float)x[D19][2 * j]) : 0u;
    store_vec<S, K, D01, RAW, N>(dst + D01 * pe + me, x[D01], rh);
    store_vec<S, K, D03, RAW, N>(dst + D03 * pe + me, x[D03], rh);
    store_vec<S, K, D05, RAW, N>(dst + D05 * pe + me, x[D05], rh);
    store_vec<S, K, D08, RAW, N>(dst + D08 * pe + me, x[D08], rh);
    store_vec<S, K, D10, RAW, N>(dst + D10 * pe + me, x[D10], rh);
    store_vec<S, K, D12, RAW, N>(dst + D12 * pe + me, x[D12], rh);
    store_vec<S, K, D14, RAW, N>(dst + D14 * pe + me, x[D14], rh);
    store_vec<S, K, D17, RAW, N>(dst + D17 * pe + me, x[D17], rh);
    store_vec<S, K, D19, RAW, N>(dst + D19 * pe + me, x[D19], rh);

    const bool rules = rowb || obsz || (k == 0 && !left_cell) || (k == nv - 1 && !right_cell);
    if (rules) {
        const int xe = min(xv + N - 1, L.lx);
#pragma unroll 1
        for (int xc = xv; xc <= xe; ++xc)
            if (needs_rule<HAS_OBS>(L, xc, y) && !(RAW && ((xc == 1 && left_cell) || (xc == L.lx && right_cell))))
                pp_cell_slow<S, K, HAS_OBS, CV, COLLIDE>(L, src, dst, xc, y);
    }
}

// Bulk prefetch into L2 of the source segments of the block L.pf_ahead places further on in
// launch order (one row of one plane per thread, 9 * TY threads): by the time that block runs,
// its loads hit L2 instead of HBM.  Which plane and row a direction reads: ping-pong, plane q of
// the source buffer at row y - c_q.y; AA P step, plane opp(q) at row y - c_q.y; AA L step, plane q
// at row y.
enum PrefetchKind { PF_PP = 0, PF_AA_P = 1, PF_AA_L = 2 };

// segment of thread t (< 9 * TY) of tile (bx, by) of lattice L
template <typename S, int TXV, int TY, int N, int KIND>
__device__ __forceinline__ void prefetch_segment(const Lattice &L, const int parity, const int t, const int bx,
                                                 const int by)
{
    constexpr int VEC = vec_of<S>();
    const int q = t % 9, y = by * TY + t / 9 + 1;
    if (y > L.ly) return;
    const int row = KIND == PF_AA_L ? y : y - cy_of(q);
    const int plane = KIND == PF_PP ? (parity ? 9 : 0) + q : KIND == PF_AA_P ? opp_of(q) : q;
    const int x0 = 1 + bx * TXV * N;
    const int x1 = min(x0 + TXV * N, L.lx + 1);
    const int64_t rs = (int64_t)row * L.pitch;
    const int64_t lo = (cell_index<S>(L, x0 - 1, row) - rs) / VEC * VEC;
    const int64_t hi = min((int64_t)L.pitch, (cell_index<S>(L, x1, row) - rs) / VEC * VEC + VEC);
    const S *p = reinterpret_cast<const S *>(L.planes) + plane * L.plane_elems + rs + lo;
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"((uint32_t)((hi - lo) * sizeof(S))) : "memory");
}

template <typename S, int TXV, int TY, int N, int KIND>
__device__ __forceinline__ void prefetch_tile(const Lattice &L, const int parity)
{
    const int t = threadIdx.x + threadIdx.y * TXV;
    if (t >= 9 * TY) return;
    const long long lin = (long long)blockIdx.y * gridDim.x + blockIdx.x + L.pf_ahead;
    if (lin >= (long long)gridDim.x * gridDim.y) return;
    prefetch_segment<S, TXV, TY, N, KIND>(L, parity, t, (int)(lin % gridDim.x),
                                          tile_row((int)(lin / gridDim.x), (int)gridDim.y));
}

// COLLIDE = false: the streaming half of the two-pass form (SRC/movef.F90 with the boundary
// rules folded in, the rest population copied); the collision then runs in col_kernel.
template <typename S, typename K, int TXV, int TY, bool HAS_OBS, int N, int CV = 0, bool COLLIDE = true>
__global__ void __launch_bounds__(TXV *TY, TXV * TY != 128 ? 1 : (N * sizeof(S) <= 8 || (sizeof(S) == 4 && N == 4)) ? 8 : (sizeof(S) == 2 ? 4 : 1)) pp_kernel(const Lattice L, const int parity)
{
    if (L.pf_ahead > 0) prefetch_tile<S, TXV, TY, N, PF_PP>(L, parity);
    pp_tile<S, K, TXV, TY, HAS_OBS, N, CV, COLLIDE>(L, blockIdx.x, tile_row(blockIdx.y, gridDim.y), parity);
}

// The Smagorinsky ping-pong step of the 16-bit kinds with an explicit register budget (MINB
// resident blocks of 128 threads per SM): its collision holds more live values than the plain
// one, and the best split between registers and occupancy is chosen by timing.
template <typename S, typename K, bool HAS_OBS, int N, int MINB>
__global__ void __launch_bounds__(128, MINB) pp_les_kernel(const Lattice L, const int parity)
{
    if (L.pf_ahead > 0) prefetch_tile<S, 128, 1, N, PF_PP>(L, parity);
    pp_tile<S, K, 128, 1, HAS_OBS, N, CV_LES>(L, blockIdx.x, tile_row(blockIdx.y, gridDim.y), parity);
}

// Persistent ping-pong step over many lattices.  The work list holds (lattice, tile x, tile y)
// sorted by lattice; block b takes the contiguous chunk b of it and copies a lattice's
// descriptor to shared memory only when the lattice changes.  Lattice i uses buffer
// cur[i] ^ parity.
template <typename S, typename K, int TXV, int TY, int N>
__global__ void __launch_bounds__(TXV *TY, TXV * TY != 128 ? 1 : (N * sizeof(S) <= 8 || (sizeof(S) == 4 && N == 4)) ? 8 : (sizeof(S) == 2 ? 4 : 1))
    batch_pp_kernel(const Lattice *__restrict__ lats, const int *__restrict__ cur, const int4 *__restrict__ tiles,
                    const int ntiles, const int parity)
{
    __shared__ Lattice sL;
    constexpr int NW = (int)(sizeof(Lattice) / sizeof(int));
    const int tid = threadIdx.y * TXV + threadIdx.x;
    const int per = (ntiles + gridDim.x - 1) / gridDim.x;
    const int t0 = blockIdx.x * per, t1 = min(ntiles, t0 + per);
    int dom = -1, par = 0;
    for (int t = t0; t < t1; ++t) {
        const int4 tile = __ldg(tiles + t);
        if (tile.x != dom) {
            __syncthreads();
            const int *srcw = reinterpret_cast<const int *>(lats + tile.x);
            int *dstw = reinterpret_cast<int *>(&sL);
            for (int i = tid; i < NW; i += TXV * TY) dstw[i] = __ldg(srcw + i);
            __syncthreads();
            dom = tile.x;
            par = __ldg(cur + dom) ^ parity;
        }
        pp_tile<S, K, TXV, TY, true, N>(sL, tile.y, tile.z, par);
    }
}

// ---------------------------------------------------------------------------------------------
// AA kernels
// ---------------------------------------------------------------------------------------------

// Where the value of direction q pushed by (x, y) is needed next, and what it must be.
// Returns false when the push leaves the domain through a face that absorbs it.
template <typename S, typename K, bool HAS_OBS>
__device__ __forceinline__ void aa_push_rule(const Lattice &L, S *base, int q, int x, int y, K g)
{
    const int64_t pe = L.plane_elems;
    const int l = L.lx, m = L.ly;
    int tx = x + cx_of(q), ty = y + cy_of(q);
    const int oq = opp_of(q);
    const S gs = Store<S>::template putq<K>(g, q);
    // the reference adds the wall term to the stored value (SRC/bcond.driven.F90:141-143)
    const K gr = Store<S>::template getq<K>(gs, q);
    if ((ty < 1 || ty > m) && !(L.corner_x && (tx < 1 || tx > l))) {
        const int f = ty < 1 ? YLO : YHI;
        if (L.faces[f] == FK_PERIODIC) {
            ty = (ty < 1) ? m : 1;
        } else {
            base[q * pe + cell_index<S>(L, tx, ty)] = gs;  // raw value kept in the ghost frame
            const K wt = (K)L.wt[f][oq];
            const S b = wt != (K)0 ? Store<S>::template putq<K>(gr + wt, oq) : Store<S>::template putq<K>(gr, oq);
            base[oq * pe + cell_index<S>(L, x, y)] = b;
            return;
        }
    }
    if (tx < 1 || tx > l) {
        const int f = tx < 1 ? XLO : XHI;
        const int kind = L.faces[f];
        if (kind == FK_PERIODIC) {
            tx = (tx < 1) ? l : 1;
        } else {
            base[q * pe + cell_index<S>(L, tx, ty)] = gs;
            // below the inflow rows of a backward-facing step the x_lo face is the step's wall
            if (kind == FK_WALL || (HAS_OBS && kind == FK_INFLOW && ty < L.inflow_y0)) {
                const K wt = (K)L.wt[f][oq];
                const S b = wt != (K)0 ? Store<S>::template putq<K>(gr + wt, oq) : Store<S>::template putq<K>(gr, oq);
                base[oq * pe + cell_index<S>(L, x, y)] = b;
            }
            return;
        }
    }
    if (HAS_OBS) {
        // backward-facing step (step_bounce).  A target whose input q is the bounce-back of its
        // own opposite population takes nothing from this push: the slot keeps the target's own
        // phase-0 value, which the target pulls in this step (pull_rule), and no other cell
        // touches it; the pushed value goes to L.step_aux[5..9] instead, where the readers of the
        // phase-1 state find it (post_value).  The cell whose input oq is such a bounce-back
        // keeps the value of this push in L.step_aux[0..4], where its next (local) step reads it
        // (aa_l_kernel): its own slot oq belongs to the neighbour x - c_oq during this step.
        S *aux = reinterpret_cast<S *>(L.step_aux);
        if (step_bounce(L, x, y, oq)) aux[step_slot(L, x, oq)] = gs;
        if (step_bounce(L, tx, ty, q)) {
            aux[5 + step_slot(L, tx, q)] = gs;
            return;
        }
        if (obs_bit(L, tx, ty)) {
            base[oq * pe + cell_index<S>(L, x, y)] = Store<S>::template putq<K>(gr, oq);
            return;
        }
    }
    base[q * pe + cell_index<S>(L, tx, ty)] = gs;
}

// values entering (x, y) next step from an x_lo inflow or x_hi outflow ghost (the cells that
// own those slots write them); g holds the post-collision values of (x, y), already rounded
// through storage.
template <typename S, typename K>
__device__ __forceinline__ void aa_incoming(const Lattice &L, S *base, int x, int y, const K (&g)[9])
{
    const int64_t pe = L.plane_elems;
    const int l = L.lx, m = L.ly;
    if (x == 1 && L.faces[XLO] == FK_INFLOW) {
#pragma unroll
        for (int t = 0; t < 3; ++t) {
            const int q = t == 0 ? D01 : t == 1 ? D03 : D05;
            int sy = y - cy_of(q);
            if (sy < 1 || sy > m) {
                if (L.faces[sy < 1 ? YLO : YHI] != FK_PERIODIC) continue;  // bounced instead
                sy = sy < 1 ? m : 1;
            }
            if (sy < L.inflow_y0) continue;  // the step's wall below the inflow rows: bounced instead
            base[q * pe + cell_index<S>(L, x, y)] =
                Store<S>::template putq<K>((K)L.inflow[(int64_t)t * (m + 2) + sy], q);
        }
    }
    if (x == l && (L.faces[XHI] == FK_OUTFLOW_EQ || L.faces[XHI] == FK_OUTFLOW_ZG)) {
        // cell (l, y) supplies direction q of cell (l, y + cy_q) for q = 10, 12, 14
#pragma unroll
        for (int t = 0; t < 3; ++t) {
            const int q = t == 0 ? D10 : t == 1 ? D12 : D14;
            int ty = y + cy_of(q);
            if (ty < 1 || ty > m) {
                if (L.faces[ty < 1 ? YLO : YHI] != FK_PERIODIC) continue;
                ty = ty < 1 ? m : 1;
            }
            K v = (L.faces[XHI] == FK_OUTFLOW_ZG)
                      ? g[q]
                      : outflow_eq<K>(q, g[0], g[1], g[2], g[3], g[4], g[5], g[6], g[7], L.noshift != 0);
            base[q * pe + cell_index<S>(L, l, ty)] = Store<S>::template putq<K>(v, q);
        }
    }
}

// Phase-0 ghost column x = lx+1 for outflow faces: value of direction q (10,12,14) at
// (lx+1, y), stored in plane opp(q), computed from cell (lx, y)'s post-collision values.
template <typename S, typename K>
__device__ __forceinline__ void aa_outflow_ghost(const Lattice &L, S *base, int y, const K (&g)[9])
{
    const int64_t pe = L.plane_elems;
    const int l = L.lx;
#pragma unroll
    for (int t = 0; t < 3; ++t) {
        const int q = t == 0 ? D10 : t == 1 ? D12 : D14;
        K v = (L.faces[XHI] == FK_OUTFLOW_ZG) ? g[q]
                                              : outflow_eq<K>(q, g[0], g[1], g[2], g[3], g[4], g[5], g[6], g[7], L.noshift != 0);
        base[opp_of(q) * pe + cell_index<S>(L, l + 1, y)] = Store<S>::template putq<K>(v, q);
    }
}

template <typename S, typename K, bool HAS_OBS, int CV = 0>
__device__ void aa_p_cell_slow(const Lattice &L, S *base, int x, int y)
{
    const int64_t pe = L.plane_elems;
    const int64_t me = cell_index<S>(L, x, y);
    if (HAS_OBS) {
        if (obs_bit(L, x, y)) return;  // obstacle interiors are not advanced by the AA scheme
    }
    // phase 0: f*_q(c) is in plane opp(q) at c
    auto plane_at = [&](int q, int sx, int sy) -> K {
        const int oq = opp_of(q);
        return ldq<S, K>(base + oq * pe, cell_index<S>(L, sx, sy), q);
    };
    auto own = [&](int q) -> K { return ldq<S, K>(base + opp_of(q) * pe, me, q); };
    auto ghost_xhi = [&](int q, int sy) -> K { return plane_at(q, L.lx + 1, sy); };
    K v[9];
#pragma unroll 1
    for (int q = 0; q < 8; ++q) v[q] = pull_rule<S, K, HAS_OBS>(L, q, x, y, plane_at, own, ghost_xhi);
    v[8] = ldq<S, K>(base + D19 * pe, me, D19);
    collide_stored<S, K, CV>(v, lat_omega<K>(L), lat_fgrad<K>(L), L.forced, lat_cte_s<K>(L));
#pragma unroll 1
    for (int q = 0; q < 8; ++q) aa_push_rule<S, K, HAS_OBS>(L, base, q, x, y, v[q]);
    base[D19 * pe + me] = Store<S>::template putq<K>(v[8], D19);
    K g[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) g[q] = rnd<S, K>(q, v[q]);
    aa_incoming<S, K>(L, base, x, y, g);
}

// First/last cell of a row in the AA P step, handled inside the vector path (rows 2..ly-1,
// no obstacle nearby): only the x-face rules apply.  Before the collision the three inputs that
// come from the x ghost column are replaced; after the vector push the three pushes that leave
// through the x face are redone with the push rules, and the incoming inflow/outflow values
// are written.  C is the cell's position in the lane's vector.
template <typename S, typename K, bool HAS_OBS, bool RAW, int C, bool LOW, int N>
__device__ __forceinline__ void aa_edge_pull(const Lattice &L, const S *base, int x, int y, K (&v)[9][N])
{
    const int64_t pe = L.plane_elems;
    const int64_t me = cell_index<S>(L, x, y);
    auto plane_at = [&](int q, int sx, int sy) -> K {
        return ldq<S, K>(base + opp_of(q) * pe, cell_index<S>(L, sx, sy), q);
    };
    auto own = [&](int q) -> K { return ldq<S, K>(base + opp_of(q) * pe, me, q); };
    auto ghost_xhi = [&](int q, int sy) -> K { return plane_at(q, L.lx + 1, sy); };
    constexpr int q0 = LOW ? D01 : D10, q1 = LOW ? D03 : D12, q2 = LOW ? D05 : D14;
    const K a = pull_rule<S, K, HAS_OBS>(L, q0, x, y, plane_at, own, ghost_xhi);
    const K b = pull_rule<S, K, HAS_OBS>(L, q1, x, y, plane_at, own, ghost_xhi);
    const K c = pull_rule<S, K, HAS_OBS>(L, q2, x, y, plane_at, own, ghost_xhi);
    v[q0][C] = RAW ? (K)((float)a * scale_of(q0)) : a;
    v[q1][C] = RAW ? (K)((float)b * scale_of(q1)) : b;
    v[q2][C] = RAW ? (K)((float)c * scale_of(q2)) : c;
}

template <typename S, typename K, bool HAS_OBS, bool RAW, int C, bool LOW, int N>
__device__ __forceinline__ void aa_edge_push(const Lattice &L, S *base, int x, int y, const K (&v)[9][N])
{
    K g[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) g[q] = RAW ? (K)((float)v[q][C] * (1.0f / scale_of(q))) : v[q][C];
    constexpr int q0 = LOW ? D10 : D01, q1 = LOW ? D12 : D03, q2 = LOW ? D14 : D05;
    aa_push_rule<S, K, HAS_OBS>(L, base, q0, x, y, g[q0]);
    aa_push_rule<S, K, HAS_OBS>(L, base, q1, x, y, g[q1]);
    aa_push_rule<S, K, HAS_OBS>(L, base, q2, x, y, g[q2]);
    K gr[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) gr[q] = rnd<S, K>(q, g[q]);
    aa_incoming<S, K>(L, base, x, y, gr);
}

// push N values of direction q to (x + c_q) in plane q; lanes at an edge (segment end or a
// neighbour on the slow path) store the elements that cross into the neighbour's vector.
// 16-bit kinds (RAW) round the shifted vector in pairs, as it is stored, with the lane's pair
// hash words `rh`; lone elements at an edge use the lone-value rounding.
template <typename S, typename K, int q, int W, bool RAW, int N>
__device__ __forceinline__ void push_vec(const Lattice &L, S *plane, int xv, int y, bool left_edge,
                                         bool right_edge, const K (&g)[N], bool store,
                                         const uint32_t (&rh)[npair<N>()])
{
    constexpr int cx = cx_of(q), cy = cy_of(q);
    const int64_t idx = cell_index<S>(L, xv, y + cy);
    auto cvt = [](K v) -> S {
        if constexpr (RAW) return Store<S>::raw_put((float)v);
        else return Store<S>::template put<K, q>(v);
    };
    if constexpr (RAW) {
        static_assert(N == 4 || N == 8, "16-bit vectors hold 4 or 8 elements");
        K sh[N];  // the vector as stored at idx
        if (cx == 0) {
#pragma unroll
            for (int c = 0; c < N; ++c) sh[c] = g[c];
        } else if (cx == 1) {
            sh[0] = shfl_up(g[N - 1], W);
#pragma unroll
            for (int c = 1; c < N; ++c) sh[c] = g[c - 1];
        } else {
#pragma unroll
            for (int c = 0; c < N - 1; ++c) sh[c] = g[c + 1];
            sh[N - 1] = shfl_down(g[0], W);
        }
        // Every lane rounds its shifted vector in pairs.  A lane at an edge stores only the part
        // of it that it owns (the element from the neighbouring lane is missing or belongs to a
        // slow neighbour): halves and words of the same rounded pairs, as predicated stores, so
        // the warp runs no divergent branch here.  The one element that crosses into the next
        // segment is rounded alone.
        using U = typename VecT<S, N>::U;
        union { U u; uint32_t w[N / 2]; } t;
#pragma unroll
        for (int j = 0; j < N / 2; ++j)
            t.w[j] = Store<S>::pack2_rs((float)sh[2 * j], (float)sh[2 * j + 1], pair_bits<q>(rh[j]));
        const bool full = cx == 0 || (cx == 1 ? !left_edge : !right_edge);
        if (store && full) *reinterpret_cast<U *>(plane + idx) = t.u;
        if constexpr (cx == 1) {
            // owned: elements 1 .. N-1 of the vector at idx
            if (store && left_edge) {
                reinterpret_cast<uint16_t *>(plane)[idx + 1] = (uint16_t)(t.w[0] >> 16);
                reinterpret_cast<uint32_t *>(plane + idx + 2)[0] = t.w[1];
                if constexpr (N == 8) *reinterpret_cast<uint2 *>(plane + idx + 4) = make_uint2(t.w[2], t.w[3]);
            }
            if (store && right_edge) plane[idx + N] = cvt(g[N - 1]);
        } else if constexpr (cx == -1) {
            // owned: elements 0 .. N-2 of the vector at idx
            if (store && right_edge) {
                if constexpr (N == 8) {
                    *reinterpret_cast<uint2 *>(plane + idx) = make_uint2(t.w[0], t.w[1]);
                    reinterpret_cast<uint32_t *>(plane + idx + 4)[0] = t.w[2];
                } else {
                    reinterpret_cast<uint32_t *>(plane + idx)[0] = t.w[0];
                }
                reinterpret_cast<uint16_t *>(plane)[idx + N - 2] = (uint16_t)(t.w[N / 2 - 1] & 0xffffu);
            }
            if (store && left_edge) plane[idx - 1] = cvt(g[0]);
        }
    } else {
        S s[N];
#pragma unroll
        for (int c = 0; c < N; ++c) s[c] = cvt(g[c]);
        if (cx == 0) {
            if (store) stn<S, N>(plane + idx, s);
        } else if (cx == 1) {
            K fl = shfl_up(g[N - 1], W);
            if (!store) return;
            if (!left_edge) {
                S v[N];
                v[0] = cvt(fl);
#pragma unroll
                for (int c = 1; c < N; ++c) v[c] = s[c - 1];
                stn<S, N>(plane + idx, v);
            } else {
#pragma unroll
                for (int c = 0; c < N - 1; ++c) plane[idx + 1 + c] = s[c];
            }
            if (right_edge) plane[idx + N] = s[N - 1];
        } else {
            K fr = shfl_down(g[0], W);
            if (!store) return;
            if (!right_edge) {
                S v[N];
#pragma unroll
                for (int c = 0; c < N - 1; ++c) v[c] = s[c + 1];
                v[N - 1] = cvt(fr);
                stn<S, N>(plane + idx, v);
            } else {
#pragma unroll
                for (int c = 1; c < N; ++c) plane[idx - 1 + c] = s[c];
            }
            if (left_edge) plane[idx - 1] = s[0];
        }
    }
}

template <typename S, typename K, int TXV, int TY, bool HAS_OBS, int CV = 0, int N = vec_of<S>()>
__global__ void __launch_bounds__(TXV *TY, TXV * TY != 128 ? 1 : (N * sizeof(S) <= 8 ? 8 : (sizeof(S) == 2 ? 4 : 1)))
    aa_p_kernel(const Lattice L)
{
    constexpr int VEC = N;  // cells per thread
    constexpr int W = TXV < 32 ? TXV : 32;
    if (L.pf_ahead > 0) prefetch_tile<S, TXV, TY, VEC, PF_AA_P>(L, 0);
    const int nv = (L.lx + VEC - 1) / VEC;
    const int tx = threadIdx.x;
    const int k = blockIdx.x * TXV + tx;
    const int y = tile_row(blockIdx.y, gridDim.y) * TY + threadIdx.y + 1;
    static_assert(TXV % 32 == 0, "a warp covers one row segment");
    constexpr bool RAW = Is16<S>::value;
    const bool in_rows = y <= L.ly;
    if (RAW && !in_rows) return;  // as in pp_tile
    const bool loads = RAW || (in_rows && k <= nv);
    const bool active = in_rows && k < nv;
    const int xv = 1 + k * VEC;
    const int xl = RAW ? 1 + min(k, nv) * VEC : xv;
    const int64_t pe = L.plane_elems;
    S *base = reinterpret_cast<S *>(L.planes);

    // pull f*_q from plane opp(q) at x - c_q
    K x[9][VEC];
    pull_vec<S, K, D01, RAW, VEC>(L, base + D12 * pe, xl, y, loads, x[D01]);
    pull_vec<S, K, D03, RAW, VEC>(L, base + D10 * pe, xl, y, loads, x[D03]);
    pull_vec<S, K, D05, RAW, VEC>(L, base + D14 * pe, xl, y, loads, x[D05]);
    pull_vec<S, K, D08, RAW, VEC>(L, base + D17 * pe, xl, y, loads, x[D08]);
    pull_vec<S, K, D10, RAW, VEC>(L, base + D03 * pe, xl, y, loads, x[D10]);
    pull_vec<S, K, D12, RAW, VEC>(L, base + D01 * pe, xl, y, loads, x[D12]);
    pull_vec<S, K, D14, RAW, VEC>(L, base + D05 * pe, xl, y, loads, x[D14]);
    pull_vec<S, K, D17, RAW, VEC>(L, base + D08 * pe, xl, y, loads, x[D17]);
    pull_vec<S, K, D19, RAW, VEC>(L, base + D19 * pe, xl, y, loads, x[D19]);

    // lanes on the scalar path: boundary rows, a ragged row end, obstacle surroundings
    bool slow = (y == 1) || (y == L.ly) || (nv == 1) || (k == nv - 1 && (L.lx % VEC) != 0);
    if (HAS_OBS) slow = slow || (y >= L.ob_y0 && y <= L.ob_y1 && xv + VEC - 1 >= L.ob_x0 && xv <= L.ob_x1);
    slow = slow || !active;
    const bool left_cell = !slow && k == 0;             // x = 1 is element 0
    const bool right_cell = !slow && k == nv - 1;       // x = lx is element VEC-1
    if (left_cell) aa_edge_pull<S, K, HAS_OBS, RAW, 0, true, VEC>(L, base, xv, y, x);
    if (right_cell) aa_edge_pull<S, K, HAS_OBS, RAW, VEC - 1, false, VEC>(L, base, xv + VEC - 1, y, x);
    // neighbours on the slow path do not take part in the vector stores
    const bool left_slow = __shfl_up_sync(0xffffffffu, slow ? 1 : 0, 1, W) != 0;
    const bool right_slow = __shfl_down_sync(0xffffffffu, slow ? 1 : 0, 1, W) != 0;
    const bool left_edge = (tx % W) == 0 || left_slow;
    const bool right_edge = (tx % W) == W - 1 || right_slow;

    relax_vec<S, K, RAW, VEC, CV>(x, lat_omega<K>(L), lat_fgrad<K>(L), L.forced, lat_cte_s<K>(L));
    K (&g)[9][VEC] = x;
    const bool store = !slow;
    uint32_t rh[npair<VEC>()] = {};
    const uint32_t me = (uint32_t)cell_index<S>(L, xv, y);
#pragma unroll
    for (int j = 0; j < VEC / 2; ++j) rh[j] = RAW ? cell_hash(me + 2 * j, (float)g[D19][2 * j]) : 0u;
    push_vec<S, K, D01, W, RAW, VEC>(L, base + D01 * pe, xv, y, left_edge, right_edge, g[D01], store, rh);
    push_vec<S, K, D03, W, RAW, VEC>(L, base + D03 * pe, xv, y, left_edge, right_edge, g[D03], store, rh);
    push_vec<S, K, D05, W, RAW, VEC>(L, base + D05 * pe, xv, y, left_edge, right_edge, g[D05], store, rh);
    push_vec<S, K, D08, W, RAW, VEC>(L, base + D08 * pe, xv, y, left_edge, right_edge, g[D08], store, rh);
    push_vec<S, K, D10, W, RAW, VEC>(L, base + D10 * pe, xv, y, left_edge, right_edge, g[D10], store, rh);
    push_vec<S, K, D12, W, RAW, VEC>(L, base + D12 * pe, xv, y, left_edge, right_edge, g[D12], store, rh);
    push_vec<S, K, D14, W, RAW, VEC>(L, base + D14 * pe, xv, y, left_edge, right_edge, g[D14], store, rh);
    push_vec<S, K, D17, W, RAW, VEC>(L, base + D17 * pe, xv, y, left_edge, right_edge, g[D17], store, rh);
    push_vec<S, K, D19, W, RAW, VEC>(L, base + D19 * pe, xv, y, left_edge, right_edge, g[D19], store, rh);
    if (left_cell) aa_edge_push<S, K, HAS_OBS, RAW, 0, true, VEC>(L, base, xv, y, g);
    if (right_cell) aa_edge_push<S, K, HAS_OBS, RAW, VEC - 1, false, VEC>(L, base, xv + VEC - 1, y, g);
    if (!active || !slow) return;
    const int xe = min(xv + VEC - 1, L.lx);
#pragma unroll 1
    for (int xc = xv; xc <= xe; ++xc) aa_p_cell_slow<S, K, HAS_OBS, CV>(L, base, xc, y);
}

// L step: local collision, phase 1 -> 0
template <typename S, typename K, int TXV, int TY, bool HAS_OBS, int CV = 0, int N = vec_of<S>()>
__global__ void __launch_bounds__(TXV *TY, TXV * TY != 128 ? 1 : (N * sizeof(S) <= 8 ? 8 : (sizeof(S) == 2 ? 4 : 1)))
    aa_l_kernel(const Lattice L)
{
    constexpr int VEC = N;  // cells per thread
    if (L.pf_ahead > 0) prefetch_tile<S, TXV, TY, VEC, PF_AA_L>(L, 0);
    const int nv = (L.lx + VEC - 1) / VEC;
    const int k = blockIdx.x * TXV + threadIdx.x;
    const int y = tile_row(blockIdx.y, gridDim.y) * TY + threadIdx.y + 1;
    if (y > L.ly || k >= nv) return;
    const int xv = 1 + k * VEC;
    const int64_t pe = L.plane_elems;
    S *base = reinterpret_cast<S *>(L.planes);
    const int64_t me = cell_index<S>(L, xv, y);
    const bool outflow = L.faces[XHI] == FK_OUTFLOW_EQ || L.faces[XHI] == FK_OUTFLOW_ZG;
    bool slow = (k == nv - 1) && ((L.lx % VEC) != 0 || outflow);
    if (HAS_OBS) slow = slow || (y >= L.ob_y0 && y <= L.ob_y1 && xv + VEC - 1 >= L.ob_x0 && xv <= L.ob_x1);
    const K omega = lat_omega<K>(L), fgrad = lat_fgrad<K>(L);
    const int forced = L.forced;
    if (slow) {
        const int xe = min(xv + VEC - 1, L.lx);
#pragma unroll 1
        for (int xc = xv; xc <= xe; ++xc) {
            const int64_t i = cell_index<S>(L, xc, y);
            if (HAS_OBS) {
                if (obs_bit(L, xc, y)) continue;
            }
            K v[9];
#pragma unroll
            for (int q = 0; q < 9; ++q) v[q] = ldq<S, K>(base + q * pe, i, q);
            if (HAS_OBS && L.step_x > 0) {
                // backward-facing step: an input that is the bounce-back of the cell's own opposite
                // population comes from L.step_aux, where the previous step's push kept it
                // (aa_push_rule); the cell's own slot for it was left unwritten
#pragma unroll 1
                for (int q = 0; q < 8; ++q)
                    if (step_bounce(L, xc, y, q))
                        v[q] = Store<S>::template getq<K>(reinterpret_cast<const S *>(L.step_aux)[step_slot(L, xc, q)], q);
            }
            collide_stored<S, K, CV>(v, omega, fgrad, forced, lat_cte_s<K>(L));
            K g[9];
#pragma unroll
            for (int q = 0; q < 9; ++q) {
                const S s = Store<S>::template putq<K>(v[q], q);
                base[opp_of(q) * pe + i] = s;
                g[q] = Store<S>::template getq<K>(s, q);
            }
            if (xc == L.lx && outflow) aa_outflow_ghost<S, K>(L, base, y, g);
        }
        return;
    }
    constexpr bool RAW = Is16<S>::value;
    K x[9][VEC];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        S v[VEC];
        ldn<S, VEC>(base + q * pe + me, v);
#pragma unroll
        for (int c = 0; c < VEC; ++c) {
            if constexpr (RAW) x[q][c] = (K)Store<S>::raw_get(v[c]);
            else x[q][c] = Store<S>::template getq<K>(v[c], q);
        }
    }
    relax_vec<S, K, RAW, VEC, CV>(x, omega, fgrad, forced, lat_cte_s<K>(L));
    uint32_t rh[npair<VEC>()] = {};
#pragma unroll
    for (int j = 0; j < VEC / 2; ++j)
        rh[j] = RAW ? cell_hash((uint32_t)me + 2 * j, (float)x[D19][2 * j]) : 0u;
    store_vec<S, K, D01, RAW, VEC>(base + D12 * pe + me, x[D01], rh);
    store_vec<S, K, D03, RAW, VEC>(base + D10 * pe + me, x[D03], rh);
    store_vec<S, K, D05, RAW, VEC>(base + D14 * pe + me, x[D05], rh);
    store_vec<S, K, D08, RAW, VEC>(base + D17 * pe + me, x[D08], rh);
    store_vec<S, K, D10, RAW, VEC>(base + D03 * pe + me, x[D10], rh);
    store_vec<S, K, D12, RAW, VEC>(base + D01 * pe + me, x[D12], rh);
    store_vec<S, K, D14, RAW, VEC>(base + D05 * pe + me, x[D14], rh);
    store_vec<S, K, D17, RAW, VEC>(base + D08 * pe + me, x[D17], rh);
    store_vec<S, K, D19, RAW, VEC>(base + D19 * pe + me, x[D19], rh);
}

// One block per work-list tile (the hardware schedules the blocks); the lattice descriptor is
// read through the read-only cache.
template <typename S, typename K, int TXV, int TY, int N>
__global__ void __launch_bounds__(TXV *TY, TXV * TY != 128 ? 1 : (N * sizeof(S) <= 8 || (sizeof(S) == 4 && N == 4)) ? 8 : (sizeof(S) == 2 ? 4 : 1))
    batch_pp_flat_kernel(const Lattice *__restrict__ lats, const int *__restrict__ cur, const int4 *__restrict__ tiles,
                         const int ntiles, const int parity, const int pf)
{
    if (pf > 0) {  // L2 prefetch of the work-list entry pf places ahead (see prefetch_tile)
        const int t = threadIdx.x + threadIdx.y * TXV;
        const int ahead = blockIdx.x + pf;
        if (t < 9 * TY && ahead < ntiles) {
            const int4 ta = __ldg(tiles + ahead);
            prefetch_segment<S, TXV, TY, N, PF_PP>(lats[ta.x], __ldg(cur + ta.x) ^ parity, t, ta.y, ta.z);
        }
    }
    const int4 tile = __ldg(tiles + blockIdx.x);
    const Lattice &L = lats[tile.x];
    pp_tile<S, K, TXV, TY, true, N>(L, tile.y, tile.z, __ldg(cur + tile.x) ^ parity);
}

// Batch members with the Smagorinsky collision: one block of 128 x 1 threads per work-list entry,
// the tile of the single-domain LES step (N cells per thread).
template <typename S, typename K, int N>
__global__ void __launch_bounds__(128, (N * sizeof(S) <= 8 || (sizeof(S) == 4 && N == 4)) ? 8 : (sizeof(S) == 2 ? 4 : 1))
    batch_les_kernel(const Lattice *__restrict__ lats, const int *__restrict__ cur, const int4 *__restrict__ tiles,
                     const int parity)
{
    const int4 tile = __ldg(tiles + blockIdx.x);
    pp_tile<S, K, 128, 1, true, N, CV_LES>(lats[tile.x], tile.y, tile.z, __ldg(cur + tile.x) ^ parity);
}

// Collision half of the two-pass form (SRC/col.F90): every interior cell of buffer `parity`
// relaxes in place, obstacle cells included, as the reference's col loop does.
template <typename S, typename K, int TXV, int TY, int N, int CV = 0>
__global__ void __launch_bounds__(TXV *TY, TXV * TY != 128 ? 1 : (N * sizeof(S) <= 8 || (sizeof(S) == 4 && N == 4)) ? 8 : (sizeof(S) == 2 ? 4 : 1))
    col_kernel(const Lattice L, const int parity)
{
    const int nv = (L.lx + N - 1) / N;
    const int k = blockIdx.x * TXV + threadIdx.x;
    const int y = tile_row(blockIdx.y, gridDim.y) * TY + threadIdx.y + 1;
    if (y > L.ly || k >= nv) return;
    const int xv = 1 + k * N;
    const int64_t pe = L.plane_elems;
    S *base = reinterpret_cast<S *>(L.planes) + (parity ? 9 : 0) * pe;
    const int64_t me = cell_index<S>(L, xv, y);
    const K omega = lat_omega<K>(L), fgrad = lat_fgrad<K>(L);
    const int forced = L.forced;
    if (k == nv - 1 && (L.lx % N) != 0) {  // ragged row end: the cells up to lx one by one
        const int xe = L.lx;
#pragma unroll 1
        for (int xc = xv; xc <= xe; ++xc) {
            const int64_t i = cell_index<S>(L, xc, y);
            K v[9];
#pragma unroll
            for (int q = 0; q < 9; ++q) v[q] = ldq<S, K>(base + q * pe, i, q);
            collide_stored<S, K, CV>(v, omega, fgrad, forced, lat_cte_s<K>(L));
#pragma unroll
            for (int q = 0; q < 9; ++q) base[q * pe + i] = Store<S>::template putq<K>(v[q], q);
        }
        return;
    }
    constexpr bool RAW = Is16<S>::value;
    K x[9][N];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        S v[N];
        ldn<S, N>(base + q * pe + me, v);
#pragma unroll
        for (int c = 0; c < N; ++c) {
            if constexpr (RAW) x[q][c] = (K)Store<S>::raw_get(v[c]);
            else x[q][c] = Store<S>::template getq<K>(v[c], q);
        }
    }
    relax_vec<S, K, RAW, N, CV>(x, omega, fgrad, forced, lat_cte_s<K>(L));
    uint32_t rh[npair<N>()] = {};
#pragma unroll
    for (int j = 0; j < N / 2; ++j) rh[j] = RAW ? cell_hash((uint32_t)me + 2 * j, (float)x[D19][2 * j]) : 0u;
    store_vec<S, K, D01, RAW, N>(base + D01 * pe + me, x[D01], rh);
    store_vec<S, K, D03, RAW, N>(base + D03 * pe + me, x[D03], rh);
    store_vec<S, K, D05, RAW, N>(base + D05 * pe + me, x[D05], rh);
    store_vec<S, K, D08, RAW, N>(base + D08 * pe + me, x[D08], rh);
    store_vec<S, K, D10, RAW, N>(base + D10 * pe + me, x[D10], rh);
    store_vec<S, K, D12, RAW, N>(base + D12 * pe + me, x[D12], rh);
    store_vec<S, K, D14, RAW, N>(base + D14 * pe + me, x[D14], rh);
    store_vec<S, K, D17, RAW, N>(base + D17 * pe + me, x[D17], rh);
    store_vec<S, K, D19, RAW, N>(base + D19 * pe + me, x[D19], rh);
}

}  // namespace bgk
