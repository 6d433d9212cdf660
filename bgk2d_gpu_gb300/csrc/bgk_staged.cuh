// bgk_staged.cuh -- ping-pong step with the source rows staged in shared memory by bulk async
// copies (the TMA engine).  Written for the 16-bit storage kinds, whose threads hold too few bytes
// of loads in flight to cover the HBM latency; instantiated for every kind.
//
// A block owns a band of BW = T * N columns and a stripe of consecutive rows.  Output row y needs
// row y - c_q.y of plane q for the nine directions, columns x0 - 1 .. x0 + BW: per row one
// contiguous, 16-byte aligned segment of each plane (one vector of halo on each side).  STAGES
// rows of segments are in flight at a time as `cp.async.bulk` copies (completion counted in bytes
// on one mbarrier per stage), so the HBM latency is covered by copies in flight rather than by
// registers held in loads.  The threads read their cells from shared memory, relax them with the
// same code as pp_tile and store straight to HBM; the last warp to finish reading a row issues
// the copies of the row STAGES further on into the same stage, so no warp waits for another.
// The launch gives each block a stripe of STAGES rows (step_staged), so all its copies go out
// at once and the refill path serves only longer stripes.  The result is identical to pp_tile:
// the same arithmetic per cell, the same hash words for the stochastic rounding, and the same
// boundary-rule recomputation from the source buffer afterwards.
//
// Every wait on an mbarrier is bounded (0.5 s).  When a wait runs out, the warp sets the lattice's status
// word and leaves the row loop; the other warps then run out too (nobody refills the stage they
// wait for), and the block waits (bounded again) for its own copies still in flight before it
// returns.  The host reads the status word at the next synchronisation, and later launches return
// at once while it is set.
#pragma once

#include "bgk_kernels.cuh"

namespace bgk {

constexpr uint64_t STAGED_WAIT_NS = 500000000ull;  // a wait gives up after 0.5 s (global timer)
constexpr uint32_t STAGED_WAIT_POLLS = 1u << 26;    // and after this many polls in any case
constexpr uint32_t STAGED_TIMEOUT = 0x5747u;        // status word value written on a timeout

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// bulk copy of `bytes` (multiple of 16, both addresses 16-byte aligned) from global to shared,
// completing on `bar`
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// bounded wait for the phase with parity `par` of `bar` to complete: false after 0.5 s
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t par)
{
    const uint32_t a = smem_u32(bar);
    uint64_t t0 = 0;
    for (uint32_t i = 0; i < STAGED_WAIT_POLLS; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(par)
            : "memory");
        if (done) return true;
        if ((i & 63u) == 63u) {
            const uint64_t t = global_ns();
            if (t0 == 0) t0 = t;
            else if (t - t0 > STAGED_WAIT_NS) return false;
        }
    }
    return false;
}

// Shared-memory bytes of one block: STAGES x 9 segments of BW + 2 VEC elements, then the barriers.
template <typename S, int T, int N, int STAGES>
__host__ __device__ constexpr int staged_seg_elems() { return T * N + 2 * vec_of<S>(); }
template <typename S, int T, int N, int STAGES>
__host__ __device__ constexpr size_t staged_smem_bytes()
{
    return (size_t)STAGES * 9 * staged_seg_elems<S, T, N, STAGES>() * sizeof(S) + (size_t)STAGES * sizeof(uint64_t);
}

// direction q of the thread's N cells from the staged segment of plane q (index i0 = first cell)
template <typename S, typename K, int q, bool RAW, int N>
__device__ __forceinline__ void pull_staged(const S *seg, int i0, K (&out)[N])
{
    auto cvt = [](S v) -> K {
        if constexpr (RAW) return (K)Store<S>::raw_get(v);
        else return Store<S>::template get<K, q>(v);
    };
    using U = typename VecT<S, N>::U;
    union { U u; S s[N]; } t;
    t.u = *reinterpret_cast<const U *>(seg + i0);
    K kv[N];
#pragma unroll
    for (int c = 0; c < N; ++c) kv[c] = cvt(t.s[c]);
    constexpr int sx = -cx_of(q);
    if (sx == 0) {
#pragma unroll
        for (int c = 0; c < N; ++c) out[c] = kv[c];
    } else if (sx == -1) {
        out[0] = cvt(seg[i0 - 1]);
#pragma unroll
        for (int c = 1; c < N; ++c) out[c] = kv[c - 1];
    } else {
#pragma unroll
        for (int c = 0; c < N - 1; ++c) out[c] = kv[c + 1];
        out[N - 1] = cvt(seg[i0 + N]);
    }
}

// Grid: (bands, stripes); block b.x covers columns 1 + b.x * BW .., block b.y rows
// 1 + b.y * rows .. min(ly, (b.y + 1) * rows).  CV: the collision variant.  MINB > 0 sets
// the blocks per SM that the register budget is sized for (the shared-memory stages bound the
// residency anyway, so the eddy-viscosity collision can take the registers it needs).
template <typename S, typename K, int T, int N, int STAGES, bool HAS_OBS, int CV = 0, int MINB = 0>
__global__ void __launch_bounds__(T, MINB > 0 ? MINB : ((N * sizeof(S) <= 8) ? 1024 : 512) / T)
    pp_staged_kernel(const Lattice L, const int parity, const int rows)
{
    constexpr int VEC = vec_of<S>();
    constexpr int BW = T * N;
    constexpr int SEG = staged_seg_elems<S, T, N, STAGES>();
    constexpr bool RAW = Is16<S>::value;
    extern __shared__ __align__(128) unsigned char staged_smem[];
    S *segs = reinterpret_cast<S *>(staged_smem);
    uint64_t *full = reinterpret_cast<uint64_t *>(staged_smem + (size_t)STAGES * 9 * SEG * sizeof(S));

    const int t = threadIdx.x;
    const int band = blockIdx.x;
    const int ya = 1 + tile_row(blockIdx.y, gridDim.y) * rows;  // the last stripe runs second
    const int yb = min(L.ly, ya + rows - 1);  // inclusive
    if (ya > L.ly) return;
    const int64_t pe = L.plane_elems;
    S *base = reinterpret_cast<S *>(L.planes);
    const S *src = base + (parity ? 9 : 0) * pe;
    S *dst = base + (parity ? 0 : 9) * pe;

    // segment of a row: elements band*BW .. band*BW + SEG - 1 (cells x0 - VEC .. x0 + BW + VEC - 1),
    // clipped to the row (the clipped part holds no cell of this band)
    const int e0 = band * BW;
    const int len = min(SEG, L.pitch - e0);
    const uint32_t row_bytes = (uint32_t)len * (uint32_t)sizeof(S);

    __shared__ int cnt[STAGES];   // warps done with the row now in each stage
    __shared__ int uses[STAGES];  // rows issued into each stage so far
    auto issue = [&](int y, int s) {
        uses[s] += 1;
        // (a test hook declares 16 bytes that never arrive, so that the waits run out)
        mbar_expect_tx(&full[s], 9u * row_bytes + (L.inject_stall ? 16u : 0u));
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            const int ry = y - cy_of(q);
            bulk_g2s(segs + (size_t)(s * 9 + q) * SEG, src + q * pe + (int64_t)ry * L.pitch + e0, row_bytes, &full[s]);
        }
    };

    __shared__ int skip;  // an earlier step already failed: the whole block returns
    if (t == 0) {
        skip = L.status && *(volatile uint32_t *)L.status != 0;
        if (!skip) {
            for (int s = 0; s < STAGES; ++s) {
                mbar_init(&full[s], 1);
                cnt[s] = 0;
                uses[s] = 0;
            }
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
            for (int s = 0; s < STAGES && ya + s <= yb; ++s) issue(ya + s, s);
        }
    }
    __syncthreads();
    if (skip) return;

    const int nv = (L.lx + N - 1) / N;
    const int k = band * T + t;
    const bool active = k < nv;
    const int xv = 1 + k * N;
    const int i0 = VEC + t * N;  // staged index of the thread's first cell
    const K omega = lat_omega<K>(L), fgrad = lat_fgrad<K>(L), cte_s = lat_cte_s<K>(L);
    const int forced = L.forced;
    constexpr int NW = T / 32;

    // No block-wide barrier per row: each warp moves on as soon as its next row has landed, and
    // the last warp to finish a row refills that stage with the row STAGES further on.
    for (int y = ya, it = 0; y <= yb; ++y, ++it) {
        const int s = it % STAGES;
        const uint32_t par = (uint32_t)(it / STAGES) & 1u;
        if (!__all_sync(0xffffffffu, mbar_wait(&full[s], par))) {
            if (L.status) atomicExch(L.status, STAGED_TIMEOUT);
            break;  // this warp stops refilling, so the others run out too and leave the loop
        }
        const S *sg = segs + (size_t)s * 9 * SEG;
        K x[9][N];
        pull_staged<S, K, D01, RAW, N>(sg + D01 * SEG, i0, x[D01]);
        pull_staged<S, K, D03, RAW, N>(sg + D03 * SEG, i0, x[D03]);
        pull_staged<S, K, D05, RAW, N>(sg + D05 * SEG, i0, x[D05]);
        pull_staged<S, K, D08, RAW, N>(sg + D08 * SEG, i0, x[D08]);
        pull_staged<S, K, D10, RAW, N>(sg + D10 * SEG, i0, x[D10]);
        pull_staged<S, K, D12, RAW, N>(sg + D12 * SEG, i0, x[D12]);
        pull_staged<S, K, D14, RAW, N>(sg + D14 * SEG, i0, x[D14]);
        pull_staged<S, K, D17, RAW, N>(sg + D17 * SEG, i0, x[D17]);
        pull_staged<S, K, D19, RAW, N>(sg + D19 * SEG, i0, x[D19]);

        // the warp's reads of stage s are complete: count it, and the last warp refills the stage
        __syncwarp();
        if ((t & 31) == 0) {
            __threadfence_block();
            if (atomicAdd(&cnt[s], 1) == NW - 1) {
                cnt[s] = 0;  // published by the release of the next expect_tx
                if (y + STAGES <= yb) {
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    issue(y + STAGES, s);
                }
            }
        }

        if (active) {
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

            relax_vec<S, K, RAW, N, CV>(x, omega, fgrad, forced, cte_s);
            const int64_t me = cell_index<S>(L, xv, y);
            uint32_t rh[npair<N>()] = {};
#pragma unroll
            for (int j = 0; j < N / 2; ++j) rh[j] = RAW ? cell_hash((uint32_t)me + 2 * j, (float)x[D19][2 * j]) : 0u;
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
                        pp_cell_slow<S, K, HAS_OBS, CV>(L, src, dst, xc, y);
            }
        }
    }

    // no copy may still be writing this block's shared memory when it exits: after a normal
    // sweep every issued row has landed; after a timeout wait (bounded) for the last row of
    // each stage
    __syncthreads();
    if (t == 0) {
        for (int s = 0; s < STAGES; ++s)
            if (uses[s] > 0 && !mbar_wait(&full[s], (uint32_t)(uses[s] - 1) & 1u) && L.status)
                atomicExch(L.status, STAGED_TIMEOUT);
    }
}

}  // namespace bgk
