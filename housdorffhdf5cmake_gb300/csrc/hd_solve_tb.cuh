// hd_solve_tb.cuh -- temporally blocked frontier dilation: T steps per grid
// barrier (sm_103a).
//
// Same job model, queues, stamps, ping-pong buffers and barrier as
// hd_solve.cuh, but one queue item advances a brick by T dilation steps:
//
//   brick     IW = 4 words (128 voxels) in x  x  32 R - 2T rows  x  BZ
//             planes, R = tb_rows(T) rows per lane (1 in this build)
//   warp      lane = R consecutive rows: per row the 4 interior words plus
//             one halo word holding the 16 voxels on each side of them, rows
//             y0 - T .. y0 + 32 R - T - 1 (T halo rows above and below the
//             interior), streamed plane by plane along z from z0 - T to
//             z0 + BZ + T - 1
//   levels    level 0 is the loaded state; level s is the state after s
//             steps, computed one plane behind level s - 1 from three of its
//             planes; rows come from the lane's own registers and, for its
//             first and last row, from the neighbouring lanes by shuffle; x
//             carries from the neighbouring words of the row
//   staging   planes arrive by cp.async (zero fill outside the domain) in
//             a ring of shared-memory slots two planes ahead of the one
//             being computed; a plane leaves the ring after its final step
//             has been compared with it.  Per level the lane keeps the
//             pending plane's partial result and the last plane's z terms in
//             registers (3 CTAs of 4 warps per SM; 4 for 1-2 steps)
//   jobs      a launch with at most kJobCache jobs in play (a single pair, a
//             server tick with one resident request) reads them from a
//             per-CTA shared-memory copy of their first line
//
// Level s is exact on rows [s, 32 R - s) and planes [s, BZ + 2T - s) of the
// streamed block (errors from the unknown outside creep in one voxel per
// step; the halo word absorbs x for T < 16), so the interior is exact for all
// s <= T.  At every level the interior is cover-tested (hits are counted with
// step k_base + s, the distance of those voxels) and the final level is
// written to the other ping-pong buffer.
//
// Frontier rule: a brick is queued for the next iteration iff its state, or a
// neighbour's state within T voxels of their shared face, changed during this
// iteration (T steps reach no further; for edge and corner neighbours the
// flags of all the faces involved must be set).  A brick not
// queued has D^{(i+1)T} = D^{iT} on itself and its halo, so its next T steps
// change nothing and both ping-pong buffers already hold its state.
#pragma once
#include "hd_solve.cuh"

namespace hdk {

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, uint32_t src_bytes) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async4(uint32_t dst, const void* src, uint32_t src_bytes) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
// Waits until at most n groups are pending (n known at compile time after
// unrolling; counts above N wait for N, which is stricter).
template <int N>
__device__ __forceinline__ void cp_async_wait_upto(int n) {
    if constexpr (N == 0) {
        cp_async_wait<0>();
    } else {
        if (n >= N) cp_async_wait<N>();
        else cp_async_wait_upto<N - 1>(n);
    }
}

// Shared memory of one warp: ring slots of streamed planes (interior words
// as 16-byte rows, then the two halo words of each row), then the brick's
// target rows (18-neighbour element: target minus state, updated per level).
// Row k of every lane is contiguous within a slot (lane-consecutive 16-byte
// rows: conflict-free 128-bit accesses).
template <int T, int BZ>
struct TbSmem {
    static constexpr int R = tb_rows(T);    // rows per lane
    static constexpr int NP = BZ + 2 * T;  // planes streamed per brick
    static constexpr int RS = tb_ring_slots(T, BZ);
    static constexpr int PF = kTbPrefetch;  // planes in flight ahead of the one computed
    static constexpr int kInBytes = RS * R * 32 * 16;
    static constexpr int kHaloBytes = RS * R * 32 * 8;
    static constexpr int kUOff = kInBytes + kHaloBytes;
    static constexpr int kWarpBytes = kUOff + BZ * R * 32 * 16;
    static_assert(kWarpBytes == tb_warp_bytes(T, BZ), "shared layout");
    static_assert(RS >= T + 1 + PF || RS == NP, "a plane must stay until its final step");
};

// One queue item of the blocked kernel, decoded.
struct TbItem {
    const Job* Jp;
    JobState* st;
    int jid;
    unsigned epoch;
    unsigned lb;
    int iter, kb;
    int bx, by, bz;
    int active;  // the job's active flag as loaded at issue (checked when the item is computed)
    bool live;
};

// Where this lane's rows of a streamed plane come from: domain plane z, row
// y, words wx0 .. wx0 + 3 of the brick are at src + (z + zoff) * plane +
// rowoff[k] for the lane's row k (brick row R lane + k).  The level-0 state
// is the job's ping-pong buffer, except in the job's first iteration, which
// reads the source (vol[0]); the target always comes from vol[1].  Every
// row copy is one 16-byte copy: the domain layout and the packed masks (rows
// padded to a multiple of 4 words, read in place only when the domain starts
// on a multiple of 4 words) keep a brick's 4 words in its row, and those past
// the domain are row padding or outside the bounding box of A u B (zero).
template <int R>
struct TbRow {
    const uint32_t* src;
    int plane, zoff, z0, Dd;
    int rowoff[R];
    bool rowv[R], hl_ok[R], hr_ok[R];
};

template <int T, int BZ>
__device__ __forceinline__ TbRow<tb_rows(T)> tb_row(const TbItem& it, bool target) {
    constexpr int IW = 4;
    constexpr int R = tb_rows(T);
    constexpr int BYI = tb_brick_rows(T);
    const int lane = threadIdx.x & 31;
    const Job* Jp = it.Jp;
    TbRow<R> w;
    const int Wx = Jp->wx, Hd = Jp->h;
    const int wx0 = it.bx * IW;
    const bool first = target || it.iter == 0;
    const int pitch = first ? Jp->vpitch : Jp->pitch;
    const int rbase = first ? Jp->vy0 : 0;
    const int xbase = (first ? Jp->vx0 : 0) + wx0;
    w.src = first ? Jp->vol[target ? 1 : 0] : Jp->buf[it.iter & 1];
    w.plane = first ? Jp->vpitch * Jp->vh : Jp->pitch * Hd;
    w.zoff = first ? Jp->vz0 : 0;
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int y = it.by * BYI - T + lane * R + k;
        w.rowv[k] = y >= 0 && y < Hd;
        w.rowoff[k] = ((w.rowv[k] ? y : 0) + rbase) * pitch + xbase;
        w.hl_ok[k] = w.rowv[k] && wx0 > 0;
        w.hr_ok[k] = w.rowv[k] && wx0 + IW < Wx;
    }
    w.z0 = it.bz * BZ;
    w.Dd = Jp->d;
    return w;
}

// Copies streamed plane r of the brick into its ring slot (one group).
template <int T, int BZ>
__device__ __forceinline__ void tb_copy_plane(const TbRow<tb_rows(T)>& w, int r, unsigned char* wsm) {
    using SM = TbSmem<T, BZ>;
    constexpr int IW = 4;
    const int lane = threadIdx.x & 31;
    const int z = w.z0 - T + r;
    const bool zok = z >= 0 && z < w.Dd;
    const int slot = r % SM::RS;
    const uint32_t base = (uint32_t)__cvta_generic_to_shared(wsm);
#pragma unroll
    for (int k = 0; k < SM::R; ++k) {
        const bool ok = w.rowv[k] && zok;
        const uint32_t* gp = w.src + (ok ? (z + w.zoff) * w.plane + w.rowoff[k] : 0);
        const uint32_t s_in = base + (uint32_t)(((slot * SM::R + k) * 32 + lane) * 16);
        const uint32_t s_h = base + SM::kInBytes + (uint32_t)(((slot * SM::R + k) * 32 + lane) * 8);
        cp_async16(s_in, gp, ok ? 16u : 0u);
        cp_async4(s_h, (ok && w.hl_ok[k]) ? gp - 1 : gp, (ok && w.hl_ok[k]) ? 4u : 0u);
        cp_async4(s_h + 4, (ok && w.hr_ok[k]) ? gp + IW : gp, (ok && w.hr_ok[k]) ? 4u : 0u);
    }
    cp_async_commit();
}

// Decodes a queue entry and decides whether the item runs (the entry is not
// left over from a slot's previous pair, the step cap is not passed).  The
// job's active flag and every job field the item reads are loaded in one
// batch, so their latencies overlap; the flag is checked when the item is
// computed.
template <int T>
__device__ __forceinline__ bool tb_decode(const SolveParams& p, unsigned long long e, int g, const Job* jcache,
                                          TbItem& it) {
    const int lane = threadIdx.x & 31;
    it.jid = (int)((e >> 32) & kEntryJobMask);
    it.lb = (unsigned)e;
    it.epoch = (unsigned)(e >> 56);
    it.st = p.states + it.jid;
    const unsigned jc = (unsigned)(it.jid - p.job_cache_base);
    it.Jp = jc < (unsigned)p.job_cache ? jcache + jc : p.jobs + it.jid;
    it.live = false;
    const Job* Jp = it.Jp;
    // the job's active flag is only needed when the item is computed: the
    // copies do not wait for it (an item of a job that finished meanwhile is
    // dropped then, after its copies have landed)
    it.active = ld_relaxed_s32(&it.st->active);
    const uint32_t jep = Jp->epoch;
    const int k0 = Jp->k0, kmax = Jp->kmax, nbx = Jp->nbx, nby = Jp->nby;
    // one load per 32-byte sector of the job's first line, so that the
    // issue and compute phases find its fields in L1
    const int warm = (int)(size_t)Jp->vol[1] + Jp->wx + Jp->vpitch + (int)(size_t)Jp->hist;
    asm volatile("" ::"r"(warm));
    if ((jep & 0xffu) != it.epoch) return false;  // left over from the slot's previous pair
    it.iter = g - k0;
    it.kb = it.iter * T;
    if (it.kb + 1 > kmax) {
        if (lane == 0) {
            it.st->status = kErrIterLimit;
            atomicCAS(&p.ctl->err, 0, kErrIterLimit);
        }
        return false;
    }
    it.bx = (int)(it.lb % (unsigned)nbx);
    const unsigned tq = it.lb / (unsigned)nbx;
    it.by = (int)(tq % (unsigned)nby);
    it.bz = (int)(tq / (unsigned)nby);
    it.live = true;
    return true;
}

// Decodes a queue entry (tb_decode) and issues the copies of the brick's
// target rows (one group) and of its first planes (one group each).  No
// wait.
template <int T, int BZ>
__device__ __forceinline__ void tb_issue(const SolveParams& p, unsigned long long e, int g, const Job* jcache,
                                         unsigned char* wsm,
                                         TbItem& it) {
    using SM = TbSmem<T, BZ>;
    const int lane = threadIdx.x & 31;
    if (!tb_decode<T>(p, e, g, jcache, it)) return;
    {
        const TbRow<SM::R> t = tb_row<T, BZ>(it, true);
        const uint32_t s_u = (uint32_t)__cvta_generic_to_shared(wsm) + SM::kUOff;
#pragma unroll
        for (int k = 0; k < SM::R; ++k) {
            const int yr = lane * SM::R + k;  // row of the streamed block
            const bool inter = t.rowv[k] && yr >= T && yr < 32 * SM::R - T;
#pragma unroll
            for (int i = 0; i < BZ; ++i) {
                const int z = t.z0 + i;
                const bool ok = inter && z < t.Dd;
                cp_async16(s_u + (uint32_t)(((i * SM::R + k) * 32 + lane) * 16),
                           t.src + (ok ? (z + t.zoff) * t.plane + t.rowoff[k] : 0), ok ? 16u : 0u);
            }
        }
        cp_async_commit();
    }
    const TbRow<SM::R> w = tb_row<T, BZ>(it, false);
#pragma unroll
    for (int r = 0; r < SM::PF && r < SM::NP; ++r) tb_copy_plane<T, BZ>(w, r, wsm);
}

// What the epilogue of an item needs from its compute phase.
constexpr int kTbMaxSteps = 5;
constexpr unsigned kTbClaimRounds = 4;  // items per warp from which the queue's tail is claimed
struct TbOut {
    unsigned cnt[kTbMaxSteps];  // newly covered voxels per step of the item
    bool any, fxl, fxh, fyl, fyh, fzl, fzh;
    bool skip;                  // the job had finished: nothing computed, no epilogue
};

// Runs the item's T steps plane by plane, copying planes into the ring PF
// ahead (per level the pending plane's partial result and the last plane's Z
// stay in registers), and writes its state back (in the job's first
// iteration to both ping-pong buffers: a brick that is not queued for the
// next iteration must find its state in either).  The state only grows, so
// the target voxels a step covers are those in its result and not in its
// input: the 6-neighbour element finds the input plane in registers, the
// 18-neighbour element keeps target minus state per row in shared memory.
// An item whose job finished since it was issued is dropped here.
template <int T, int BZ, bool SE18>
__device__ __forceinline__ void tb_compute(const SolveParams& p, const TbItem& it, unsigned char* wsm, TbOut& res) {
    static_assert(T >= 1 && T <= kTbMaxSteps && kTbMaxSteps < 16, "steps per barrier out of range");
    constexpr int IW = 4;
    constexpr int NW = IW + 1;  // [combined halo word, 4 interior words]
    constexpr int R = tb_rows(T);
    constexpr int ROWS = 32 * R;  // rows of the streamed block
    constexpr int BYI = tb_brick_rows(T);
    using SM = TbSmem<T, BZ>;
    constexpr int NP = SM::NP;
    const int lane = threadIdx.x & 31;
    const Job* Jp = it.Jp;
    res.skip = it.active == 0;
    if (res.skip) {  // job finished: let the item's copies land (the ring is reused next) and drop it
        cp_async_wait<0>();
        return;
    }
    const TbRow<R> w = tb_row<T, BZ>(it, false);
    const int Wx = Jp->wx;
    const int wx0 = it.bx * IW;
    bool inter[R];  // the lane's rows that belong to the brick (not halo, inside the domain)
#pragma unroll
    for (int k = 0; k < R; ++k) inter[k] = w.rowv[k] && lane * R + k >= T && lane * R + k < ROWS - T;
    uint32_t* __restrict__ dst = Jp->buf[(it.iter + 1) & 1];
    uint32_t* __restrict__ dst2 = it.iter == 0 ? Jp->buf[0] : nullptr;
    const int bplane = Jp->pitch * Jp->h;
    const int brow0 = it.by * BYI - T + lane * R;  // block row of the lane's row 0
    uint32_t wmx[NW];  // valid bits of each word of a row (x only)
    {
        uint32_t w6[IW + 2];
#pragma unroll
        for (int j = 0; j < IW + 2; ++j) {
            const int x = wx0 - 1 + j;
            w6[j] = (x >= 0 && x < Wx) ? (x == Wx - 1 ? Jp->tailmask : kFull) : 0u;
        }
        wmx[0] = (w6[0] & 0xffff0000u) | (w6[IW + 1] & 0x0000ffffu);
#pragma unroll
        for (int j = 1; j <= IW; ++j) wmx[j] = w6[j];
    }

    auto plane_ok = [&](int r) {  // streamed plane index r -> inside the domain
        const int z = w.z0 - T + r;
        return z >= 0 && z < w.Dd;
    };
    auto in_row = [&](int r, int k) -> uint4 {
        return *reinterpret_cast<const uint4*>(wsm + (((r % SM::RS) * R + k) * 32 + lane) * 16);
    };
    auto halo_row = [&](int r, int k) -> uint2 {
        return *reinterpret_cast<const uint2*>(wsm + SM::kInBytes + (((r % SM::RS) * R + k) * 32 + lane) * 8);
    };
    auto u_row = [&](int i, int k) -> uint32_t* {
        return reinterpret_cast<uint32_t*>(wsm + SM::kUOff + ((i * R + k) * 32 + lane) * 16);
    };
    // In-plane terms of one level's plane: M = C | sx(C) | sy(C) [| sx(sy(C))],
    // Z = C [| sx(sy(C))]: what the plane contributes to itself and to the
    // planes above and below.
    auto terms = [&](const uint32_t (&C)[R][NW], uint32_t (&M)[R][NW], uint32_t (&Z)[R][NW]) {
        // rows: the lane's first row takes its upper neighbour from the
        // previous lane's last row, its last row the lower neighbour from the
        // next lane's first row, by shuffle; the others are in registers.
        // Lanes 0 and 31 get their own value back from the shuffle: lane 0's
        // last row (R = 1: the row itself, already in M; R = 2: the first
        // row's lower neighbour, already in Y), lane 31's first row (likewise)
        uint32_t Y[R][NW];
#pragma unroll
        for (int j = 0; j < NW; ++j) {
            const uint32_t up = __shfl_up_sync(kFull, C[R - 1][j], 1);
            const uint32_t dn = __shfl_down_sync(kFull, C[0][j], 1);
#pragma unroll
            for (int k = 0; k < R; ++k) Y[k][j] = (k == 0 ? up : C[k - 1][j]) | (k == R - 1 ? dn : C[k + 1][j]);
        }
        // x: one funnel shift per direction carries the neighbour word's
        // bit.  The words form a ring [H, I0, I1, I2, I3]: the halo word H
        // holds the left neighbour word's high half (x0 - 16 .. x0 - 1) in
        // bits 16-31 and the right neighbour word's low half (x1 + 1 ..
        // x1 + 16) in bits 0-15, so I3 is H's left and I0 its right
        // neighbour; the two halves trade bits 15 and 16, 16 voxels from the
        // interior, which T <= kTbMaxSteps (< 16) steps never carry back
#pragma unroll
        for (int k = 0; k < R; ++k) {
#pragma unroll
            for (int j = 0; j < NW; ++j) {
                const uint32_t l = C[k][(j + NW - 1) % NW], r = C[k][(j + 1) % NW];
                const uint32_t sx = __funnelshift_l(l, C[k][j], 1) | __funnelshift_r(C[k][j], r, 1);
                if constexpr (!SE18) {
                    M[k][j] = C[k][j] | sx | Y[k][j];
                    Z[k][j] = C[k][j];
                } else {
                    const uint32_t yl = Y[k][(j + NW - 1) % NW], yr = Y[k][(j + 1) % NW];
                    const uint32_t sxy = __funnelshift_l(yl, Y[k][j], 1) | __funnelshift_r(Y[k][j], yr, 1);
                    M[k][j] = C[k][j] | sx | Y[k][j] | sxy;
                    Z[k][j] = C[k][j] | sxy;
                }
            }
        }
    };

    // Per level l < T: acc = M(p) | Z(p - 1) of the pending plane p and
    // zp = Z(p); the next plane's terms complete plane p at level l + 1.
    uint32_t acc[T][R][NW], zp[T][R][NW];
    unsigned cnt[T];
#pragma unroll
    for (int s = 0; s < T; ++s) {
        cnt[s] = 0;
#pragma unroll
        for (int k = 0; k < R; ++k)
#pragma unroll
            for (int j = 0; j < NW; ++j) acc[s][k][j] = zp[s][k][j] = 0u;
    }
    uint32_t d_xl = 0, d_xh = 0, d_zl = 0, d_zh = 0, d_yl = 0, d_yh = 0, d_any = 0;
    (void)p;

#pragma unroll
    for (int q = 0; q < NP; ++q) {
        // keep PF planes in flight, then wait for plane q (groups committed
        // after it: planes q + 1 .. min(q + PF, NP - 1))
        if (q + SM::PF < NP) tb_copy_plane<T, BZ>(w, q + SM::PF, wsm);
        cp_async_wait_upto<SM::PF>((NP - 1 - q) < SM::PF ? (NP - 1 - q) : SM::PF);
        // level 0: the loaded plane q
        uint32_t M[R][NW], Z[R][NW];
        {
            // zero outside the domain already (zero-fill copies, clean tail
            // bits), so no mask here
            uint32_t C[R][NW];
#pragma unroll
            for (int k = 0; k < R; ++k) {
                const uint4 v = in_row(q, k);
                const uint2 h = halo_row(q, k);
                C[k][0] = (h.x & 0xffff0000u) | (h.y & 0x0000ffffu);
                C[k][1] = v.x;
                C[k][2] = v.y;
                C[k][3] = v.z;
                C[k][4] = v.w;
            }
            terms(C, M, Z);
        }
        // (M, Z) hold level s - 1 terms of plane q - s + 1: they complete
        // plane r = q - s at level s
#pragma unroll
        for (int s = 1; s <= T; ++s) {
            const int r = q - s;
            uint32_t out[R][NW];
            // 6-neighbour element: a plane's z term is the plane itself, so
            // zp[s - 1] holds plane r at level s - 1 until it is replaced here
            uint32_t prev[R][NW];
#pragma unroll
            for (int k = 0; k < R; ++k)
#pragma unroll
                for (int j = 0; j < NW; ++j) {
                    if constexpr (!SE18) prev[k][j] = zp[s - 1][k][j];
                    out[k][j] = acc[s - 1][k][j] | Z[k][j];
                    acc[s - 1][k][j] = M[k][j] | zp[s - 1][k][j];
                    zp[s - 1][k][j] = Z[k][j];
                }
            if (!(r >= s && r <= NP - 1 - s)) break;  // nothing complete at level s yet
            // Clip to the domain.  The 6-neighbour element needs it only at
            // the last level: the domain is a box and every shortest
            // 6-neighbour path between two of its voxels stays inside it, so
            // dilating past its faces for a few levels changes nothing inside
            // (and the target words are zero outside).  The
            // 18-neighbour element's paths can leave and re-enter a box (its
            // domain has a margin for that): it is clipped at every level,
            // like the reference's border guards.
            if (SE18 || s == T) {
                const bool pv = plane_ok(r);
#pragma unroll
                for (int k = 0; k < R; ++k)
#pragma unroll
                    for (int j = 0; j < NW; ++j) out[k][j] = (pv && w.rowv[k]) ? (out[k][j] & wmx[j]) : 0u;
            }
            if (r >= T && r < T + BZ) {
                // cover test of the interior at step kb + s (target rows of
                // non-interior rows and planes are zero).  The state only
                // grows, so the voxels step kb + s covers are the target
                // voxels in plane r at level s but not at level s - 1.
#pragma unroll
                for (int k = 0; k < R; ++k) {
                    uint32_t* ur = u_row(r - T, k);
                    uint4 u = *reinterpret_cast<const uint4*>(ur);
                    if constexpr (!SE18) {
                        u.x &= ~prev[k][1];
                        u.y &= ~prev[k][2];
                        u.z &= ~prev[k][3];
                        u.w &= ~prev[k][4];
                    } else if (s == 1) {
                        // the 18-neighbour z term is not the plane: the row keeps
                        // the uncovered target, target minus the level-0 state
                        const uint4 c0 = in_row(r, k);
                        u.x &= ~c0.x;
                        u.y &= ~c0.y;
                        u.z &= ~c0.z;
                        u.w &= ~c0.w;
                    }
                    const uint32_t h0 = out[k][1] & u.x, h1 = out[k][2] & u.y, h2 = out[k][3] & u.z,
                                   h3 = out[k][4] & u.w;
                    cnt[s - 1] += __popc(h0) + __popc(h1) + __popc(h2) + __popc(h3);
                    if constexpr (SE18) {
                        if (s < T) {  // the last level reads the row for the last time
                            u.x &= ~h0;
                            u.y &= ~h1;
                            u.z &= ~h2;
                            u.w &= ~h3;
                            *reinterpret_cast<uint4*>(ur) = u;
                        }
                    }
                }
            }
            if (s < T) {
                terms(out, M, Z);  // level s terms of plane r, for level s + 1
            } else {
                // final level: store, record changes
                const int z = w.z0 - T + r;
#pragma unroll
                for (int k = 0; k < R; ++k) {
                    if (inter[k] && z < w.Dd) {
                        const int off = z * bplane + (brow0 + k) * Jp->pitch + wx0;
                        const uint4 o4 = make_uint4(out[k][1], out[k][2], out[k][3], out[k][4]);
                        *reinterpret_cast<uint4*>(dst + off) = o4;
                        if (dst2) *reinterpret_cast<uint4*>(dst2 + off) = o4;
                        const uint4 c0 = in_row(r, k);
                        const uint32_t dx0 = out[k][1] ^ (c0.x & wmx[1]), dx3 = out[k][4] ^ (c0.w & wmx[4]);
                        const uint32_t dall = dx0 | (out[k][2] ^ (c0.y & wmx[2])) | (out[k][3] ^ (c0.z & wmx[3])) | dx3;
                        // only changes within T voxels of an x face can reach
                        // the x neighbour's interior during its next T steps
                        constexpr uint32_t kLoBits = (1u << T) - 1u, kHiBits = ~(0xffffffffu >> T);
                        const int yb = lane * R + k - T;  // row within the brick
                        d_any |= dall;
                        d_xl |= dx0 & kLoBits;
                        d_xh |= dx3 & kHiBits;
                        if (yb < T) d_yl |= dall;
                        if (yb >= BYI - T) d_yh |= dall;
                        if (r - T < T) d_zl |= dall;
                        if (r - T >= BZ - T) d_zh |= dall;
                    }
                }
            }
        }
    }

    // per-step hit counts and frontier flags
#pragma unroll
    for (int s = 0; s < T; ++s) {
        unsigned c = cnt[s];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(kFull, c, o);
        res.cnt[s] = c;
    }
    res.any = __any_sync(kFull, d_any != 0);
    res.fxl = __any_sync(kFull, d_xl != 0);
    res.fxh = __any_sync(kFull, d_xh != 0);
    res.fyl = __any_sync(kFull, d_yl != 0);
    res.fyh = __any_sync(kFull, d_yh != 0);
    res.fzl = __any_sync(kFull, d_zl != 0);
    res.fzh = __any_sync(kFull, d_zh != 0);
}

// Counts, frontier, completion.  The completion atomic's return value is
// consumed last, so its latency overlaps the frontier atomics.
template <int T, bool SE18>
__device__ __forceinline__ void tb_epilogue(const SolveParams& p, const TbItem& it, const TbOut& res, int g) {
    if (res.skip) return;
    const int lane = threadIdx.x & 31;
    const Job* Jp = it.Jp;
    JobState* st = it.st;
    unsigned long long tot = 0, left = ~0ull;
    if (lane == 0) {
#pragma unroll
        for (int s = 0; s < T; ++s) {
            if (res.cnt[s]) {
                const int k = it.kb + s + 1;
                tot += res.cnt[s];
                atomicAdd(&st->sum, (unsigned long long)k * res.cnt[s]);
                atomicMax(&st->hd, k);
                atomicAdd(&Jp->hist[k], (unsigned long long)res.cnt[s]);
            }
        }
        if (tot) left = atomicAdd(&st->remaining, (unsigned long long)(-(long long)tot));
        if (p.stats) atomicAdd(&st->bricks, 1ull);
    }
    if (res.any) {
        const int nbx = Jp->nbx, nby = Jp->nby, nbz = Jp->nbz;
        bool need = false;
        unsigned nlb = 0;
        if (lane < 27) {
            const int ox = lane % 3 - 1, oy = (lane / 3) % 3 - 1, oz = lane / 9 - 1;
            const int nnz = (ox != 0) + (oy != 0) + (oz != 0);
            need = SE18 || T > 1 || nnz <= 1;
            if (ox < 0) need = need && res.fxl;
            if (ox > 0) need = need && res.fxh;
            if (oy < 0) need = need && res.fyl;
            if (oy > 0) need = need && res.fyh;
            if (oz < 0) need = need && res.fzl;
            if (oz > 0) need = need && res.fzh;
            const int nx = it.bx + ox, ny = it.by + oy, nz = it.bz + oz;
            need = need && nx >= 0 && nx < nbx && ny >= 0 && ny < nby && nz >= 0 && nz < nbz;
            if (need) {
                nlb = (unsigned)((nz * nby + ny) * nbx + nx);
                need = atomicMax(&p.stamps[Jp->brick0 + nlb], g + 1) < g + 1;
            }
        }
        const unsigned m = __ballot_sync(kFull, need);
        if (m) {
            const int qn = (g + 1) % 3;
            unsigned long long* qdst = qn == 0 ? p.queue[0] : (qn == 1 ? p.queue[1] : p.queue[2]);
            unsigned base = 0;
            if (lane == 0) base = atomicAdd(&p.ctl->qcount[qn], (unsigned)__popc(m));
            base = __shfl_sync(kFull, base, 0);
            if (need) qdst[base + __popc(m & ((1u << lane) - 1u))] = make_entry(it.epoch, (uint32_t)it.jid, nlb);
        }
    }
    if (lane == 0 && tot && left == tot) {  // this brick covered the job's last target voxel
        st->active = 0;
        atomicSub(&p.ctl->jobs_active, 1);
    }
}

template <int T, int BZ, bool SE18>
__global__ void __launch_bounds__(kTbWarps * 32, tb_min_ctas(T)) solve_tb_kernel(SolveParams p) {
    extern __shared__ __align__(16) unsigned char tb_smem[];
    __shared__ int s_flag;
    __shared__ unsigned s_gen, s_cnt;
    __shared__ Job s_jobs[kJobCache];
    Ctl* ctl = p.ctl;
    if (threadIdx.x == 0) {
        s_gen = (unsigned)(ld_acquire_u64(&ctl->release) >> 32);
        s_cnt = ld_relaxed_u32(&ctl->qcount[p.g0 % 3]);
    }
    // the first line of each cached job (every field an item reads)
    if (threadIdx.x < 32 * p.job_cache)
        reinterpret_cast<uint32_t*>(&s_jobs[threadIdx.x >> 5])[threadIdx.x & 31] =
            reinterpret_cast<const uint32_t*>(p.jobs + p.job_cache_base + (threadIdx.x >> 5))[threadIdx.x & 31];
    __syncthreads();
    unsigned gen = s_gen;
    unsigned cnt = s_cnt;
    const int wpb = blockDim.x >> 5;
    // warp number: CTA-major (consecutive queue items on one CTA's warps,
    // neighbouring bricks share halo lines in L1) or spread over the SMs
    const unsigned gw = p.spread ? (threadIdx.x >> 5) * gridDim.x + blockIdx.x : blockIdx.x * wpb + (threadIdx.x >> 5);
    const unsigned nw = gridDim.x * wpb;
    int g = p.g0;
    int it = 0;
    unsigned long long e_spec = 0ull;  // this warp's first entry of the step, read before the barrier
    unsigned char* wsm = tb_smem + (threadIdx.x >> 5) * tb_warp_bytes(T, BZ);
    if (cnt > 0) {
        for (;;) {
            const int qi = g % 3;
            unsigned long long* Q = qi == 0 ? p.queue[0] : (qi == 1 ? p.queue[1] : p.queue[2]);
            // Items to warps: a static stride (warp w takes entries w,
            // w + warps, ...) for the first part of the queue, the rest one
            // at a time from a counter, to whichever warp is free first
            // (warps with the same number of items finish up to a fifth
            // apart).  With at least kTbClaimRounds items per warp the last
            // quarter is claimed, each claim issued one item ahead so that
            // its round trip overlaps the brick in between; with fewer, the
            // entries past the last full stride are claimed after a warp's
            // last static brick (its round trip then waits, for those items
            // only, but they go to the warps that finished first).
            const unsigned rounds = cnt / nw;
            const bool ahead = rounds >= kTbClaimRounds;
            const unsigned S = ahead ? (rounds - rounds / 4) * nw : (rounds > 0 ? rounds * nw : cnt);
            unsigned* claimp = &ctl->claim[g % 3];
            const bool lane0 = (threadIdx.x & 31) == 0;
            unsigned c_next = 0u;
            // two-stage pipeline per warp: the next brick's copies are in
            // flight while this brick's epilogue atomics run
            TbItem cur;
            cur.live = false;
            unsigned i = gw;
            // ahead: a claim precedes every dynamic next item, the first one
            // here when the warp's static share is its first item alone
            if (ahead && S < cnt && i < cnt && i + nw >= S && lane0) c_next = atomicAdd(claimp, 1u);
            // The warp's first entry: the one read before the barrier if that
            // slot was already written (a slot below spec_first is zero until
            // its step's entry is written, so a non-zero value is that
            // entry), else a load now.  The slot is then cleared, and a slot
            // of the launch's first queue without an entry is zeroed.
            unsigned long long e0 = 0ull;
            if (i < cnt) e0 = e_spec != 0ull ? e_spec : Q[i];
            if ((int)gw < p.spec_first && (i < cnt || it == 0)) {
                __syncwarp();  // every lane's read of the slot precedes the clear
                if (lane0) Q[gw] = 0ull;
            }
            if (i < cnt) tb_issue<T, BZ>(p, e0, g, s_jobs, wsm, cur);
            while (i < cnt) {
                unsigned in = i + nw;
                const bool late = !ahead && in >= S && S < cnt;  // claimed after this brick
                if (ahead && in >= S && S < cnt) in = S + __shfl_sync(kFull, c_next, 0);  // claimed one item ago
                if (ahead && S < cnt && in < cnt && in + nw >= S && lane0) c_next = atomicAdd(claimp, 1u);
                unsigned long long en = (!late && in < cnt) ? Q[in] : 0ull;
                TbOut res;
                if (cur.live) tb_compute<T, BZ, SE18>(p, cur, wsm, res);
                if (late) {
                    in = S + __shfl_sync(kFull, lane0 ? atomicAdd(claimp, 1u) : 0u, 0);
                    en = in < cnt ? Q[in] : 0ull;
                }
                TbItem nxt;
                nxt.live = false;
                if (in < cnt) tb_issue<T, BZ>(p, en, g, s_jobs, wsm, nxt);
                if (cur.live) tb_epilogue<T, SE18>(p, cur, res, g);
                cur = nxt;
                i = in;
            }
            // the first entry of the next step, if its producer has written
            // it already (the barrier's wait hides the load)
            {
                const int qn = (g + 1) % 3;
                const unsigned long long* Qn = qn == 0 ? p.queue[0] : (qn == 1 ? p.queue[1] : p.queue[2]);
                e_spec = (int)gw < p.spec_first ? ld_relaxed_u64(Qn + gw) : 0ull;
            }
            const bool cont = grid_step_barrier(ctl, gen, g, p.timeout_ns, &s_flag, &s_cnt, p.yield, p.yield_gen);
            ++g;
            ++it;
            if (!cont || it >= p.max_iters) break;
            cnt = s_cnt;  // the next queue's length, published by the barrier
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        ctl->g_end = g;
        ctl->iters_run = it;
    }
    // results on the device: one warp per pair, after the last barrier
    if (p.out)
        for (unsigned i = gw; i < (unsigned)p.npairs; i += nw) decode_pair_warp(p, (int)i, it);
}

}  // namespace hdk
