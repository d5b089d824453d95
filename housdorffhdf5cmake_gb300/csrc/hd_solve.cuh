// hd_solve.cuh -- persistent frontier dilation kernel (sm_103a).
//
// Replaces the reference's per-iteration host loop around `dilate`
// (forBench/HausdorffDistance.cu:21-98 and :146-172) and the prototype's
// cooperative persistent kernel (hello.cu:1067-1896, grid.sync at :1727,1882).
//
// One launch runs many dilation steps.  Step g processes the bricks of the
// queue Q[g % 3]; each brick is one warp:
//   1. read the brick's word columns plus a one-word / one-row / one-plane
//      halo from the previous state buf[(k-1) & 1] (k = the job's local step);
//   2. dilate with the structuring element, x-axis bit carries through warp
//      shuffles (halo words at the brick's x edges), y through shuffles
//      (halo rows), z through a sliding window of planes;
//   3. write the new state to buf[k & 1]; the cover test hit = new & U counts
//      target voxels reached at step k (their distance is k) and clears them
//      from U (the test of forBench/HausdorffDistance.cu:96 made incremental;
//      the per-voxel value is the one hello.cu:1616-1618 records);
//   4. if anything changed, queue the brick and every neighbour whose shared
//      face changed into Q[(g + 1) % 3], deduplicated by a per-brick stamp.
// A grid barrier with a bounded wait ends each step.  Bricks that did not
// change and whose neighbours' faces did not change keep their state and are
// not visited: a brick is equal in both ping-pong buffers whenever it is not
// queued, so skipping it is exact.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "hd_device.cuh"

namespace hdk {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ int ld_relaxed_s32(const int* p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
// Arrival at the grid barrier: release (this CTA's writes before it) and
// acquire (the writes of the CTAs that arrived before) in one atomic.
__device__ __forceinline__ unsigned atom_add_acq_rel_u32(unsigned* p, unsigned v) {
    unsigned old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}
// Release of the grid barrier: every write before it is visible to a CTA
// that reads the new value with an acquire load.
__device__ __forceinline__ void atom_exch_release_u64(unsigned long long* p, unsigned long long v) {
    unsigned long long old;
    asm volatile("atom.release.gpu.global.exch.b64 %0, [%1], %2;" : "=l"(old) : "l"(p), "l"(v) : "memory");
    (void)old;
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned ld_relaxed_u32(const unsigned* p) {
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

constexpr int kErrTimeout = 5;    // HD_ERR_TIMEOUT
constexpr int kErrIterLimit = 7;  // HD_ERR_ITER_LIMIT

// Grid-wide barrier for a cooperative launch.  The last CTA to arrive
// decides whether the loop continues (no error, jobs left, next queue not
// empty, no yield requested through `yield`), resets the queue counter that
// step g + 2 will fill, and releases the others.  Every wait is bounded: after timeout_ns (or 2^26 polls) the
// waiting CTA records HD_ERR_TIMEOUT and leaves, and every other waiter sees
// the error and leaves as well.  Returns the continue flag (CTA-uniform).
__device__ __forceinline__ bool grid_step_barrier(Ctl* ctl, unsigned& gen, int g, long long timeout_ns, int* s_flag,
                                                  unsigned* s_cnt, const int32_t* yield, int32_t yield_gen) {
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned target = gen + 1u;
        unsigned long long rel = 0ull;
        // the CTA's threads wrote before the __syncthreads above; the
        // acq_rel arrival publishes those writes (cumulativity) and makes the
        // earlier arrivals' writes visible to the last CTA
        const unsigned arrived = atom_add_acq_rel_u32(&ctl->bar_count, 1u);
        if (arrived == gridDim.x - 1u) {
            ctl->bar_count = 0u;
            const int err = ld_relaxed_s32(&ctl->err);
            const int jobs = ld_relaxed_s32(&ctl->jobs_active);
            const unsigned nq = ld_relaxed_u32(&ctl->qcount[(g + 1) % 3]);
            const bool yl = yield != nullptr && ld_relaxed_s32(yield) != yield_gen;
            const bool cont = err == 0 && jobs > 0 && nq > 0u && !yl;
            ctl->qcount[(g + 2) % 3] = 0u;
            ctl->claim[(g + 1) % 3] = 0u;  // nobody claims from the next step's queue yet
            rel = ((unsigned long long)target << 32) | (cont ? 0x80000000ull : 0ull) | (nq & 0x7fffffffu);
            atom_exch_release_u64(&ctl->release, rel);
        } else {
            // poll hot at first (a barrier normally completes within a few
            // microseconds), then with short sleeps; bounded in time and count
            const unsigned long long t0 = globaltimer_ns();
            unsigned polls = 0;
            for (;;) {
                rel = ld_acquire_u64(&ctl->release);
                if ((unsigned)(rel >> 32) == target) break;
                if (ld_relaxed_s32(&ctl->err) != 0) break;
                if (++polls > 64u) __nanosleep(64);
                if ((long long)(globaltimer_ns() - t0) > timeout_ns || polls > (1u << 26)) {
                    atomicCAS(&ctl->err, 0, kErrTimeout);
                    break;
                }
            }
        }
        // the release word carries the decision: no further load
        const bool released = (unsigned)(rel >> 32) == target;
        *s_flag = (released && (rel & 0x80000000ull)) ? 1 : 0;
        *s_cnt = (unsigned)(rel & 0x7fffffffull);
    }
    gen += 1u;
    __syncthreads();
    return *s_flag != 0;
}

// Robust HD on the device, one warp: the stopping rule of hello.cu:1751-1758
// (keep dilating while (float)total * p > covered, covered = voxels with
// distance 1..k) on a per-step histogram, for both directions; the result is
// the later of their stopping steps.  covered grows with k, so the first k
// that stops is found 32 steps at a time by a prefix sum and a ballot (a
// single thread would wait on one load per step); the two histograms' words
// of a round are loaded together, and a direction that has stopped loads
// nothing more.
__device__ __forceinline__ int robust_k_warp2(const unsigned long long* ha, unsigned long long ta,
                                              const unsigned long long* hb, unsigned long long tb, int len,
                                              float p) {
    const int lane = threadIdx.x & 31;
    const float tfa = (float)ta * p, tfb = (float)tb * p;
    unsigned long long base_a = 0, base_b = 0;
    int ka = -1, kb = -1;
    for (int k0 = 0; k0 < len && (ka < 0 || kb < 0); k0 += 32) {
        const int k = k0 + lane;
        const bool in = k > 0 && k < len;
        unsigned long long ca = (ka < 0 && in) ? ha[k] : 0ull;
        unsigned long long cb = (kb < 0 && in) ? hb[k] : 0ull;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long xa = __shfl_up_sync(kFull, ca, o);
            const unsigned long long xb = __shfl_up_sync(kFull, cb, o);
            if (lane >= o) {
                ca += xa;
                cb += xb;
            }
        }
        if (ka < 0) {
            const unsigned m = __ballot_sync(kFull, k < len && !(tfa > (float)(base_a + ca)));
            if (m) ka = k0 + __ffs(m) - 1;
            base_a += __shfl_sync(kFull, ca, 31);
        }
        if (kb < 0) {
            const unsigned m = __ballot_sync(kFull, k < len && !(tfb > (float)(base_b + cb)));
            if (m) kb = k0 + __ffs(m) - 1;
            base_b += __shfl_sync(kFull, cb, 31);
        }
    }
    return max(ka < 0 ? len - 1 : ka, kb < 0 ? len - 1 : kb);
}

// Decodes pair i's result on the device (one warp), with the rules of the
// host decoder: statuses, one-sided distances, exact sums, average (one
// double division), robust HD.  Runs after the launch's last grid barrier,
// when every job's state is final.
static __device__ __noinline__ void decode_pair_warp(const SolveParams& p, int i, int iters) {
    const PairDesc& P = p.descs[i];
    if (p.decode_done_only) {
        if (P.info == nullptr) return;  // slot not in use
        if (p.states[P.job0].active != 0 || p.states[P.job0 + 1].active != 0) return;  // still running
    }
    const PairInfo I = *P.info;
    const JobState s0 = p.states[P.job0], s1 = p.states[P.job0 + 1];
    hd_result r;
    memset(&r, 0, sizeof r);
    r.n_a = I.n_a;
    r.n_b = I.n_b;
    r.n_a_not_b = I.n_a - I.n_ab;
    r.n_b_not_a = I.n_b - I.n_ab;
    r.iterations = iters;
    if (I.n_a == 0 && I.n_b == 0) {
        r.status = HD_OK;
    } else if (I.n_a == 0 || I.n_b == 0) {
        r.status = HD_EMPTY_MASK;
        r.hd = r.hd_ab = r.hd_ba = r.hd_robust = -1;
        r.avg_hd = __longlong_as_double(0x7ff8000000000000LL);  // quiet NaN
    } else {
        int st = ld_relaxed_s32(&p.ctl->err);
        if (!st) st = s0.status ? s0.status : s1.status;
        if (!st && (s0.remaining != 0 || s1.remaining != 0)) st = HD_ERR_ITER_LIMIT;
        r.status = st;
        r.hd_ba = s0.hd;  // job 0 dilates A and covers B
        r.sum_ba = s0.sum;
        r.hd_ab = s1.hd;
        r.sum_ab = s1.sum;
        r.hd = max(r.hd_ab, r.hd_ba);
        r.avg_hd = (double)(r.sum_ab + r.sum_ba) / (double)(r.n_a + r.n_b);
        const int kp1 = P.kmax + 1;
        r.hd_robust = robust_k_warp2(P.hist[1], r.n_a_not_b, P.hist[0], r.n_b_not_a, kp1, p.pct);
        if (st != HD_OK) r.hd = r.hd_ab = r.hd_ba = r.hd_robust = -1;
    }
    if ((threadIdx.x & 31) == 0) p.out[i] = r;
}

template <int BXW, int BZ, bool SE18>
__device__ __forceinline__ void brick_step(const SolveParams& p, int jid, unsigned lb, unsigned epoch, int g) {
    constexpr int BY = 32 / BXW;
    const int lane = threadIdx.x & 31;
    const int lx = lane % BXW, ly = lane / BXW;
    JobState* st = p.states + jid;
    if (ld_relaxed_s32(&st->active) == 0) return;  // job finished: nothing left to cover
    const Job* Jp = p.jobs + jid;
    if ((Jp->epoch & 0xffu) != epoch) return;      // left over from the slot's previous pair
    const int k = g - Jp->k0 + 1;  // local step, >= 1
    if (k > Jp->kmax) {
        if (lane == 0) {
            st->status = kErrIterLimit;
            atomicCAS(&p.ctl->err, 0, kErrIterLimit);
        }
        return;
    }
    const int nbx = Jp->nbx, nby = Jp->nby;
    const int Wx = Jp->wx, Hd = Jp->h, Dd = Jp->d;
    const int bx = (int)(lb % (unsigned)nbx);
    const unsigned t = lb / (unsigned)nbx;
    const int by = (int)(t % (unsigned)nby);
    const int bz = (int)(t / (unsigned)nby);
    const int wx = bx * BXW + lx, y = by * BY + ly, z0 = bz * BZ;
    const bool vx = wx < Wx, vy = y < Hd;
    const bool valid = vx && vy;
    const uint32_t* __restrict__ src = Jp->buf[(k - 1) & 1];
    uint32_t* __restrict__ dst = Jp->buf[k & 1];
    uint32_t* __restrict__ U = Jp->U;
    // Word offsets fit in 32 bits: the host rejects domains of 2^31 words or more.
    const int pitch = Jp->pitch;
    const int plane = pitch * Hd;
    const int rowoff = y * pitch + wx;
    const int nz = min(BZ, Dd - z0);
    const uint32_t tm = (wx == Wx - 1) ? Jp->tailmask : kFull;

    // Halo words: a lane sits on at most one x edge and one y edge of the
    // brick (BXW >= 2, BY >= 2), so it fetches at most one x-halo word, one
    // y-halo word and (18-neighbour element) one corner word per plane.
    const bool e_xl = lx == 0, e_xh = lx == BXW - 1, e_yl = ly == 0, e_yh = ly == BY - 1;
    const int hx_dx = e_xl ? -1 : 1;
    const bool f_hx = vy && ((e_xl && wx > 0) || (e_xh && wx + 1 < Wx));
    const int hy_dy = e_yl ? -1 : 1;
    const bool f_hy = vx && ((e_yl && y > 0) || (e_yh && y + 1 < Hd));
    const bool f_hc = SE18 && (e_xl || e_xh) && (e_yl || e_yh) && (wx + hx_dx >= 0) &&
                      (wx + hx_dx < Wx) && (y + hy_dy >= 0) && (y + hy_dy < Hd);
    const int o_hx = hx_dx, o_hy = hy_dy * (int)pitch, o_hc = o_hx + o_hy;

    // Phase 1: issue every load of the brick (planes z0-1 .. z0+BZ).
    uint32_t c[BZ + 2], hx[BZ + 2], hy[BZ + 2], hc[SE18 ? BZ + 2 : 1];
    uint32_t uu[BZ];
#pragma unroll
    for (int i = 0; i < BZ + 2; ++i) {
        const int pz = z0 - 1 + i;
        const bool inz = pz >= 0 && pz < Dd;
        const int off = pz * plane + rowoff;
        c[i] = (valid && inz) ? src[off] : 0u;
        hx[i] = (f_hx && inz) ? src[off + o_hx] : 0u;
        hy[i] = (f_hy && inz) ? src[off + o_hy] : 0u;
        if constexpr (SE18) hc[i] = (f_hc && inz) ? src[off + o_hc] : 0u;
    }
#pragma unroll
    for (int i = 0; i < BZ; ++i) uu[i] = (valid && i < nz) ? U[(z0 + i) * plane + rowoff] : 0u;

    // Phase 2: per plane, the in-plane dilation M and the part Z that the
    // planes above and below receive.
    //   SE6 : M = c | sx(c) | sy(c),                   Z = c
    //   SE18: M = c | sx(c) | sy(c) | sx(sy(c)),       Z = c | sx(sy(c))
    // where sx / sy are the +-1 shifts along x / y (without the identity).
    auto plane_terms = [&](int i, uint32_t& M, uint32_t& Z) {
        const uint32_t cc = c[i];
        uint32_t left = __shfl_up_sync(kFull, cc, 1);
        uint32_t right = __shfl_down_sync(kFull, cc, 1);
        uint32_t up = __shfl_up_sync(kFull, cc, BXW);
        uint32_t dn = __shfl_down_sync(kFull, cc, BXW);
        if (e_xl) left = hx[i];
        if (e_xh) right = hx[i];
        if (e_yl) up = hy[i];
        if (e_yh) dn = hy[i];
        const uint32_t sx = (cc << 1) | (left >> 31) | (cc >> 1) | (right << 31);
        const uint32_t Y = up | dn;
        if constexpr (!SE18) {
            M = cc | sx | Y;
            Z = cc;
        } else {
            // sy of the halo column: the x-halo words of the rows above and
            // below (held by the lanes with the same lx), or the corner word.
            uint32_t Yl = __shfl_up_sync(kFull, Y, 1);
            uint32_t Yr = __shfl_down_sync(kFull, Y, 1);
            const uint32_t hx_up = __shfl_up_sync(kFull, hx[i], BXW);
            const uint32_t hx_dn = __shfl_down_sync(kFull, hx[i], BXW);
            const uint32_t ycol = (e_yl ? hc[i] : hx_up) | (e_yh ? hc[i] : hx_dn);
            if (e_xl) Yl = ycol;
            if (e_xh) Yr = ycol;
            const uint32_t sxY = (Y << 1) | (Yl >> 31) | (Y >> 1) | (Yr << 31);
            M = cc | sx | Y | sxY;
            Z = cc | sxY;
        }
    };

    uint32_t Mdummy, Zprev, Mcur, Zcur;
    plane_terms(0, Mdummy, Zprev);
    plane_terms(1, Mcur, Zcur);
    (void)Mdummy;
    unsigned cnt = 0;
    uint32_t d_all = 0, d_lo = 0, d_hi = 0, d_z0 = 0, d_zl = 0;
    // instrumented runs: which of the (at most two) 32-plane tile layers got new voxels
    uint32_t tile_bits = 0;
    int32_t* map = (jid & 1) ? p.map[1] : p.map[0];
#pragma unroll
    for (int i = 0; i < BZ; ++i) {
        uint32_t Mn, Zn;
        plane_terms(i + 2, Mn, Zn);
        if (i < nz) {
            const uint32_t nw = (Mcur | Zprev | Zn) & tm;
            const uint32_t old = c[i + 1];
            const uint32_t diff = valid ? (nw ^ old) : 0u;
            const int off = (z0 + i) * plane + rowoff;
            if (valid) {
                dst[off] = nw;
                uint32_t hit = nw & uu[i];
                if (hit) {
                    // claim the hits: a voxel is counted once even if two warps
                    // ever process the same brick in one step
                    hit &= atomicAnd(&U[off], ~hit);
                    cnt += __popc(hit);
                    if (map != nullptr) {
                        const long long vz = Jp->oz + z0 + i, vyy = Jp->oy + y;
                        const long long base =
                            (vz * p.map_h + vyy) * (long long)p.map_w + Jp->ox + 32LL * wx;
                        uint32_t h = hit;
                        while (h) {
                            const int b = __ffs(h) - 1;
                            h &= h - 1u;
                            map[base + b] = k;
                        }
                    }
                }
            }
            d_all |= diff;
            d_lo |= diff & 1u;
            d_hi |= diff >> 31;
            if (i == 0) d_z0 |= diff;
            if (i == BZ - 1) d_zl |= diff;
            if (p.stats && diff) tile_bits |= 1u << (((Jp->oz + z0 + i) >> 5) - ((Jp->oz + z0) >> 5));
        }
        Zprev = Zcur;
        Mcur = Mn;
        Zcur = Zn;
    }

    // Cover counts: one set of atomics per brick.
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) cnt += __shfl_xor_sync(kFull, cnt, s);
    if (lane == 0 && cnt) {
        atomicAdd(&st->sum, (unsigned long long)k * cnt);
        atomicMax(&st->hd, k);
        atomicAdd(&Jp->hist[k], (unsigned long long)cnt);
        const unsigned long long left = atomicAdd(&st->remaining, (unsigned long long)(-(long long)cnt));
        if (left == cnt) {  // this brick covered the job's last target voxel
            st->active = 0;
            atomicSub(&p.ctl->jobs_active, 1);
        }
    }
    if (p.stats) {
        if (lane == 0) atomicAdd(&st->bricks, 1ull);
        if (valid && tile_bits) {
            const int tx = (Jp->ox >> 5) + wx, ty = (Jp->oy + y) >> 5, tz0 = (Jp->oz + z0) >> 5;
#pragma unroll
            for (int s = 0; s < 2; ++s) {
                if (tile_bits & (1u << s)) {
                    const long long tid = ((long long)(tz0 + s) * Jp->th + ty) * Jp->tw + tx;
                    if (atomicMax(&Jp->tstamp[tid], k) < k) atomicAdd(&Jp->tcount[k], 1ull);
                }
            }
        }
    }

    // Frontier: queue this brick and the neighbours that see a changed face.
    if (!__any_sync(kFull, d_all != 0)) return;
    const bool fxl = __any_sync(kFull, lx == 0 && d_lo != 0);
    const bool fxh = __any_sync(kFull, lx == BXW - 1 && d_hi != 0);
    const bool fyl = __any_sync(kFull, ly == 0 && d_all != 0);
    const bool fyh = __any_sync(kFull, ly == BY - 1 && d_all != 0);
    const bool fzl = __any_sync(kFull, d_z0 != 0);
    const bool fzh = __any_sync(kFull, d_zl != 0);
    bool need = false;
    unsigned nlb = 0;
    if (lane < 27) {
        const int ox = lane % 3 - 1, oy = (lane / 3) % 3 - 1, oz = lane / 9 - 1;
        const int nnz = (ox != 0) + (oy != 0) + (oz != 0);
        need = SE18 || nnz <= 1;
        if (ox < 0) need = need && fxl;
        if (ox > 0) need = need && fxh;
        if (oy < 0) need = need && fyl;
        if (oy > 0) need = need && fyh;
        if (oz < 0) need = need && fzl;
        if (oz > 0) need = need && fzh;
        const int nbx2 = bx + ox, nby2 = by + oy, nbz2 = bz + oz;
        need = need && nbx2 >= 0 && nbx2 < nbx && nby2 >= 0 && nby2 < nby && nbz2 >= 0 &&
               nbz2 < Jp->nbz;
        if (need) {
            nlb = (unsigned)((nbz2 * nby + nby2) * nbx + nbx2);
            const unsigned long long gid = Jp->brick0 + nlb;
            need = atomicMax(&p.stamps[gid], g + 1) < g + 1;
        }
    }
    const unsigned m = __ballot_sync(kFull, need);
    if (m) {
        const int qn = (g + 1) % 3;
        unsigned long long* qdst = qn == 0 ? p.queue[0] : (qn == 1 ? p.queue[1] : p.queue[2]);
        unsigned base = 0;
        if (lane == 0) base = atomicAdd(&p.ctl->qcount[qn], (unsigned)__popc(m));
        base = __shfl_sync(kFull, base, 0);
        if (need)
            qdst[base + __popc(m & ((1u << lane) - 1u))] = make_entry(epoch, (uint32_t)jid, nlb);
    }
}

template <int BXW, int BZ, bool SE18>
__global__ void __launch_bounds__(256, 2) solve_kernel(SolveParams p) {
    __shared__ int s_flag;
    __shared__ unsigned s_gen, s_cnt;
    Ctl* ctl = p.ctl;
    if (threadIdx.x == 0) {
        s_gen = (unsigned)(ld_acquire_u64(&ctl->release) >> 32);
        s_cnt = ld_relaxed_u32(&ctl->qcount[p.g0 % 3]);  // global memory: dynamic index is fine
    }
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
    if (cnt > 0) {
        for (;;) {
            const int qi = g % 3;
            const unsigned long long* Q = qi == 0 ? p.queue[0] : (qi == 1 ? p.queue[1] : p.queue[2]);
            for (unsigned i = gw; i < cnt; i += nw) {
                const unsigned long long e = Q[i];
                brick_step<BXW, BZ, SE18>(p, (int)((e >> 32) & kEntryJobMask), (unsigned)e, (unsigned)(e >> 56), g);
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
