// hd_pack.cu -- packing and set-up kernels (sm_103a).
//
// pack_kernel   replaces boolPrepareKernel (hello.cu:539-748) and the bounding
//               box of getMinMaxes (hello.cu:398-526): uint8 masks -> 32 voxels
//               per uint32 along x (the prototype packs along z, :598-631),
//               with |A|, |B|, |A n B| and the bounding box of A u B (x in
//               whole words).  One pass over the bytes, 128-bit streaming
//               loads; rows stored at a pitch of a multiple of 4 words.
// setup_kernel  replaces firstMetaPrepareKernel (hello.cu:763-877): writes
//               the job descriptors and queues every brick of each job for
//               its first step; for the one-step kernel it also crops the
//               packed masks to each job's domain and builds the
//               uncovered-target words.
// map_init_kernel  -1 / 0 initialisation of the optional per-voxel maps.
#include <algorithm>
#include <climits>
#include <cuda_runtime.h>
#include <stdint.h>

#include "hd/hd.h"
#include "hd_device.cuh"
#include "hd_kernels.h"

namespace hdk {

// Foreground bytes of a 32-bit word as flags at bits 28..31 (byte i -> bit
// 28 + i).  Foreground = nonzero, or (kLabel) equal to the label, whose
// byte `pat` repeats four times: the XOR turns those bytes into zeros and
// the zero-byte flags are the complement of the nonzero ones.  The
// normalised word has bits only at 7, 15, 23, 31; times 2^0 + 2^7 + 2^14 +
// 2^21 its partial products land on distinct bits (7, 14, 15, 21, 22, 23
// below 28, the flags at 28..31), so nothing carries.
template <bool kLabel>
__device__ __forceinline__ uint32_t fg4_top(uint32_t w, uint32_t pat) {
    if constexpr (kLabel) w ^= pat;
    uint32_t t = (((w & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | w) & 0x80808080u;
    if constexpr (kLabel) t ^= 0x80808080u;
    return t * 0x00204081u;
}

// Foreground bytes of 16 bytes -> 16 bits (byte i -> bit i).  The partial
// products below bit 24 vanish in the two larger shifts and are masked off in
// the two smaller ones.
template <bool kLabel>
__device__ __forceinline__ uint32_t fg16(uint4 v, uint32_t pat) {
    return (fg4_top<kLabel>(v.x, pat) >> 28) | (fg4_top<kLabel>(v.y, pat) >> 24) |
           ((fg4_top<kLabel>(v.z, pat) >> 20) & 0xF00u) | ((fg4_top<kLabel>(v.w, pat) >> 16) & 0xF000u);
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) v += __shfl_xor_sync(0xffffffffu, v, s);
    return v;
}
__device__ __forceinline__ int warp_min(int v) {
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, s));
    return v;
}
__device__ __forceinline__ int warp_max(int v) {
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, s));
    return v;
}

// The pair that owns work tile `tile` (first tiles increase with the pair
// index; setup = false: packing tiles, true: set-up tiles).
__device__ __forceinline__ int pair_of_tile(const PairDesc* __restrict__ descs, int npairs, long long tile,
                                            bool setup) {
    int lo = 0, hi = npairs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if ((setup ? descs[mid].stile0 : descs[mid].tile0) <= tile) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Counts and bounding box of the packed words a thread has seen in one pair.
// 32-bit counts: a thread packs at most 2^31 / 256 words of a pair.  The
// box is kept as word columns (x), rows (y) and row indices r = y + H z (z
// follows at the flush: r -> r / H is monotone).
struct PackAcc {
    uint32_t na = 0, nb = 0, nab = 0;
    int wmin = INT_MAX, wmax = -1, ymin = INT_MAX, ymax = -1, rmin = INT_MAX, rmax = -1;
    __device__ __forceinline__ void add(uint32_t wa, uint32_t wb, int r, int y, int w) {
        na += __popc(wa);
        nb += __popc(wb);
        nab += __popc(wa & wb);
        if (wa | wb) {
            wmin = min(wmin, w);
            wmax = max(wmax, w);
            ymin = min(ymin, y);
            ymax = max(ymax, y);
            rmin = min(rmin, r);
            rmax = max(rmax, r);
        }
    }
};

// Block-wide reduction of the accumulators, then one set of atomics per CTA
// (many CTAs update one PairInfo: per-warp atomics serialise on its lines).
// Called by all threads of the CTA.
__device__ __forceinline__ void flush_acc(const PairDesc& P, const PackAcc& acc) {
    __shared__ unsigned long long s_cnt[3][8];
    __shared__ int s_bb[6][8];
    const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    unsigned long long na = warp_sum_u64(acc.na), nb = warp_sum_u64(acc.nb), nab = warp_sum_u64(acc.nab);
    int bb[6] = {warp_min(acc.wmin), warp_max(acc.wmax), warp_min(acc.ymin),
                 warp_max(acc.ymax), warp_min(acc.rmin), warp_max(acc.rmax)};
    __syncthreads();  // earlier readers of the scratch are done
    if ((threadIdx.x & 31) == 0) {
        s_cnt[0][warp] = na;
        s_cnt[1][warp] = nb;
        s_cnt[2][warp] = nab;
#pragma unroll
        for (int i = 0; i < 6; ++i) s_bb[i][warp] = bb[i];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < nwarps; ++w) {
            na += s_cnt[0][w];
            nb += s_cnt[1][w];
            nab += s_cnt[2][w];
            for (int i = 0; i < 6; i += 2) {
                bb[i] = min(bb[i], s_bb[i][w]);
                bb[i + 1] = max(bb[i + 1], s_bb[i + 1][w]);
            }
        }
        PairInfo* I = P.info;
        if (na) atomicAdd(&I->n_a, na);
        if (nb) atomicAdd(&I->n_b, nb);
        if (nab) atomicAdd(&I->n_ab, nab);
        if (bb[1] >= 0) {
            const int H = P.H;
            atomicMin(&I->bb[0], bb[0]);
            atomicMax(&I->bb[1], bb[1]);
            atomicMin(&I->bb[2], bb[2]);
            atomicMax(&I->bb[3], bb[3]);
            atomicMin(&I->bb[4], bb[4] / H);
            atomicMax(&I->bb[5], bb[5] / H);
        }
    }
}

// Foreground bytes (nonzero, or equal to a nonzero label) among the 16 at p
// that lie inside [lo, hi), as 16 bits (a mask's first and last 16-byte
// chunks may stick out of it).  The byte loads
// are predicated, not branched over, so all sixteen are in flight together.
__device__ __noinline__ uint32_t chunk_bits_edge(const uint8_t* p, const uint8_t* lo, const uint8_t* hi, int label) {
    uint32_t bits = 0;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const bool in = p + i >= lo && p + i < hi;
        const uint8_t v = in ? __ldg(p + i) : (uint8_t)0;
        const bool fg = label ? (in && v == (uint8_t)label) : (v != 0);
        bits |= (fg ? 1u : 0u) << i;
    }
    return bits;
}

constexpr int kPackThreads = 256;
constexpr int kPackGroups = 4;  // words per thread and tile: a warp packs 32 * kPackGroups consecutive words
constexpr int kPackMinCtas = 2;  // resident CTAs per SM (register budget: 65536 / (kPackThreads * kPackMinCtas))
static_assert(kPackTileWords == (kPackThreads / 32) * 32 * kPackGroups, "one tile = one span per warp");

// Constants of one pair's packing walk (taken when a CTA's run of tiles
// enters the pair).
struct PackWalk {
    const uint8_t* src[2];
    const uint8_t* end[2];
    unsigned wxf, W, H, total;  // words per row, bytes per row, rows per plane, words of the pair
    unsigned pitch, npad;       // packed row pitch (words): wxf rounded up to 4, npad zero words
    unsigned dq, dr;            // 32 words = dq rows + dr words
    uint32_t tail;              // valid bits of a row's last word
};

__device__ __forceinline__ PackWalk make_walk(const PairDesc& P) {
    PackWalk k;
    const size_t nbytes = (size_t)P.W * P.H * P.D;
    k.src[0] = P.a;
    k.src[1] = P.b;
    k.end[0] = P.a + nbytes;
    k.end[1] = P.b + nbytes;
    k.wxf = (unsigned)P.wxf;
    k.pitch = (unsigned)packed_pitch(P.W);
    k.npad = k.pitch - k.wxf;
    k.W = (unsigned)P.W;
    k.H = (unsigned)P.H;
    k.total = (unsigned)((long long)P.wxf * P.H * P.D);  // < 2^31 words
    k.dq = 32u / k.wxf;
    k.dr = 32u - k.dq * k.wxf;
    const unsigned tb = k.W - 32u * (k.wxf - 1);
    k.tail = tb >= 32 ? 0xffffffffu : ((1u << tb) - 1u);
    return k;
}

// One tile of a pair, any width, alignment or memory kind (device or
// host-mapped).  Warp v packs words w_lo + 128 v + 32 i + lane (i < 4) of
// both masks (word t = row r, word w is stored at r * pitch + w; the row's
// last word also zeroes the padding after it).  Word t holds the mask bytes [o, o + n) with
// o = r W + 32 w, n = min(32, W - 32 w); with q = o rounded down to 16 and
// s = o - q they lie in the 16-byte chunks at q, q + 16 and, if s + n > 32,
// q + 32.  Rows are contiguous, so word t + 1 starts at o + n, and when
// s + n > 32 (then 32 < s + n <= 47) its first chunk is the one at q + 32.
// Each thread therefore loads two chunks per word and takes the third from
// the thread that holds word t + 1: the next lane, or lane 0's next group
// for lane 31.  Only lane 31's last group (and a pair's last word) loads a
// third chunk.  All loads are issued before any is used, as streaming loads.
// kEdge = false: every word of the tile is in the pair and every chunk it
// touches lies inside the masks (see pack_kernel); kEdge = true: both are
// checked word by word.
template <bool kEdge, bool kLabel>
__device__ __forceinline__ void pack_tile(const PairDesc& P, const PackWalk& k, long long tile_in_pair,
                                          PackAcc& acc, int label, uint32_t pat) {
    const int lane = threadIdx.x & 31;
    const unsigned t0 = (unsigned)(tile_in_pair * kPackTileWords) + (threadIdx.x >> 5) * (32u * kPackGroups) + lane;
    unsigned r = t0 / k.wxf, w = t0 - r * k.wxf;
    unsigned y = r % k.H;
    uint4 c[kPackGroups][2][2];
    uint4 c3[2] = {make_uint4(0u, 0u, 0u, 0u), make_uint4(0u, 0u, 0u, 0u)};
    unsigned rr[kPackGroups], ww[kPackGroups], yy[kPackGroups];
#pragma unroll
    for (int i = 0; i < kPackGroups; ++i) {
        rr[i] = r;
        ww[i] = w;
        yy[i] = y;
        const unsigned t = t0 + 32u * i;
        const size_t off = (size_t)r * k.W + 32u * w;
        const bool valid = !kEdge || t < k.total;
        const unsigned nbits = w + 1 == k.wxf ? k.W - 32u * w : 32u;
        const bool own3 = (i == kPackGroups - 1 && lane == 31) || (kEdge && t + 1 == k.total);
#pragma unroll
        for (int m = 0; m < 2; ++m) {
            const uint8_t* x = k.src[m] + off;
            const uint8_t* q = (const uint8_t*)((uintptr_t)x & ~(uintptr_t)15);
            const unsigned sh = (unsigned)((uintptr_t)x & 15);
            if (!kEdge || (valid && q >= k.src[m] && q + 48 <= k.end[m])) {
                c[i][m][0] = __ldcs(reinterpret_cast<const uint4*>(q));
                c[i][m][1] = __ldcs(reinterpret_cast<const uint4*>(q) + 1);
                if (own3 && sh + nbits > 32) c3[m] = __ldcs(reinterpret_cast<const uint4*>(q) + 2);
            } else {
                c[i][m][0] = c[i][m][1] = make_uint4(0u, 0u, 0u, 0u);
            }
        }
        // next group: 32 words on
        w += k.dr;
        unsigned dy = k.dq;
        if (w >= k.wxf) {
            w -= k.wxf;
            ++dy;
        }
        r += dy;
        y += dy;
        if (y >= k.H) y %= k.H;
    }
    // mask bits of each word's first two chunks
    uint32_t lo[kPackGroups][2];
#pragma unroll
    for (int i = 0; i < kPackGroups; ++i) {
        const size_t off = (size_t)rr[i] * k.W + 32u * ww[i];
        const unsigned t = t0 + 32u * i;
#pragma unroll
        for (int m = 0; m < 2; ++m) {
            if (kEdge) {
                const uint8_t* q = (const uint8_t*)((uintptr_t)(k.src[m] + off) & ~(uintptr_t)15);
                if (t < k.total && !(q >= k.src[m] && q + 48 <= k.end[m])) {
                    lo[i][m] = chunk_bits_edge(q, k.src[m], k.end[m], label) |
                               (chunk_bits_edge(q + 16, k.src[m], k.end[m], label) << 16);
                    continue;
                }
            }
            lo[i][m] = fg16<kLabel>(c[i][m][0], pat) | (fg16<kLabel>(c[i][m][1], pat) << 16);
        }
    }
#pragma unroll
    for (int i = 0; i < kPackGroups; ++i) {
        const unsigned t = t0 + 32u * i;
        const unsigned wi = ww[i];
        const size_t off = (size_t)rr[i] * k.W + 32u * wi;
        const bool last = wi + 1 == k.wxf;
        const unsigned nbits = last ? k.W - 32u * wi : 32u;
        const bool own3 = (i == kPackGroups - 1 && lane == 31) || (kEdge && t + 1 == k.total);
        uint32_t out[2];
#pragma unroll
        for (int m = 0; m < 2; ++m) {
            const unsigned sh = (unsigned)((uintptr_t)(k.src[m] + off) & 15);
            uint32_t hi = __shfl_down_sync(0xffffffffu, lo[i][m] & 0xffffu, 1);
            if (i + 1 < kPackGroups) {
                const uint32_t wrap = __shfl_sync(0xffffffffu, lo[i + 1 < kPackGroups ? i + 1 : i][m] & 0xffffu, 0);
                if (lane == 31) hi = wrap;
            }
            if (own3 && sh + nbits > 32) {  // rare: the warp's last word, the pair's last word
                if (kEdge) {
                    const uint8_t* q = (const uint8_t*)((uintptr_t)(k.src[m] + off) & ~(uintptr_t)15);
                    hi = (q >= k.src[m] && q + 48 <= k.end[m]) ? fg16<kLabel>(c3[m], pat)  // loaded above
                                                                : chunk_bits_edge(q + 32, k.src[m], k.end[m], label);
                } else {
                    hi = fg16<kLabel>(c3[m], pat);
                }
            }
            out[m] = __funnelshift_r(lo[i][m], hi, sh) & (last ? k.tail : 0xffffffffu);
        }
        if (!kEdge || t < k.total) {
            const size_t o = (size_t)rr[i] * k.pitch + wi;
            P.pa[o] = out[0];
            P.pb[o] = out[1];
            if (last && k.npad) {  // the row's last word also writes its padding (1-3 words)
                P.pa[o + 1] = P.pb[o + 1] = 0u;
                if (k.npad > 1) P.pa[o + 2] = P.pb[o + 2] = 0u;
                if (k.npad > 2) P.pa[o + 3] = P.pb[o + 3] = 0u;
            }
            acc.add(out[0], out[1], (int)rr[i], (int)yy[i], (int)wi);
        }
    }
}

// Packing launch: one wave of resident CTAs, each over a contiguous run of
// tiles (a run crosses few pairs, so the pair lookup and the accumulator
// flush are rare).  A tile takes the checked path if it is a pair's first
// tile or reaches within 48 words of the pair's end: every other word then
// starts at byte >= kPackTileWords (each word holds >= 1 byte) and ends >= 48
// bytes before the mask's end, so its three chunks lie inside the mask.
template <bool kLabel>
__global__ void __launch_bounds__(kPackThreads, kPackMinCtas) pack_kernel(const PairDesc* __restrict__ descs, int npairs,
                                                               long long ntiles, int label) {
    const uint32_t pat = (uint32_t)label * 0x01010101u;
    PackAcc acc;
    PackWalk walk;
    int pi = -1;
    const long long per = (ntiles + gridDim.x - 1) / gridDim.x;
    const long long t_lo = (long long)blockIdx.x * per, t_hi = min(ntiles, t_lo + per);
    for (long long tile = t_lo; tile < t_hi; ++tile) {
        // tiles only increase: walk forward to the owning pair
        int np = pi < 0 ? pair_of_tile(descs, npairs, tile, false) : pi;
        while (np + 1 < npairs && descs[np + 1].tile0 <= tile) ++np;
        if (np != pi) {
            if (pi >= 0) {
                flush_acc(descs[pi], acc);
                acc = PackAcc();
            }
            pi = np;
            walk = make_walk(descs[pi]);
        }
        const long long tp = tile - descs[pi].tile0;
        if (tp >= 1 && (tp + 1) * kPackTileWords + 48 <= (long long)walk.total)
            pack_tile<false, kLabel>(descs[pi], walk, tp, acc, label, pat);
        else
            pack_tile<true, kLabel>(descs[pi], walk, tp, acc, label, pat);
    }
    if (pi >= 0) flush_acc(descs[pi], acc);
}

struct Domain {
    int ox, oy, oz, wv, h, d, wx0, wx, pitch;
};

// Bounding box of the domain, before any rounding of its first word: the
// 6-neighbour element uses the bounding box of A u B (x in whole words), the
// 18-neighbour element that box widened by one word in x and one row and
// plane in y and z, clipped to the volume.  Exactness: a shortest
// 6-neighbour path between two voxels of a box is monotone and stays in it.
// An 18-neighbour step (the 6 face neighbours, the 4 in-plane diagonals and
// the 8 corners) changes z by at most 1 and x and y together through the
// corners; between two voxels at offsets (a, b, c) a shortest path takes c
// z steps whose corners' x and y moves alternate around the needed offset,
// plus king moves in the plane, so it leaves the box of the two voxels by
// at most one voxel in x or y and never in z (where it would need two more
// z steps).  Where the widened box is clipped by the volume, the whole
// volume offers no detour on that side either.  (Without the margin the
// results differ: offset (0, 2, 2) takes the corners (1, 1, 1) and
// (-1, 1, 1), 2 steps, against 4 inside a box one voxel wide in x.)
struct DomainBox {
    int w0, w1, y0, y1, z0, z1;  // inclusive: word columns, rows, planes
};
__device__ __forceinline__ DomainBox domain_box(const PairDesc& P, const PairInfo& I) {
    DomainBox b{I.bb[0], I.bb[1], I.bb[2], I.bb[3], I.bb[4], I.bb[5]};
    if (P.se != 0) {
        const int wxf = (P.W + 31) >> 5;
        b.w0 = max(0, b.w0 - 1);
        b.w1 = min(wxf - 1, b.w1 + 1);
        b.y0 = max(0, b.y0 - 1);
        b.y1 = min(P.H - 1, b.y1 + 1);
        b.z0 = max(0, b.z0 - 1);
        b.z1 = min(P.D - 1, b.z1 + 1);
    }
    return b;
}

// The domain of a pair (quad: its first word rounded down to a multiple of
// 4, so that its rows start on 16-byte boundaries of the packed masks; any
// box inside the volume that contains the one above is as exact).
__device__ __forceinline__ Domain make_domain(const PairDesc& P, const PairInfo& I, bool quad) {
    const DomainBox b = domain_box(P, I);
    Domain m;
    m.wx0 = quad ? (b.w0 & ~3) : b.w0;  // word columns
    m.ox = 32 * m.wx0;
    m.wv = min(P.W, 32 * (b.w1 + 1)) - m.ox;
    m.oy = b.y0;
    m.h = b.y1 - b.y0 + 1;
    m.oz = b.z0;
    m.d = b.z1 - b.z0 + 1;
    m.wx = (m.wv + 31) >> 5;
    m.pitch = (m.wx + 3) & ~3;
    return m;
}

// Blocked kernel: can the domain start on a multiple of 4 words (its rows
// then start on 16-byte boundaries of the packed masks, which the kernel
// reads in place) without adding a brick column?
__device__ __forceinline__ bool blocked_in_place(const PairDesc& P, const PairInfo& I) {
    const DomainBox b = domain_box(P, I);
    const int w1 = b.w1 + 1;  // the domain's words end here (inside the volume)
    return (w1 - b.w0 + 3) / 4 == (w1 - (b.w0 & ~3) + 3) / 4;
}

__device__ __forceinline__ long long setup_tile(const PairDesc& P, long long tile_in_pair, Job* jobs,
                                                JobState* states, unsigned long long* queue0, Ctl* ctl, int g0,
                                                int bxw, int by, int bz, int mode, unsigned* s_base);

// 1D grid, block 256: CTAs stride over the tiles of all pairs
// (setup_tiles_of per pair); tile 0 of a pair also writes its job
// descriptors.  Modes:
//   kSetupOneStep         crop the packed masks into both ping-pong buffers
//                         and the uncovered-target array of each job
//   kSetupBlocked         the blocked kernel reads the packed masks in place
//                         when blocked_in_place, else crops of A and B (one
//                         pair: an extra brick column costs a whole
//                         latency-bound first iteration more than the copy)
//   kSetupBlockedCrop     crops of A and B (the packed masks are freed after
//                         set-up)
//   kSetupBlockedInPlace  the packed masks in place (batches: the copy costs
//                         more than the extra bricks)
__global__ void __launch_bounds__(256) setup_kernel(const PairDesc* __restrict__ descs, int npairs, long long ntiles,
                                                    Job* jobs, JobState* states, unsigned long long* queue0,
                                                    Ctl* ctl, int g0, int bxw, int by, int bz, int mode,
                                                    unsigned long long* zq1, unsigned long long* zq2, int nz) {
    __shared__ unsigned s_base;
    int pi = -1;
    const long long G = gridDim.x;
    // the first nz slots of the two queues the first step does not read
    // (the dilation kernel reads a warp's next first entry early where a
    // slot is non-zero)
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < nz; t += G * blockDim.x) {
        zq1[t] = 0ull;
        zq2[t] = 0ull;
    }
    // CTAs stride over the tiles: a pair's domain fills only the first of
    // its tiles, so contiguous runs would leave some CTAs without work
    for (long long tile = blockIdx.x; tile < ntiles; tile += G) {
        int np = pi < 0 ? pair_of_tile(descs, npairs, tile, true) : pi;
        while (np + 1 < npairs && descs[np + 1].stile0 <= tile) ++np;  // tiles only increase
        pi = np;
        const long long t0 = descs[pi].stile0;
        const long long need = setup_tile(descs[pi], tile - t0, jobs, states, queue0, ctl, g0, bxw, by, bz, mode,
                                          &s_base);
        // The pair's tiles from `need` on have nothing to do (the host sizes
        // the tiles for the largest domain and for copies that reading the
        // packed masks in place makes unnecessary): continue at this CTA's
        // first tile of the next pair.  CTA-uniform.
        if (tile - t0 + G >= need) {
            const long long next0 = pi + 1 < npairs ? descs[pi + 1].stile0 : ntiles;
            const long long first = next0 + ((((long long)blockIdx.x - next0) % G) + G) % G;  // >= tile + G
            tile = first - G;
        }
    }
}

// Returns the number of tiles of the pair that have work (descriptors,
// copies or queue entries): later tiles return at once.
__device__ __forceinline__ long long setup_tile(const PairDesc& P, long long tile_in_pair, Job* jobs,
                                                JobState* states, unsigned long long* queue0, Ctl* ctl, int g0,
                                                int bxw, int by, int bz, int mode, unsigned* s_base) {
    const PairInfo I = *P.info;
    const bool empty_a = I.n_a == 0, empty_b = I.n_b == 0;
    const unsigned long long rem[2] = {I.n_b - I.n_ab, I.n_a - I.n_ab};
    const long long cap = domain_cap_words(P.W, P.H, P.D);  // copying modes: the tiles cover [0, cap) words
    const long long ntiles_pair = setup_tiles_of(P.W, P.H, P.D, mode, bxw, by, bz);
    const long long w_lo = tile_in_pair * kTileWords, w_hi = min(cap, w_lo + kTileWords);
    const long long tid0 = threadIdx.x;
    const long long nthr = blockDim.x;
    const bool first = tile_in_pair == 0;
    const int kmax = P.kmax;
    // histograms are zeroed for every pair
    if (first)
        for (int j = 0; j < 2; ++j)
            for (int t = (int)tid0; t <= kmax; t += (int)nthr) P.hist[j][t] = 0ull;
    if (empty_a || empty_b) {
        if (first && tid0 == 0) {
            for (int j = 0; j < 2; ++j) {
                JobState& s = states[P.job0 + j];
                s.sum = 0; s.remaining = 0; s.bricks = 0; s.hd = 0; s.last_k = 0;
                s.status = (empty_a && empty_b) ? 0 : 1;  // HD_EMPTY_MASK
                s.active = 0;
                Job& J = jobs[P.job0 + j];
                J.nbx = J.nby = J.nbz = 0;
                J.epoch = P.epoch;
            }
        }
        return 1;
    }
    const bool one_step = mode == kSetupOneStep;
    const bool in_place = mode == kSetupBlockedInPlace || (mode == kSetupBlocked && blocked_in_place(P, I));
    const Domain m = make_domain(P, I, in_place);
    const int nbx = (m.wx + bxw - 1) / bxw, nby = (m.h + by - 1) / by, nbz = (m.d + bz - 1) / bz;
    const long long nbricks = (long long)nbx * nby * nbz;
    // crops of A and B (blocked kernel) live in the two jobs' U slots
    uint32_t* const crop[2] = {P.jb[0][2], P.jb[1][2]};
    if (first && tid0 == 0) {
        for (int j = 0; j < 2; ++j) {
            Job& J = jobs[P.job0 + j];
            J.buf[0] = P.jb[j][0];
            J.buf[1] = P.jb[j][1];
            J.U = one_step ? P.jb[j][2] : nullptr;
            if (in_place) {
                J.vol[0] = j == 0 ? P.pa : P.pb;
                J.vol[1] = j == 0 ? P.pb : P.pa;
                J.vpitch = packed_pitch(P.W);
                J.vh = P.H;
                J.vx0 = m.wx0;
                J.vy0 = m.oy;
                J.vz0 = m.oz;
            } else {
                J.vol[0] = crop[j];
                J.vol[1] = crop[1 - j];
                J.vpitch = m.pitch;
                J.vh = m.h;
                J.vx0 = J.vy0 = J.vz0 = 0;
            }
            J.hist = P.hist[j];
            J.wv = m.wv; J.h = m.h; J.d = m.d;
            J.wx = m.wx; J.pitch = m.pitch;
            const int tb = m.wv - 32 * (m.wx - 1);
            J.tailmask = tb >= 32 ? 0xffffffffu : ((1u << tb) - 1u);
            J.nbx = nbx; J.nby = nby; J.nbz = nbz;
            J.k0 = g0;
            J.kmax = kmax;
            J.ox = m.ox; J.oy = m.oy; J.oz = m.oz;
            J.tw = (P.W + 31) >> 5; J.th = (P.H + 31) >> 5;
            J.brick0 = P.brick0[j];
            J.tstamp = P.tstamp[j];
            J.tcount = P.tcount[j];
            J.epoch = P.epoch;
            JobState& s = states[P.job0 + j];
            s.sum = 0; s.remaining = rem[j]; s.bricks = 0; s.hd = 0; s.last_k = 0; s.status = 0;
            s.active = rem[j] > 0 ? 1 : 0;
            if (rem[j] > 0) atomicAdd(&ctl->jobs_active, 1);
        }
    }
    // Crop copy.  Job 0 dilates A and must cover B; job 1 dilates B and covers A.
    const bool act0 = rem[0] > 0, act1 = rem[1] > 0;
    const long long words_all = (one_step || !in_place) ? (long long)m.pitch * m.h * m.d : 0;
    const long long words = min(words_all, w_hi);
    const int vpitch = packed_pitch(P.W);
    for (long long t = w_lo + tid0; t < words; t += nthr) {
        // domain word index < 2^31: 32-bit divisions
        const unsigned tu = (unsigned)t;
        const unsigned r = tu / (unsigned)m.pitch;
        const int w = (int)(tu - r * (unsigned)m.pitch);
        uint32_t a = 0, b = 0;
        if (w < m.wx) {
            const unsigned zq = r / (unsigned)m.h;
            const int yl = (int)(r - zq * (unsigned)m.h), zl = (int)zq;
            const long long src = ((long long)(m.oz + zl) * P.H + (m.oy + yl)) * vpitch + m.wx0 + w;
            a = __ldg(P.pa + src);
            b = __ldg(P.pb + src);
        }
        if (one_step) {
            if (act0) {
                P.jb[0][0][t] = a;
                P.jb[0][1][t] = a;
                P.jb[0][2][t] = b & ~a;
            }
            if (act1) {
                P.jb[1][0][t] = b;
                P.jb[1][1][t] = b;
                P.jb[1][2][t] = a & ~b;
            }
        } else {  // source and target of both jobs
            crop[0][t] = a;
            crop[1][t] = b;
        }
    }
    // First step of each active job: every brick of its domain.  The
    // bricks go to the pair's first tiles, at least 256 per tile, and each
    // such tile reserves its queue entries with one atomic per job.
    const long long b_even = (long long)(((unsigned)nbricks + (unsigned)ntiles_pair - 1u) / (unsigned)ntiles_pair);
    const long long b_per = mode == kSetupBlockedInPlace ? kSetupBricks
                                                          : (b_even > 256 ? b_even : 256);  // < 2^31 bricks, tiles
    const long long b_lo = tile_in_pair * b_per, b_hi = min(nbricks, b_lo + b_per);
    const long long need = max(max((words_all + kTileWords - 1) / kTileWords, (nbricks + b_per - 1) / b_per), 1ll);
    if (b_lo >= b_hi) return need;  // CTA-uniform
    for (int j = 0; j < 2; ++j) {
        if (!(j == 0 ? act0 : act1)) continue;
        if (tid0 == 0) *s_base = atomicAdd(&ctl->qcount[g0 % 3], (unsigned)(b_hi - b_lo));
        __syncthreads();
        const unsigned base = *s_base;
        for (long long t = b_lo + tid0; t < b_hi; t += nthr)
            queue0[base + (unsigned)(t - b_lo)] = make_entry(P.epoch, (uint32_t)(P.job0 + j), (uint32_t)t);
        __syncthreads();  // s_base is written again next
    }
    return need;
}

// Start values of each pair's counts and bounding box (one thread per pair).
__global__ void info_init_kernel(const PairDesc* __restrict__ descs, int npairs, PairDesc* __restrict__ slot_descs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npairs) return;
    if (slot_descs) slot_descs[descs[i].job0 / 2] = descs[i];  // serving: the slot's copy for the result decode
    PairInfo* I = descs[i].info;
    I->n_a = I->n_b = I->n_ab = 0ull;
    I->bb[0] = I->bb[2] = I->bb[4] = INT_MAX;
    I->bb[1] = I->bb[3] = I->bb[5] = -1;
    I->pad[0] = I->pad[1] = 0;
}

// Serving: retire finished pairs' slots.  list holds (slot, epoch) pairs: the
// slot's jobs take the new epoch (queue entries still listed for them are
// dropped) and the slot's descriptor copy is marked unused (info = null).
__global__ void retire_kernel(Job* __restrict__ jobs, PairDesc* __restrict__ slot_descs,
                              const uint32_t* __restrict__ list, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t slot = list[2 * i], ep = list[2 * i + 1];
    jobs[2 * slot].epoch = ep;
    jobs[2 * slot + 1].epoch = ep;
    slot_descs[slot].info = nullptr;
}

// Instrumented runs: zero the per-tile stamps and per-step tile counters.
__global__ void zero_i32_kernel(int32_t* p, long long n) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x)
        p[t] = 0;
}

// Per-voxel maps: -1 outside the mask, 0 on the overlap, and (filled later by
// the dilation) the distance on voxels of one mask outside the other.
__global__ void map_init_kernel(const PairDesc* __restrict__ descs, int32_t* map_a, int32_t* map_b, int label) {
    const PairDesc& P = descs[0];
    const long long n = (long long)P.W * P.H * P.D;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const bool a = label ? P.a[t] == label : P.a[t] != 0, b = label ? P.b[t] == label : P.b[t] != 0;
        map_a[t] = a ? (b ? 0 : -2) : -1;  // -2: to be filled by the dilation
        map_b[t] = b ? (a ? 0 : -2) : -1;
    }
}

}  // namespace hdk

// ---- launch wrappers (called from the host orchestration) -----------------
namespace hdk {

cudaError_t launch_pack(const PairDesc* d_descs, int npairs, long long ntiles, int grid, int label, int sms,
                        cudaStream_t s) {
    // one wave of resident CTAs (per device and variant, from the occupancy calculator)
    static int resident[2][64] = {{0}};
    static int per_sm_of[2][64] = {{0}};
    const int v = label ? 1 : 0;
    const void* fn = label ? reinterpret_cast<const void*>(&pack_kernel<true>)
                           : reinterpret_cast<const void*>(&pack_kernel<false>);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 64 && resident[v][dev] == 0) {
        int per_sm = 0, sms_dev = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kPackThreads, 0);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms_dev, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return e;
        resident[v][dev] = std::max(1, per_sm) * std::max(1, sms_dev);
        per_sm_of[v][dev] = std::max(1, per_sm);
    }
    if (dev < 64) grid = sms > 0 ? per_sm_of[v][dev] * sms : resident[v][dev];
    if (grid > ntiles) grid = (int)ntiles;
    if (grid < 1) grid = 1;
    if (label) pack_kernel<true><<<grid, kPackThreads, 0, s>>>(d_descs, npairs, ntiles, label);
    else pack_kernel<false><<<grid, kPackThreads, 0, s>>>(d_descs, npairs, ntiles, 0);
    return cudaGetLastError();
}

cudaError_t launch_setup(const PairDesc* d_descs, int npairs, long long ntiles, int sms, Job* jobs,
                         JobState* states, unsigned long long* queue0, Ctl* ctl, int g0, int bxw, int by, int bz,
                         int mode, cudaStream_t s, unsigned long long* zq1, unsigned long long* zq2, int nz) {
    // one wave of resident CTAs (per device, from the occupancy calculator):
    // CTAs whose tiles have nothing to do leave at once, later waves would
    // only add their scheduling
    static int per_sm_of[64] = {0};
    static int sms_of[64] = {0};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    int per_sm = 8, nsm = sms > 0 ? sms : 1;
    if (dev < 64) {
        if (per_sm_of[dev] == 0) {
            int occ = 0, sms_dev = 0;
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, reinterpret_cast<const void*>(&setup_kernel), 256,
                                                              0);
            if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms_dev, cudaDevAttrMultiProcessorCount, dev);
            if (e != cudaSuccess) return e;
            per_sm_of[dev] = std::max(1, occ);
            sms_of[dev] = std::max(1, sms_dev);
        }
        per_sm = per_sm_of[dev];
        if (sms <= 0) nsm = sms_of[dev];
    }
    long long grid = std::min<long long>((long long)per_sm * nsm, ntiles);
    if (grid < 1) grid = 1;
    setup_kernel<<<(unsigned)grid, 256, 0, s>>>(d_descs, npairs, ntiles, jobs, states, queue0, ctl, g0, bxw, by, bz,
                                                mode, zq1, zq2, zq1 && zq2 ? nz : 0);
    return cudaGetLastError();
}

cudaError_t launch_info_init(const PairDesc* d_descs, int npairs, cudaStream_t s, PairDesc* slot_descs) {
    if (npairs <= 0) return cudaSuccess;
    info_init_kernel<<<(npairs + 255) / 256, 256, 0, s>>>(d_descs, npairs, slot_descs);
    return cudaGetLastError();
}

cudaError_t launch_retire(Job* jobs, PairDesc* slot_descs, const uint32_t* list, int n, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    retire_kernel<<<(n + 127) / 128, 128, 0, s>>>(jobs, slot_descs, list, n);
    return cudaGetLastError();
}

cudaError_t launch_zero_i32(int32_t* p, long long n, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    long long blocks = (n + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    zero_i32_kernel<<<(int)blocks, 256, 0, s>>>(p, n);
    return cudaGetLastError();
}

cudaError_t launch_map_init(const PairDesc* d_descs, int32_t* map_a, int32_t* map_b, long long n, int label,
                            cudaStream_t s) {
    long long blocks = (n + 255) / 256;
    if (blocks > 8192) blocks = 8192;
    map_init_kernel<<<(int)blocks, 256, 0, s>>>(d_descs, map_a, map_b, label);
    return cudaGetLastError();
}

}  // namespace hdk
