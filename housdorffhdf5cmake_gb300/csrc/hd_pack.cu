// hd_pack.cu -- packing and set-up kernels (sm_103a).
//
// pack_kernel   replaces boolPrepareKernel (hello.cu:539-748) and the bounding
//               box of getMinMaxes (hello.cu:398-526): uint8 masks -> 32 voxels
//               per uint32 along x (the prototype packs along z, :598-631),
//               with |A|, |B|, |A n B| and the bounding box of A u B.  One pass
//               over the bytes, 128-bit loads.
// setup_kernel  replaces firstMetaPrepareKernel (hello.cu:763-877): crops the
//               packed masks to each job's domain, builds the uncovered-target
//               words, writes the job descriptors and queues every brick of
//               each job for its first step.
// map_init_kernel  -1 / 0 initialisation of the optional per-voxel maps.
#include <climits>
#include <cuda_runtime.h>
#include <stdint.h>

#include "hd_device.cuh"
#include "hd_kernels.h"

namespace hdk {

// Nonzero bytes of a 32-bit word -> 4 bits (byte i -> bit i).
__device__ __forceinline__ uint32_t nz4(uint32_t w) {
    uint32_t t = (((w & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | w) & 0x80808080u;
    // bits 7, 15, 23, 31 -> 28, 29, 30, 31 (products land on distinct bits, no carries)
    return ((t >> 7) * 0x10204080u) >> 28;
}

__device__ __forceinline__ uint32_t nz16(uint4 v) {
    return nz4(v.x) | (nz4(v.y) << 4) | (nz4(v.z) << 8) | (nz4(v.w) << 12);
}

// 16 mask bits of the 16-byte chunk `ch` of a buffer of n bytes.
__device__ __forceinline__ uint32_t chunk_bits(const uint8_t* __restrict__ p, long long ch, long long n,
                                               bool aligned) {
    const long long s = ch * 16;
    if (s >= n) return 0u;
    if (aligned && s + 16 <= n) return nz16(*reinterpret_cast<const uint4*>(p + s));
    uint32_t bits = 0;
    const int lim = (int)((n - s) < 16 ? (n - s) : 16);
    for (int i = 0; i < lim; ++i) bits |= (uint32_t)(p[s + i] != 0) << i;
    return bits;
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

// Bounding-box / count accumulation of one packed word pair.
struct PackAcc {
    unsigned long long na = 0, nb = 0, nab = 0;
    int bb[6] = {INT_MAX, -1, INT_MAX, -1, INT_MAX, -1};
    __device__ __forceinline__ void add(uint32_t wa, uint32_t wb, long long r, int w, int H) {
        na += __popc(wa);
        nb += __popc(wb);
        nab += __popc(wa & wb);
        const uint32_t u = wa | wb;
        if (u) {
            const int y = (int)(r % H), z = (int)(r / H);
            bb[0] = min(bb[0], 32 * w + __ffs(u) - 1);
            bb[1] = max(bb[1], 32 * w + 31 - __clz(u));
            bb[2] = min(bb[2], y);
            bb[3] = max(bb[3], y);
            bb[4] = min(bb[4], z);
            bb[5] = max(bb[5], z);
        }
    }
};

// 1D grid, block 256: CTAs stride over the tiles of all pairs (kTileWords
// packed words per tile).
//   fast path (rows of whole words, 16-byte aligned masks): word t covers bytes
//   [32 t, 32 t + 32), read as two 16-byte chunks by two neighbouring lanes;
//   general path: word by word, three 16-byte chunks around the word's bytes.
__device__ __forceinline__ void flush_acc(const PairDesc& P, const PackAcc& acc);

__device__ __forceinline__ void pack_tile(const PairDesc& P, long long tile_in_pair);

__global__ void __launch_bounds__(256) pack_kernel(const PairDesc* __restrict__ descs, int npairs,
                                                   long long ntiles) {
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int pi = pair_of_tile(descs, npairs, tile, false);
        pack_tile(descs[pi], tile - descs[pi].tile0);
    }
}

__device__ __forceinline__ void pack_tile(const PairDesc& P, long long tile_in_pair) {
    const int W = P.W, H = P.H, wxf = P.wxf;
    const long long total_all = (long long)wxf * H * P.D;
    const long long nbytes = (long long)W * H * P.D;
    const bool aligned = P.aligned != 0;
    // this tile's words [w_lo, w_hi) of the pair
    const long long w_lo = tile_in_pair * kTileWords;
    const long long total = min(total_all, w_lo + kTileWords);
    const long long tid = threadIdx.x;
    const long long nthr = blockDim.x;
    PackAcc acc;
    if (aligned && (W & 31) == 0) {
        // Coalesced: per load instruction the warp reads 32 consecutive
        // 16-byte chunks (512 B); lane l's chunk holds 16 voxels, even lanes
        // take the odd neighbour's 16 bits and own a word.  A warp handles 4 x
        // 16 words of each mask per round, all 8 loads issued first.
        const uint4* a4 = reinterpret_cast<const uint4*>(P.a);
        const uint4* b4 = reinterpret_cast<const uint4*>(P.b);
        const int lane = threadIdx.x & 31;
        const long long warp = tid >> 5, nwarp = nthr >> 5;
        const long long chunks = 2 * total;  // end of this tile in 16-byte chunks of one mask
        for (long long c0 = 2 * w_lo + warp * 128; c0 < chunks; c0 += nwarp * 128) {
            uint4 va[4], vb[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const long long c = c0 + i * 32 + lane;
                if (c < chunks) {
                    va[i] = a4[c];
                    vb[i] = b4[c];
                } else {
                    va[i] = vb[i] = make_uint4(0u, 0u, 0u, 0u);
                }
            }
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const uint32_t la = nz16(va[i]), lb = nz16(vb[i]);
                const uint32_t ha = __shfl_down_sync(0xffffffffu, la, 1);
                const uint32_t hb = __shfl_down_sync(0xffffffffu, lb, 1);
                const long long c = c0 + i * 32 + lane;
                if ((lane & 1) == 0 && c < chunks) {
                    const long long t = c >> 1;
                    const uint32_t wa = la | (ha << 16), wb = lb | (hb << 16);
                    P.pa[t] = wa;
                    P.pb[t] = wb;
                    const long long r = t / wxf;
                    acc.add(wa, wb, r, (int)(t - r * wxf), H);
                }
            }
        }
    } else {
        for (long long t = w_lo + tid; t < total; t += nthr) {
            const long long r = t / wxf;
            const int w = (int)(t - r * wxf);
            const long long base = r * W + 32LL * w;
            const long long ch = base >> 4;
            const int off = (int)(base & 15);
            const int nbits = min(32, W - 32 * w);
            const uint32_t keep = nbits == 32 ? 0xffffffffu : ((1u << nbits) - 1u);
            uint64_t va = chunk_bits(P.a, ch, nbytes, aligned) |
                          ((uint64_t)chunk_bits(P.a, ch + 1, nbytes, aligned) << 16);
            uint64_t vb = chunk_bits(P.b, ch, nbytes, aligned) |
                          ((uint64_t)chunk_bits(P.b, ch + 1, nbytes, aligned) << 16);
            if (off) {
                va |= (uint64_t)chunk_bits(P.a, ch + 2, nbytes, aligned) << 32;
                vb |= (uint64_t)chunk_bits(P.b, ch + 2, nbytes, aligned) << 32;
            }
            const uint32_t wa = (uint32_t)(va >> off) & keep;
            const uint32_t wb = (uint32_t)(vb >> off) & keep;
            P.pa[t] = wa;
            P.pb[t] = wb;
            acc.add(wa, wb, r, w, H);
        }
    }
    flush_acc(P, acc);
}

__device__ __forceinline__ void flush_acc(const PairDesc& P, const PackAcc& acc) {
    unsigned long long na = warp_sum_u64(acc.na), nb = warp_sum_u64(acc.nb), nab = warp_sum_u64(acc.nab);
    int bb[6];
#pragma unroll
    for (int i = 0; i < 6; i += 2) {
        bb[i] = warp_min(acc.bb[i]);
        bb[i + 1] = warp_max(acc.bb[i + 1]);
    }
    if ((threadIdx.x & 31) == 0) {
        PairInfo* I = P.info;
        if (na) atomicAdd(&I->n_a, na);
        if (nb) atomicAdd(&I->n_b, nb);
        if (nab) atomicAdd(&I->n_ab, nab);
        if (bb[1] >= 0) {
#pragma unroll
            for (int i = 0; i < 6; i += 2) {
                atomicMin(&I->bb[i], bb[i]);
                atomicMax(&I->bb[i + 1], bb[i + 1]);
            }
        }
    }
}

struct Domain {
    int ox, oy, oz, wv, h, d, wx0, wx, pitch;
};

__device__ __forceinline__ Domain make_domain(const PairDesc& P, const PairInfo& I) {
    Domain m;
    if (P.se == 0) {
        // 6-neighbour element: every shortest path between two voxels of the
        // bounding box of A u B is monotone and stays in it, so cropping to it
        // (x widened to whole words, still inside the volume) is exact.
        m.wx0 = I.bb[0] >> 5;
        const int wx1 = I.bb[1] >> 5;
        m.ox = 32 * m.wx0;
        m.wv = min(P.W, 32 * (wx1 + 1)) - m.ox;
        m.oy = I.bb[2];
        m.h = I.bb[3] - I.bb[2] + 1;
        m.oz = I.bb[4];
        m.d = I.bb[5] - I.bb[4] + 1;
    } else {
        // 18-neighbour element: shortest paths may step outside the box
        // (e.g. (1,1,1)+(1,-1,1) reaches (2,0,2) in 2 steps), so the domain
        // is the whole volume, as in the reference.
        m.wx0 = 0;
        m.ox = m.oy = m.oz = 0;
        m.wv = P.W;
        m.h = P.H;
        m.d = P.D;
    }
    m.wx = (m.wv + 31) >> 5;
    m.pitch = (m.wx + 3) & ~3;
    return m;
}

__device__ __forceinline__ void setup_tile(const PairDesc& P, long long tile_in_pair, Job* jobs, JobState* states,
                                           unsigned long long* queue0, Ctl* ctl, int g0, int bxw, int by, int bz);

// 1D grid, block 256: CTAs stride over the tiles of all pairs; tile 0 of a
// pair also writes its job descriptors.  A pair's tiles cover its full
// volume's word count, an upper bound of its domain.
__global__ void __launch_bounds__(256) setup_kernel(const PairDesc* __restrict__ descs, int npairs, long long ntiles,
                                                    Job* jobs, JobState* states, unsigned long long* queue0,
                                                    Ctl* ctl, int g0, int bxw, int by, int bz, int stats) {
    (void)stats;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int pi = pair_of_tile(descs, npairs, tile, true);
        setup_tile(descs[pi], tile - descs[pi].stile0, jobs, states, queue0, ctl, g0, bxw, by, bz);
    }
}

__device__ __forceinline__ void setup_tile(const PairDesc& P, long long tile_in_pair, Job* jobs, JobState* states,
                                           unsigned long long* queue0, Ctl* ctl, int g0, int bxw, int by, int bz) {
    const PairInfo I = *P.info;
    const bool empty_a = I.n_a == 0, empty_b = I.n_b == 0;
    const unsigned long long rem[2] = {I.n_b - I.n_ab, I.n_a - I.n_ab};
    const long long cap = domain_cap_words(P.W, P.H, P.D);  // this pair's tiles cover [0, cap) words
    const long long ntiles_pair = tiles_of(cap);
    const long long w_lo = tile_in_pair * kTileWords, w_hi = min(cap, w_lo + kTileWords);
    const long long tid0 = threadIdx.x;
    const long long nthr = blockDim.x;
    const bool first = tile_in_pair == 0;
    const int kmax = P.kmax;
    // histograms are zeroed for every pair
    if (first)
        for (long long t = tid0; t < 2LL * (kmax + 1); t += nthr) P.hist[t / (kmax + 1)][t % (kmax + 1)] = 0ull;
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
        return;
    }
    const Domain m = make_domain(P, I);
    const int nbx = (m.wx + bxw - 1) / bxw, nby = (m.h + by - 1) / by, nbz = (m.d + bz - 1) / bz;
    const long long nbricks = (long long)nbx * nby * nbz;
    if (first && tid0 == 0) {
        for (int j = 0; j < 2; ++j) {
            Job& J = jobs[P.job0 + j];
            J.buf[0] = P.jb[j][0];
            J.buf[1] = P.jb[j][1];
            J.U = P.jb[j][2];
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
    const long long words = min((long long)m.pitch * m.h * m.d, w_hi);
    const bool act0 = rem[0] > 0, act1 = rem[1] > 0;
    for (long long t = w_lo + tid0; t < words; t += nthr) {
        const long long r = t / m.pitch;
        const int w = (int)(t - r * m.pitch);
        uint32_t a = 0, b = 0;
        if (w < m.wx) {
            const int yl = (int)(r % m.h), zl = (int)(r / m.h);
            const long long src = ((long long)(m.oz + zl) * P.H + (m.oy + yl)) * P.wxf + m.wx0 + w;
            a = __ldg(P.pa + src);
            b = __ldg(P.pb + src);
        }
        if (act0) { P.jb[0][0][t] = a; P.jb[0][1][t] = a; P.jb[0][2][t] = b & ~a; }
        if (act1) { P.jb[1][0][t] = b; P.jb[1][1][t] = b; P.jb[1][2][t] = a & ~b; }
    }
    // First step of each active job: every brick of its domain (one
    // warp-aggregated append per 32 bricks).
    // the bricks are split evenly over the pair's tiles
    const int lane = threadIdx.x & 31;
    const long long gwarp = tid0 >> 5, nwarps = nthr >> 5;
    const long long b_per = (nbricks + ntiles_pair - 1) / ntiles_pair;
    const long long b_lo = tile_in_pair * b_per, b_hi = min(nbricks, b_lo + b_per);
    for (int j = 0; j < 2; ++j) {
        if (!(j == 0 ? act0 : act1)) continue;
        for (long long b0 = b_lo + gwarp * 32; b0 < b_hi; b0 += nwarps * 32) {
            const long long t = b0 + lane;
            const bool have = t < b_hi;
            const unsigned mball = __ballot_sync(0xffffffffu, have);
            unsigned base = 0;
            if (lane == 0) base = atomicAdd(&ctl->qcount[g0 % 3], (unsigned)__popc(mball));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (have)
                queue0[base + __popc(mball & ((1u << lane) - 1u))] =
                    make_entry(P.epoch, (uint32_t)(P.job0 + j), (uint32_t)t);
        }
    }
}

// Instrumented runs: zero the per-tile stamps and per-step tile counters.
__global__ void zero_i32_kernel(int32_t* p, long long n) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x)
        p[t] = 0;
}

// Per-voxel maps: -1 outside the mask, 0 on the overlap, and (filled later by
// the dilation) the distance on voxels of one mask outside the other.
__global__ void map_init_kernel(const PairDesc* __restrict__ descs, int32_t* map_a, int32_t* map_b) {
    const PairDesc& P = descs[0];
    const long long n = (long long)P.W * P.H * P.D;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const bool a = P.a[t] != 0, b = P.b[t] != 0;
        map_a[t] = a ? (b ? 0 : -2) : -1;  // -2: to be filled by the dilation
        map_b[t] = b ? (a ? 0 : -2) : -1;
    }
}

}  // namespace hdk

// ---- launch wrappers (called from the host orchestration) -----------------
namespace hdk {

cudaError_t launch_pack(const PairDesc* d_descs, int npairs, long long ntiles, int grid, cudaStream_t s) {
    pack_kernel<<<grid, 256, 0, s>>>(d_descs, npairs, ntiles);
    return cudaGetLastError();
}

cudaError_t launch_setup(const PairDesc* d_descs, int npairs, long long ntiles, int grid, Job* jobs,
                         JobState* states, unsigned long long* queue0, Ctl* ctl, int g0, int bxw, int by, int bz,
                         int stats, cudaStream_t s) {
    setup_kernel<<<grid, 256, 0, s>>>(d_descs, npairs, ntiles, jobs, states, queue0, ctl, g0, bxw, by, bz, stats);
    return cudaGetLastError();
}

cudaError_t launch_zero_i32(int32_t* p, long long n, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    long long blocks = (n + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    zero_i32_kernel<<<(int)blocks, 256, 0, s>>>(p, n);
    return cudaGetLastError();
}

cudaError_t launch_map_init(const PairDesc* d_descs, int32_t* map_a, int32_t* map_b, long long n,
                            cudaStream_t s) {
    long long blocks = (n + 255) / 256;
    if (blocks > 8192) blocks = 8192;
    map_init_kernel<<<(int)blocks, 256, 0, s>>>(d_descs, map_a, map_b);
    return cudaGetLastError();
}

}  // namespace hdk
