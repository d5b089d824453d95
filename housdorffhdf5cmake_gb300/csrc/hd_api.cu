// hd_api.cu -- host orchestration behind the C ABI (include/hd/hd.h).
//
// Replaces HausdorffDistance::computeDistance (forBench/HausdorffDistance.cu:
// 101-187) and the prototype's orchestration (hello.cu:892-1055, 1910-2062).
// Per call: one upload of descriptors, the packing launch, the set-up launch,
// ONE cooperative launch of the persistent dilation kernel that runs every
// step on the device, and one read-back of a few hundred bytes.  No host
// round trip per step (the reference does a blocking symbol read per step at
// :167), no cudaDeviceReset, no exit.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "hd/hd.h"
#include "hd_internal.h"
#include "hd_kernels.h"

using hdk::Ctl;
using hdk::Job;
using hdk::JobState;
using hdk::PairDesc;
using hdk::PairInfo;

namespace hdh {

namespace {
constexpr size_t kAlign = 256;
inline size_t align_up(size_t x, size_t a = kAlign) { return (x + a - 1) / a * a; }
constexpr long long kMaxWords = (1LL << 31) - 1;
}  // namespace

cudaError_t DeviceArena::ensure(size_t n) {
    if (n <= cap) return cudaSuccess;
    // asynchronous calls may still use the old buffer on some stream
    if (ptr) cudaDeviceSynchronize();
    release();
    size_t want = std::max(n, cap + cap / 4);
    cudaError_t e = cudaMalloc(&ptr, want);
    if (e != cudaSuccess) {
        cudaGetLastError();
        ptr = nullptr;
        e = cudaMalloc(&ptr, n);
        if (e != cudaSuccess) {
            cudaGetLastError();
            ptr = nullptr;
            cap = 0;
            return e;
        }
        want = n;
    }
    cap = want;
    return cudaSuccess;
}

void DeviceArena::release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
}

cudaError_t PinnedArena::ensure(size_t n) {
    if (n <= cap) return cudaSuccess;
    release();
    const size_t want = std::max(n, (size_t)1 << 16);
    cudaError_t e = cudaHostAlloc(&ptr, want, cudaHostAllocDefault);
    if (e != cudaSuccess) {
        cudaGetLastError();
        ptr = nullptr;
        cap = 0;
        return e;
    }
    cap = want;
    return cudaSuccess;
}

void PinnedArena::release() {
    if (ptr) cudaFreeHost(ptr);
    ptr = nullptr;
    cap = 0;
}

DeviceGuard::DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) {
        cudaGetLastError();
        prev = -1;
    }
    ok = cudaSetDevice(dev) == cudaSuccess;
    if (!ok) cudaGetLastError();
}

DeviceGuard::~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
}

hd_status set_error(hd_context* ctx, hd_status st, const char* fmt, ...) {
    if (ctx) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        ctx->last_error = buf;
    }
    return st;
}

hd_status cuda_fail(hd_context* ctx, cudaError_t e, const char* where) {
    const hd_status st = (e == cudaErrorMemoryAllocation) ? HD_ERR_OOM : HD_ERR_CUDA;
    set_error(ctx, st, "%s: %s (%s)", where, cudaGetErrorString(e), cudaGetErrorName(e));
    cudaGetLastError();
    return st;
}

hd_status check_dims(hd_context* ctx, int32_t W, int32_t H, int32_t D) {
    if (W <= 0 || H <= 0 || D <= 0)
        return set_error(ctx, HD_ERR_BAD_ARG, "sizes must be positive (W=%d H=%d D=%d)", W, H, D);
    const long long wx = (W + 31) / 32;
    const long long pitch = (wx + 3) / 4 * 4;
    if (pitch * H * D > kMaxWords)
        return set_error(ctx, HD_ERR_BAD_ARG, "volume %dx%dx%d exceeds 2^31 packed words", W, H, D);
    if ((long long)W + H + D > (1 << 24))
        return set_error(ctx, HD_ERR_BAD_ARG, "volume %dx%dx%d too long", W, H, D);
    return HD_OK;
}

const uint8_t* zero_copy_ptr(hd_context* ctx, const uint8_t* p) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) == cudaSuccess) {
        if (at.type == cudaMemoryTypeHost && at.devicePointer) return (const uint8_t*)at.devicePointer;
        if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) return p;
    } else {
        cudaGetLastError();
    }
    if (ctx->pageable_ats) return p;
    return nullptr;
}

int robust_k(const uint64_t* hist, int len, uint64_t total, float p) {
    // hello.cu:1751-1758: continue while (float)total * robustnessPercent > covered.
    const float tf = (float)total * p;
    uint64_t cov = 0;
    for (int k = 0; k < len; ++k) {
        if (k > 0) cov += hist[k];
        if (!(tf > (float)cov)) return k;
    }
    return len - 1;
}

int occupancy_of(hd_context* ctx, const void* fn, int threads, int smem) {
    auto it = ctx->occupancy.find(fn);
    if (it != ctx->occupancy.end()) return it->second;
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, threads, smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    n = std::max(1, n);
    ctx->occupancy[fn] = n;
    return n;
}

namespace {

// Driver entry points of the green-context API, through the runtime (no
// link against the driver library).
template <class F>
F driver_fn(const char* name, int version) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion(name, &fn, version, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return reinterpret_cast<F>(fn);
}

using GreenDestroyFn = CUresult (*)(CUgreenCtx);

}  // namespace

// The split path's SM partitions (green contexts; the granularity is 8 SMs
// on GB300).  One dilation partition: packing and set-up on 48 SMs, each
// pair's dilation on the other 104 in turn.  Two or three: packing and
// set-up on 40 / 56 SMs, the rest in equal groups (56 / 32 SMs),
// consecutive pairs dilating side by side (workspace i on group i % parts,
// two workspaces per group in turn).  A single pair's dilation is
// latency-bound: on fewer SMs it takes longer, but much less than in
// proportion (the 512x512x256 pairs: 0.124 / 0.077 ms on 104 SMs, 0.178 /
// 0.077 ms on 56, 0.179 ms on average over both on 32), so side by side the groups
// finish more pairs per second.  Measured on those two pairs alternating
// (0.142 ms per pair unsplit): one partition with 24 / 32 / 48 / 64
// packing SMs 0.155 / 0.127 / 0.107 / 0.121 ms per pair; two partitions
// with 40 / 56 packing SMs (groups of 56 / 48) 0.094 / 0.102 ms, with one
// workspace per group 0.137 ms (a packing waited for the dilation before
// last in its group); three with 56 / 32 packing SMs (groups of 32 / 40)
// 0.080 / 0.115 ms: packing and set-up on 56 SMs (0.073 ms a pair) set the
// pace.  A lone pair's latency is higher on fewer dilation SMs (0.30 ms
// on 56 against 0.23 ms on 104).
constexpr int kSplitDilations = 3;
constexpr unsigned kSplitPrepSms[hd_context::kMaxDilationParts] = {48, 40, 56};  // by dilation partitions

// HD_SPLIT_DILATIONS (1 to 3) in the environment overrides the dilation
// partitions, HD_SPLIT_SMS the packing SMs: 0 = no split (profilers that
// cannot follow kernels into green contexts), else the SMs to give to
// packing and set-up (several partitions: the rest in equal groups, rounded
// up to the granularity).
bool split_ready(hd_context* ctx) {
    constexpr int kMax = hd_context::kMaxDilationParts;
    hd_context::Split& sp = ctx->split;
    if (sp.state) return sp.state > 0;
    sp.state = -1;
    int parts = kSplitDilations;
    if (const char* env = std::getenv("HD_SPLIT_DILATIONS"))
        parts = (int)std::min<long>(std::max<long>(std::strtol(env, nullptr, 10), 1), kMax);
    unsigned prep_want = kSplitPrepSms[parts - 1];
    if (const char* env = std::getenv("HD_SPLIT_SMS")) {
        const long v = std::strtol(env, nullptr, 10);
        if (v <= 0) return false;
        prep_want = (unsigned)v;
    }
    auto get_dev = driver_fn<CUresult (*)(CUdevice*, int)>("cuDeviceGet", 2000);
    auto get_res = driver_fn<CUresult (*)(CUdevice, CUdevResource*, CUdevResourceType)>("cuDeviceGetDevResource", 12040);
    auto split = driver_fn<CUresult (*)(CUdevResource*, unsigned*, const CUdevResource*, CUdevResource*, unsigned,
                                        unsigned)>("cuDevSmResourceSplitByCount", 12040);
    auto make_desc = driver_fn<CUresult (*)(CUdevResourceDesc*, CUdevResource*, unsigned)>("cuDevResourceGenerateDesc",
                                                                                         12040);
    auto create = driver_fn<CUresult (*)(CUgreenCtx*, CUdevResourceDesc, CUdevice, unsigned)>("cuGreenCtxCreate", 12040);
    auto stream = driver_fn<CUresult (*)(CUstream*, CUgreenCtx, unsigned, int)>("cuGreenCtxStreamCreate", 12050);
    if (!get_dev || !get_res || !split || !make_desc || !create || !stream) return false;
    CUdevice dev;
    CUdevResource all{};
    if (get_dev(&dev, ctx->device) != CUDA_SUCCESS || get_res(dev, &all, CU_DEV_RESOURCE_TYPE_SM) != CUDA_SUCCESS)
        return false;
    if (all.sm.smCount < prep_want + 64) return false;  // too few SMs to give some away
    // d[0]: packing and set-up, d[1 + p]: dilation partition p
    CUdevResourceDesc d[1 + kMax];
    unsigned sms[kMax] = {}, prep_sms = 0;
    bool ok;
    if (parts > 1) {
        // equal dilation groups split off the whole device (a split's
        // remainder cannot be split again; the group size rounds up to the
        // granularity), the remainder packing
        CUdevResource grp[kMax]{}, left{};
        unsigned n = (unsigned)parts;
        ok = split(grp, &n, &all, &left, 0, (all.sm.smCount - prep_want) / parts) == CUDA_SUCCESS &&
             n == (unsigned)parts && left.sm.smCount >= 8;
        ok = ok && make_desc(&d[0], &left, 1) == CUDA_SUCCESS;
        for (int q = 0; q < parts && ok; ++q) {
            ok = make_desc(&d[1 + q], &grp[q], 1) == CUDA_SUCCESS;
            sms[q] = grp[q].sm.smCount;
        }
        prep_sms = left.sm.smCount;
    } else {
        CUdevResource prep{}, rest{};
        unsigned groups = 1;
        ok = split(&prep, &groups, &all, &rest, 0, prep_want) == CUDA_SUCCESS && groups == 1;
        ok = ok && make_desc(&d[0], &prep, 1) == CUDA_SUCCESS && make_desc(&d[1], &rest, 1) == CUDA_SUCCESS;
        sms[0] = rest.sm.smCount;
        prep_sms = prep.sm.smCount;
    }
    const int ng = 1 + parts;
    CUgreenCtx g[1 + kMax] = {};
    CUstream st[1 + kMax] = {};
    for (int i = 0; i < ng && ok; ++i) ok = create(&g[i], d[i], dev, CU_GREEN_CTX_DEFAULT_STREAM) == CUDA_SUCCESS;
    for (int i = 0; i < ng && ok; ++i) ok = stream(&st[i], g[i], CU_STREAM_NON_BLOCKING, 0) == CUDA_SUCCESS;
    cudaError_t e = ok ? cudaSuccess : cudaErrorUnknown;
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sp.caller, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sp.prep_done, cudaEventDisableTiming);
    for (int i = 0; i < hd_context::Split::kWorkspaces && e == cudaSuccess; ++i)
        e = cudaEventCreateWithFlags(&sp.ws_free[i], cudaEventDisableTiming);
    if (ctx->opt.record_timings)
        for (int i = 0; i < 5 && e == cudaSuccess; ++i) e = cudaEventCreate(&sp.ev[i]);
    for (int i = 0; i < ng; ++i) sp.green[i] = g[i];
    sp.prep = (cudaStream_t)st[0];
    for (int q = 0; q < parts; ++q) sp.solve[q] = (cudaStream_t)st[1 + q];
    if (e != cudaSuccess) {
        cudaGetLastError();
        split_release(ctx);
        sp.state = -1;
        return false;
    }
    for (int q = 0; q < parts; ++q) sp.solve_sms[q] = (int)sms[q];
    sp.prep_sms = (int)prep_sms;
    sp.parts = parts;
    sp.nws = 2 * parts;
    sp.state = 1;
    return true;
}

void split_release(hd_context* ctx) {
    hd_context::Split& sp = ctx->split;
    for (cudaStream_t& s : sp.solve)
        if (s) {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    if (sp.prep) {
        cudaStreamSynchronize(sp.prep);
        cudaStreamDestroy(sp.prep);
    }
    for (cudaEvent_t ev : {sp.caller, sp.prep_done, sp.ev[0], sp.ev[1], sp.ev[2], sp.ev[3], sp.ev[4]})
        if (ev) cudaEventDestroy(ev);
    for (cudaEvent_t ev : sp.ws_free)
        if (ev) cudaEventDestroy(ev);
    auto destroy = driver_fn<GreenDestroyFn>("cuGreenCtxDestroy", 12040);
    for (void* g : sp.green)
        if (g && destroy) destroy((CUgreenCtx)g);
    sp = hd_context::Split{};
}

// Makes `st` wait for the latest dilation in every workspace of the split
// path (an event never recorded is no wait).
cudaError_t wait_split_dilations(hd_context* ctx, cudaStream_t st) {
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < hd_context::Split::kWorkspaces && e == cudaSuccess; ++i)
        if (ctx->split.ws_free[i]) e = cudaStreamWaitEvent(st, ctx->split.ws_free[i], 0);
    return e;
}

namespace {

struct PairPlan {
    int wxf;
    long long full_words;   // packed full volume, one mask
    long long dom_words;    // domain capacity (pitch_full * H * D), one buffer
    long long bricks;       // per job, upper bound
    int kmax;
    long long tiles;        // full-volume 32^3 tiles (instrumented runs)
    size_t off_pa, off_pb, off_jb[2][3], off_in_a, off_in_b, off_hist, off_tstamp[2], off_tcount[2];
    unsigned long long brick0;
};

}  // namespace

hd_status decode_result(const hdk::PairInfo& I, const hdk::JobState& s0, const hdk::JobState& s1,
                        const uint64_t* hist_ab, const uint64_t* hist_ba, int kp1, int iters, int err,
                        float pct, hd_result* out) {
    // s0 dilates A and covers B (distances of B's voxels); s1 the reverse.
    hd_result& r = *out;
    std::memset(&r, 0, sizeof r);
    r.n_a = I.n_a;
    r.n_b = I.n_b;
    r.n_a_not_b = I.n_a - I.n_ab;
    r.n_b_not_a = I.n_b - I.n_ab;
    r.iterations = iters;
    if (I.n_a == 0 && I.n_b == 0) {
        r.status = HD_OK;
        return HD_OK;
    }
    if (I.n_a == 0 || I.n_b == 0) {
        r.status = HD_EMPTY_MASK;
        r.hd = r.hd_ab = r.hd_ba = r.hd_robust = -1;
        r.avg_hd = std::nan("");
        return HD_EMPTY_MASK;
    }
    int st = err;
    if (!st) st = s0.status ? s0.status : s1.status;
    if (!st && (s0.remaining != 0 || s1.remaining != 0)) st = HD_ERR_ITER_LIMIT;
    r.status = st;
    r.hd_ba = s0.hd;
    r.sum_ba = s0.sum;
    r.hd_ab = s1.hd;
    r.sum_ab = s1.sum;
    r.hd = std::max(r.hd_ab, r.hd_ba);
    r.avg_hd = (double)(r.sum_ab + r.sum_ba) / (double)(r.n_a + r.n_b);
    r.hd_robust = std::max(robust_k(hist_ab, kp1, r.n_a_not_b, pct), robust_k(hist_ba, kp1, r.n_b_not_a, pct));
    if (st != HD_OK) r.hd = r.hd_ab = r.hd_ba = r.hd_robust = -1;
    return (hd_status)st;
}

Shape pick_shape(hd_context* ctx, int se, const PairIn* pairs, int n) {
    // built-in default (the autotuner's winners on GB300): the blocked kernel
    // with 4 x (32 - 2 steps) x 8 bricks; 4 steps per barrier for a single
    // pair (fewest barriers), 2 for batches (the work per barrier is large)
    Shape sh;
    double vox = 0;
    for (int i = 0; i < n; ++i) vox += (double)pairs[i].W * pairs[i].H * pairs[i].D;
    vox /= std::max(1, n);
    sh.steps = n <= 1 ? 4 : 2;
    auto it = ctx->tune.entries.find(tune_key(se, vox, n));
    if (it != ctx->tune.entries.end()) sh = it->second.shape;
    const hd_options& o = ctx->opt;
    if (o.kernel == 1 || o.kernel == 2) sh.kernel = o.kernel;
    if (o.kernel == 0 && o.brick_x_words > 0 && o.steps_per_barrier == 0) sh.kernel = 1;
    if (o.brick_x_words > 0) sh.bxw = o.brick_x_words;
    if (o.brick_z > 0) sh.bz = o.brick_z;
    if (o.steps_per_barrier > 0) sh.steps = o.steps_per_barrier;
    if (o.ctas_per_sm > 0) sh.ctas_per_sm = o.ctas_per_sm;
    sh.finish();
    return sh;
}

const void* solve_fn_of(int se, const Shape& sh) {
    if (sh.kernel == 2) return hdk::solve_tb_kernel_ptr(se, sh.steps, sh.bz);
    return hdk::solve_kernel_ptr(se, sh.bxw, sh.bz);
}

hd_status run_pairs(hd_context* ctx, const PairIn* pairs, int n, cudaStream_t s, const RunOpts& ro,
                    hd_result* out) {
    if (n <= 0) return HD_OK;
    if (n > hdk::kMaxPairsPerLaunch) return set_error(ctx, HD_ERR_BAD_ARG, "too many pairs in one launch");
    const int se = ro.se;
    const bool stats = ro.stats != 0;
    Shape sh = ro.force_shape ? ro.shape : pick_shape(ctx, se, pairs, n);
    if (stats || ro.map_a || ro.map_b) {
        // instrumented runs and per-voxel maps are implemented by the one-step kernel
        if (sh.kernel != 1) {
            sh.kernel = 1;
            sh.bxw = 4;
            sh.bz = 8;
        }
    }
    sh.finish();
    if (sh.order == 1 && n > 1 && !ro.ordered && !ro.async_out) {
        // largest pairs first (stable): their bricks take the lowest ids,
        // their packing and set-up tiles come first and so do their entries
        // in the first queue; results go back to the caller's order
        std::vector<int> perm(n);
        for (int i = 0; i < n; ++i) perm[i] = i;
        std::stable_sort(perm.begin(), perm.end(), [&](int x, int y) {
            return (long long)pairs[x].W * pairs[x].H * pairs[x].D > (long long)pairs[y].W * pairs[y].H * pairs[y].D;
        });
        std::vector<PairIn> pp(n);
        for (int i = 0; i < n; ++i) pp[i] = pairs[perm[i]];
        std::vector<hd_result> tmp(n);
        RunOpts r2 = ro;
        r2.force_shape = true;
        r2.shape = sh;
        r2.ordered = true;
        const hd_status st = run_pairs(ctx, pp.data(), n, s, r2, tmp.data());
        for (int i = 0; i < n; ++i) out[perm[i]] = tmp[i];
        return st;
    }
    const void* solve_fn = solve_fn_of(se, sh);
    if (!solve_fn)
        return set_error(ctx, HD_ERR_BAD_ARG, "kernel %d with %d words x %d rows x %d planes (%d steps) not compiled in",
                         sh.kernel, sh.bxw, sh.by, sh.bz, sh.steps);
    const int bxw = sh.bxw, by = sh.by, bz = sh.bz, cps = sh.ctas_per_sm;

    // ---- layout --------------------------------------------------------
    std::vector<PairPlan> plan(n);
    size_t cur = 0;
    auto take = [&](size_t bytes) {
        const size_t o = cur;
        cur = align_up(cur + std::max<size_t>(bytes, 1));
        return o;
    };
    const size_t off_ctl = take(sizeof(Ctl));
    const size_t off_states = take(sizeof(JobState) * 2 * n);
    const size_t off_infos = take(sizeof(PairInfo) * n);
    const size_t off_descs = take(sizeof(PairDesc) * n);
    const size_t upload_bytes = cur;           // [ctl .. descs]
    const size_t off_jobs = take(sizeof(Job) * 2 * n);
    // results decoded by the persistent launch (synchronous calls read them
    // back; asynchronous ones write to the caller's array instead)
    const size_t off_out = take(sizeof(hd_result) * n);
    size_t hist_words = 0;
    unsigned long long total_bricks = 0;
    int kmax_all = 0;
    for (int i = 0; i < n; ++i) {
        PairPlan& q = plan[i];
        const PairIn& P = pairs[i];
        q.wxf = (P.W + 31) / 32;
        q.full_words = (long long)hdk::packed_pitch(P.W) * P.H * P.D;
        const long long pitch = (q.wxf + 3) / 4 * 4;
        q.dom_words = pitch * P.H * P.D;
        q.bricks = (long long)((q.wxf + bxw - 1) / bxw) * ((P.H + by - 1) / by) * ((P.D + bz - 1) / bz);
        int kmax = P.W + P.H + P.D;
        if (ctx->opt.max_iterations > 0) kmax = std::min(kmax, ctx->opt.max_iterations);
        q.kmax = kmax;
        kmax_all = std::max(kmax_all, kmax);
        q.tiles = (long long)((P.W + 31) / 32) * ((P.H + 31) / 32) * ((P.D + 31) / 32);
        q.brick0 = total_bricks;
        total_bricks += 2ULL * (unsigned long long)q.bricks;
        hist_words += 2ULL * (kmax + 1);
    }
    const size_t off_hist = take(sizeof(uint64_t) * hist_words);
    size_t hcur = 0;
    for (int i = 0; i < n; ++i) {
        plan[i].off_hist = off_hist + hcur * sizeof(uint64_t);
        hcur += 2ULL * (plan[i].kmax + 1);
    }
    const size_t qbytes = sizeof(unsigned long long) * std::max<unsigned long long>(total_bricks, 1);
    const size_t off_q[3] = {take(qbytes), take(qbytes), take(qbytes)};
    for (int i = 0; i < n; ++i) {
        PairPlan& q = plan[i];
        q.off_pa = take(4ULL * q.full_words);
        q.off_pb = take(4ULL * q.full_words);
        for (int j = 0; j < 2; ++j)
            for (int b = 0; b < 3; ++b) q.off_jb[j][b] = take(4ULL * q.dom_words);
        const size_t nb = (size_t)pairs[i].W * pairs[i].H * pairs[i].D;
        q.off_in_a = (pairs[i].host_a && !ro.async_out) ? take(nb) : 0;
        q.off_in_b = (pairs[i].host_b && !ro.async_out) ? take(nb) : 0;
        if (stats) {
            for (int j = 0; j < 2; ++j) {
                q.off_tstamp[j] = take(sizeof(int32_t) * q.tiles);
                q.off_tcount[j] = take(sizeof(uint64_t) * (q.kmax + 1));
            }
        }
    }
    const size_t total_bytes = cur;
    const size_t pinned_bytes = upload_bytes + sizeof(hd_result) * n + (stats ? sizeof(uint64_t) * hist_words : 0);

    // Pipelined single pairs of up to 2^26 voxels run on split SMs: their
    // dilation is latency-bound and fits fewer SMs, so later pairs' packing
    // and set-up run beside it, on their own SMs and workspaces, and so do
    // consecutive pairs' dilations, on separate SM groups.  Streams: sq
    // (uploads, packing, set-up) and sv (the dilation, on the workspace's
    // group), both the caller's stream otherwise.  The caller's stream waits
    // for the dilations only at a flush (or the next other call).
    const bool async = ro.async_out != nullptr;
    const bool split = async && ro.pipelined && n == 1 && sh.kernel == 2 &&
                       (double)pairs[0].W * pairs[0].H * pairs[0].D <= (double)(1 << 26) && split_ready(ctx);
    if (!split && ctx->split.pending) {  // every other call follows the pipelined ones
        const cudaError_t e0 = wait_split_dilations(ctx, s);
        if (e0 != cudaSuccess) return cuda_fail(ctx, e0, "pipeline flush");
        ctx->split.pending = false;
    }
    // the workspace alternates only once a dilation has been launched in it
    const int ws = split ? ctx->split.next : 0;
    const int part = split ? ws % ctx->split.parts : 0;  // the split path's dilation partition
    DeviceArena& arena = ws ? ctx->ws_arena[ws - 1] : ctx->arena;
    cudaStream_t sq = split ? ctx->split.prep : s, sv = split ? ctx->split.solve[part] : s;
    const int prep_sms = split ? ctx->split.prep_sms : ctx->sm_count;
    // Growing a buffer frees the old one after cudaDeviceSynchronize, which
    // waits for the primary context's streams only: the split path's streams
    // belong to green contexts and may still use it, so drain them first.
    auto drain_split = [&]() {
        if (ctx->split.state > 0) {
            for (cudaStream_t q : ctx->split.solve)
                if (q) cudaStreamSynchronize(q);
            cudaStreamSynchronize(ctx->split.prep);
        }
    };

    if (total_bytes > arena.cap) drain_split();
    cudaError_t e = arena.ensure(total_bytes);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "device workspace");
    if (split) {
        // the packing waits for the caller's earlier work and for the
        // dilation that last used this workspace
        e = cudaEventRecord(ctx->split.caller, s);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(sq, ctx->split.caller, 0);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(sq, ctx->split.ws_free[ws], 0);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "split streams");
    }
    if (total_bricks > ctx->stamp_slots || ctx->g_next > (1 << 30)) {
        const size_t want = std::max<size_t>(total_bricks, ctx->stamp_slots);
        bool grow = sizeof(int32_t) * want > ctx->stamps.cap;
        for (const DeviceArena& a : ctx->part_stamps) grow = grow || sizeof(int32_t) * want > a.cap;
        if (grow) drain_split();
        e = ctx->stamps.ensure(sizeof(int32_t) * want);
        for (DeviceArena& a : ctx->part_stamps)
            if (e == cudaSuccess) e = a.ensure(sizeof(int32_t) * want);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "brick stamps");
        // the reset follows every dilation that used the stamps (split
        // path: the latest one in each workspace, which the caller's stream
        // may not have waited for yet; the others precede the caller event
        // that sq waits for) and precedes this call's
        if (split && ctx->split.pending) {
            e = wait_split_dilations(ctx, sq);
        }
        if (e == cudaSuccess) e = cudaMemsetAsync(ctx->stamps.ptr, 0, sizeof(int32_t) * want, sq);
        for (DeviceArena& a : ctx->part_stamps)
            if (e == cudaSuccess) e = cudaMemsetAsync(a.ptr, 0, sizeof(int32_t) * want, sq);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "stamp reset");
        ctx->stamp_slots = want;
        ctx->g_next = 1;
    }
    int slot = -1;
    if (async) {
        // first asynchronous call: every staging buffer and event at once
        // (pinned allocations are slow; later calls should not meet one)
        if (!ctx->async_done[0]) {
            for (int i = 0; i < hd_context::kAsyncSlots && e == cudaSuccess; ++i) {
                e = cudaEventCreateWithFlags(&ctx->async_done[i], cudaEventDisableTiming);
                if (e == cudaSuccess) e = ctx->async_stage[i].ensure(std::max<size_t>(upload_bytes, 1 << 16));
            }
            if (e != cudaSuccess) return cuda_fail(ctx, e, "staging buffers");
        }
        // a staging buffer whose previous upload has run
        slot = ctx->async_next;
        ctx->async_next = (ctx->async_next + 1) % hd_context::kAsyncSlots;
        e = cudaEventSynchronize(ctx->async_done[slot]);
        if (e == cudaSuccess) e = ctx->async_stage[slot].ensure(upload_bytes);
    } else {
        e = ctx->pinned.ensure(pinned_bytes);
    }
    if (e != cudaSuccess) return cuda_fail(ctx, e, "pinned staging");

    char* dbase = (char*)arena.ptr;
    char* hbase = (char*)(async ? ctx->async_stage[slot].ptr : ctx->pinned.ptr);
    const int g0 = ctx->g_next;
    long long pack_tiles = 0, setup_tiles = 0;
    // blocked kernel: a single pair reads the packed masks in place unless
    // that adds a brick column, a batch always does
    const int setup_mode =
        sh.kernel == 1 ? hdk::kSetupOneStep : (n == 1 ? hdk::kSetupBlocked : hdk::kSetupBlockedInPlace);

    // ---- asynchronous calls with host masks: copy on the copy stream ------
    const uint8_t* staged[2] = {nullptr, nullptr};
    int mb = -1;
    if (async && n == 1 && (pairs[0].host_a || pairs[0].host_b)) {
        if (!ctx->copy_stream) {
            e = cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking);
            for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
                e = cudaEventCreateWithFlags(&ctx->mask_ready[i], cudaEventDisableTiming);
                if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->mask_free[i], cudaEventDisableTiming);
            }
            if (e != cudaSuccess) return cuda_fail(ctx, e, "copy stream");
        }
        mb = ctx->mask_next;
        ctx->mask_next ^= 1;
        const size_t nb = (size_t)pairs[0].W * pairs[0].H * pairs[0].D;
        e = ctx->mask_stage[mb].ensure(2 * align_up(nb));
        if (e != cudaSuccess) return cuda_fail(ctx, e, "mask staging");
        uint8_t* sa = (uint8_t*)ctx->mask_stage[mb].ptr;
        uint8_t* sb = sa + align_up(nb);
        // the packing that read this buffer two calls ago must be done
        e = cudaStreamWaitEvent(ctx->copy_stream, ctx->mask_free[mb], 0);
        if (e == cudaSuccess && pairs[0].host_a)
            e = cudaMemcpyAsync(sa, pairs[0].host_a, nb, cudaMemcpyHostToDevice, ctx->copy_stream);
        if (e == cudaSuccess && pairs[0].host_b)
            e = cudaMemcpyAsync(sb, pairs[0].host_b, nb, cudaMemcpyHostToDevice, ctx->copy_stream);
        if (e == cudaSuccess) e = cudaEventRecord(ctx->mask_ready[mb], ctx->copy_stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(sq, ctx->mask_ready[mb], 0);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "mask copy");
        staged[0] = pairs[0].host_a ? sa : nullptr;
        staged[1] = pairs[0].host_b ? sb : nullptr;
    }

    // ---- host-side descriptors ------------------------------------------
    std::memset(hbase, 0, upload_bytes);
    PairInfo* hinfo = (PairInfo*)(hbase + off_infos);
    PairDesc* hdesc = (PairDesc*)(hbase + off_descs);
    for (int i = 0; i < n; ++i) {
        const PairIn& P = pairs[i];
        const PairPlan& q = plan[i];
        PairInfo& I = hinfo[i];
        I.bb[0] = I.bb[2] = I.bb[4] = 0x7fffffff;
        I.bb[1] = I.bb[3] = I.bb[5] = -1;
        PairDesc& Dd = hdesc[i];
        Dd.a = P.host_a ? (staged[0] ? staged[0] : (const uint8_t*)(dbase + q.off_in_a)) : P.a;
        Dd.b = P.host_b ? (staged[1] ? staged[1] : (const uint8_t*)(dbase + q.off_in_b)) : P.b;
        Dd.pa = (uint32_t*)(dbase + q.off_pa);
        Dd.pb = (uint32_t*)(dbase + q.off_pb);
        for (int j = 0; j < 2; ++j) {
            for (int b = 0; b < 3; ++b) Dd.jb[j][b] = (uint32_t*)(dbase + q.off_jb[j][b]);
            Dd.hist[j] = (unsigned long long*)(dbase + q.off_hist) + (size_t)j * (q.kmax + 1);
            Dd.brick0[j] = q.brick0 + (unsigned long long)j * q.bricks;
            Dd.tstamp[j] = stats ? (int32_t*)(dbase + q.off_tstamp[j]) : nullptr;
            Dd.tcount[j] = stats ? (unsigned long long*)(dbase + q.off_tcount[j]) : nullptr;
        }
        Dd.W = P.W;
        Dd.H = P.H;
        Dd.D = P.D;
        Dd.wxf = q.wxf;
        Dd.se = se;
        Dd.aligned = ((((uintptr_t)Dd.a) | ((uintptr_t)Dd.b)) & 15) == 0;
        Dd.kmax = q.kmax;
        Dd.job0 = 2 * i;
        Dd.info = (PairInfo*)(dbase + off_infos) + i;
        Dd.tile0 = pack_tiles;
        Dd.stile0 = setup_tiles;
        pack_tiles += hdk::pack_tiles_of(P.W, P.H, P.D);
        setup_tiles += hdk::setup_tiles_of(P.W, P.H, P.D, setup_mode, bxw, by, bz);
    }

    // ---- uploads ----------------------------------------------------------
    e = cudaMemcpyAsync(dbase, hbase, upload_bytes, cudaMemcpyHostToDevice, sq);
    if (e == cudaSuccess && async) e = cudaEventRecord(ctx->async_done[slot], sq);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "descriptor upload");
    for (int i = 0; i < n && mb < 0; ++i) {
        const size_t nb = (size_t)pairs[i].W * pairs[i].H * pairs[i].D;
        if (pairs[i].host_a) {
            e = cudaMemcpyAsync(dbase + plan[i].off_in_a, pairs[i].host_a, nb, cudaMemcpyHostToDevice, sq);
            if (e != cudaSuccess) return cuda_fail(ctx, e, "mask upload");
        }
        if (pairs[i].host_b) {
            e = cudaMemcpyAsync(dbase + plan[i].off_in_b, pairs[i].host_b, nb, cudaMemcpyHostToDevice, sq);
            if (e != cudaSuccess) return cuda_fail(ctx, e, "mask upload");
        }
    }
    if (stats) {
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < 2; ++j) {
                e = hdk::launch_zero_i32((int32_t*)(dbase + plan[i].off_tstamp[j]), plan[i].tiles, s);
                if (e == cudaSuccess)
                    e = cudaMemsetAsync(dbase + plan[i].off_tcount[j], 0,
                                        sizeof(uint64_t) * (plan[i].kmax + 1), s);
                if (e != cudaSuccess) return cuda_fail(ctx, e, "instrumentation reset");
            }
    }

    // ---- pack, set-up -----------------------------------------------------
    // one CTA per tile up to 8 per SM, then striding
    const int grid_pack = (int)std::min<long long>(std::max(prep_sms * 8, 1), pack_tiles);
    const PairDesc* ddesc = (const PairDesc*)(dbase + off_descs);
    const bool timing = ctx->opt.record_timings != 0 && ctx->ev[0] != nullptr && !async;
    if (timing) cudaEventRecord(ctx->ev[0], s);
    // the split path times its phases on the streams they run on
    const bool stime = split && ctx->opt.record_timings != 0 && ctx->split.ev[0] != nullptr;
    if (stime) cudaEventRecord(ctx->split.ev[0], sq);
    e = hdk::launch_pack(ddesc, n, pack_tiles, grid_pack, ctx->opt.label, split ? prep_sms : 0, sq);
    if (e == cudaSuccess && mb >= 0) e = cudaEventRecord(ctx->mask_free[mb], sq);  // staging buffer read
    if (e != cudaSuccess) return cuda_fail(ctx, e, "pack launch");
    Ctl* dctl = (Ctl*)(dbase + off_ctl);
    Job* djobs = (Job*)(dbase + off_jobs);
    JobState* dstates = (JobState*)(dbase + off_states);
    unsigned long long* dq[3] = {(unsigned long long*)(dbase + off_q[0]),
                                 (unsigned long long*)(dbase + off_q[1]),
                                 (unsigned long long*)(dbase + off_q[2])};
    if (timing) cudaEventRecord(ctx->ev[1], s);
    if (stime) cudaEventRecord(ctx->split.ev[1], sq);
    const bool spec = sh.kernel == 2;  // the blocked kernel reads first entries early (kSpecSlots zeroed slots)
    const int nz = spec ? (int)std::min<unsigned long long>(total_bricks, hdk::kSpecSlots) : 0;
    e = hdk::launch_setup(ddesc, n, setup_tiles, split ? prep_sms : 0, djobs, dstates, dq[g0 % 3], dctl, g0, bxw, by, bz,
                          setup_mode, sq, dq[(g0 + 1) % 3], dq[(g0 + 2) % 3], nz);
    if (e == cudaSuccess && split) {
        // the dilation follows the set-up; the caller's stream follows the
        // packing's reads of its masks (work it queues later may overwrite
        // or free them) but not the dilation
        if (stime) cudaEventRecord(ctx->split.ev[2], sq);
        e = cudaEventRecord(ctx->split.prep_done, sq);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(sv, ctx->split.prep_done, 0);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s, ctx->split.prep_done, 0);
    }
    if (e != cudaSuccess) return cuda_fail(ctx, e, "setup launch");
    if (ro.map_a || ro.map_b) {
        e = hdk::launch_map_init(ddesc, ro.map_a, ro.map_b,
                                 (long long)pairs[0].W * pairs[0].H * pairs[0].D, ctx->opt.label, s);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "map init launch");
    }

    // ---- persistent dilation ------------------------------------------------
    hdk::SolveParams sp{};
    sp.jobs = djobs;
    sp.states = dstates;
    for (int q = 0; q < 3; ++q) sp.queue[q] = dq[q];
    // the split path's dilation partitions have stamps of their own (their
    // dilations may run side by side)
    sp.stamps = (int32_t*)(part > 0 ? ctx->part_stamps[part - 1].ptr : ctx->stamps.ptr);
    sp.ctl = dctl;
    sp.map[0] = ro.map_b;  // job 0 covers B
    sp.map[1] = ro.map_a;  // job 1 covers A
    sp.map_w = pairs[0].W;
    sp.map_h = pairs[0].H;
    sp.map_d = pairs[0].D;
    sp.g0 = g0;
    sp.max_iters = kmax_all / sh.steps + 2;
    sp.stats = stats ? 1 : 0;
    sp.spread = sh.spread;
    sp.job_cache = (n == 1 && sh.kernel == 2) ? hdk::kJobCache : 0;  // a single pair's two jobs
    sp.spec_first = nz;  // slots of each queue the set-up zeroed
    sp.timeout_ns = ctx->opt.barrier_timeout_ns > 0 ? ctx->opt.barrier_timeout_ns : 10000000000LL;
    const int occ = occupancy_of(ctx, solve_fn, sh.threads, sh.smem);
    if (occ <= 0) return set_error(ctx, HD_ERR_CUDA, "dilation kernel cannot be made resident");
    const int per_sm = cps > 0 ? std::min(cps, occ) : occ;
    dim3 grid((split ? ctx->split.solve_sms[part] : ctx->sm_count) * per_sm), block(sh.threads);
    const float pct = (ctx->opt.percentile > 0.f && ctx->opt.percentile <= 1.f) ? ctx->opt.percentile : 0.95f;
    // the launch decodes the results on the device (one warp per pair, after
    // its last barrier): the per-step histograms never leave the device
    sp.descs = ddesc;
    sp.npairs = n;
    sp.pct = pct;
    sp.out = async ? ro.async_out : (hd_result*)(dbase + off_out);
    void* args[] = {&sp};
    if (timing) cudaEventRecord(ctx->ev[2], s);
    if (stime) cudaEventRecord(ctx->split.ev[3], sv);  // after the previous dilation and this set-up
    e = cudaLaunchCooperativeKernel(solve_fn, grid, block, args, (size_t)sh.smem, sv);
    if (e == cudaSuccess && stime) {
        cudaEventRecord(ctx->split.ev[4], sv);
        ctx->split.timed = true;
        hd_timings& T = ctx->split.shape;
        T.grid_ctas = (int)grid.x;
        T.brick_x_words = bxw;
        T.brick_z = bz;
        T.kernel = sh.kernel;
        T.steps_per_barrier = sh.steps;
        T.brick_rows = by;
        T.dilation_partitions = ctx->split.parts;
    }
    if (e == cudaSuccess && split) {
        e = cudaEventRecord(ctx->split.ws_free[ws], sv);
        ctx->split.pending = true;
        ctx->split.next = (ws + 1) % ctx->split.nws;
    }
    if (e != cudaSuccess) return cuda_fail(ctx, e, "dilation launch");
    if (timing) cudaEventRecord(ctx->ev[3], s);
    if (async) {
        // the step counter moves past any step this launch can reach (its
        // stamps stay below the next call's steps)
        ctx->g_next = g0 + sp.max_iters + 2;
        return HD_OK;
    }

    // ---- read-back: the loop control and the decoded results ------------------
    hd_result* hres = (hd_result*)(hbase + upload_bytes);
    e = cudaMemcpyAsync(hbase + off_ctl, dbase + off_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(hres, dbase + off_out, sizeof(hd_result) * n, cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "result read-back");
    uint64_t* htc = (uint64_t*)(hres + n);
    if (stats) {
        size_t o = 0;
        for (int i = 0; i < n && e == cudaSuccess; ++i)
            for (int j = 0; j < 2 && e == cudaSuccess; ++j) {
                e = cudaMemcpyAsync(htc + o, dbase + plan[i].off_tcount[j], sizeof(uint64_t) * (plan[i].kmax + 1),
                                    cudaMemcpyDeviceToHost, s);
                o += plan[i].kmax + 1;
            }
        if (e != cudaSuccess) return cuda_fail(ctx, e, "instrumentation read-back");
    }
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "dilation");

    const Ctl* hctl = (const Ctl*)(hbase + off_ctl);
    ctx->g_next = std::max(ctx->g_next, hctl->g_end) + 2;
    if (timing) {
        ctx->split.timed = false;
        hd_timings& T = ctx->last_timings;
        cudaEventElapsedTime(&T.pack_ms, ctx->ev[0], ctx->ev[1]);
        cudaEventElapsedTime(&T.setup_ms, ctx->ev[1], ctx->ev[2]);
        cudaEventElapsedTime(&T.solve_ms, ctx->ev[2], ctx->ev[3]);
        cudaEventElapsedTime(&T.total_ms, ctx->ev[0], ctx->ev[3]);
        T.iterations = hctl->iters_run;
        T.grid_ctas = (int)grid.x;
        T.brick_x_words = bxw;
        T.brick_z = bz;
        T.kernel = sh.kernel;
        T.steps_per_barrier = sh.steps;
        T.brick_rows = by;
        T.dilation_partitions = 0;
    }
    if (stats && n == 1) {
        const int kp1 = plan[0].kmax + 1;
        for (int k = 0; k < ro.tiles_len; ++k) {
            if (ro.tiles_ba) ro.tiles_ba[k] = k < kp1 ? htc[k] : 0;
            if (ro.tiles_ab) ro.tiles_ab[k] = k < kp1 ? htc[kp1 + k] : 0;
        }
        if (ro.bricks) {
            // instrumented runs only: the brick counters of the two jobs
            JobState js[2];
            e = cudaMemcpy(js, dbase + off_states, sizeof js, cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) return cuda_fail(ctx, e, "instrumentation read-back");
            *ro.bricks = js[0].bricks + js[1].bricks;
        }
    }
    hd_status first = HD_OK;
    for (int i = 0; i < n; ++i) {
        out[i] = hres[i];
        const hd_status st = (hd_status)hres[i].status;
        if (st == HD_EMPTY_MASK && first == HD_OK) first = st;
        if (st != HD_OK && st != HD_EMPTY_MASK) {
            if (first == HD_OK || first == HD_EMPTY_MASK) first = st;
            set_error(ctx, st, "pair %d: %s", i, hd_status_string(st));
        }
    }
    return first;
}

}  // namespace hdh

// ============================================================================
// C ABI
// ============================================================================
using namespace hdh;

namespace hdk {
const void* solve_kernel_ptr(int se, int bxw, int bz) {
    return se == 0 ? solve_kernel_ptr_se6(bxw, bz) : solve_kernel_ptr_se18(bxw, bz);
}
const void* solve_tb_kernel_ptr(int se, int steps, int bz) {
    return se == 0 ? solve_tb_kernel_ptr_se6(steps, bz) : solve_tb_kernel_ptr_se18(steps, bz);
}
}  // namespace hdk

extern "C" {

void hd_options_init(hd_options* opt) {
    if (!opt) return;
    std::memset(opt, 0, sizeof *opt);
    opt->percentile = 0.95f;
    opt->zero_copy = 1;
}

const char* hd_status_string(hd_status s) {
    switch (s) {
        case HD_OK: return "ok";
        case HD_EMPTY_MASK: return "exactly one mask is empty";
        case HD_ERR_BAD_ARG: return "bad argument";
        case HD_ERR_OOM: return "out of memory";
        case HD_ERR_CUDA: return "CUDA error";
        case HD_ERR_TIMEOUT: return "device wait timed out";
        case HD_ERR_CANCELLED: return "cancelled";
        case HD_ERR_ITER_LIMIT: return "iteration limit reached";
        case HD_ERR_NOT_READY: return "not ready";
        case HD_ERR_UNSUPPORTED: return "unsupported";
        case HD_ERR_BUSY: return "server queue full";
    }
    return "unknown status";
}

const char* hd_version(void) { return "hd_gb300 1.0 sm_103a"; }

hd_status hd_context_create(int device, const hd_options* opt, hd_context** out) {
    if (!out) return HD_ERR_BAD_ARG;
    *out = nullptr;
    if (opt && (opt->label < 0 || opt->label > 255)) return HD_ERR_BAD_ARG;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return HD_ERR_CUDA;
    }
    if (device < 0 || device >= ndev) return HD_ERR_BAD_ARG;
    hd_context* ctx = new (std::nothrow) hd_context();
    if (!ctx) return HD_ERR_OOM;
    ctx->device = device;
    hd_options_init(&ctx->opt);
    if (opt) ctx->opt = *opt;
    if (opt && opt->tuning_table) ctx->tuning_path = opt->tuning_table;
    ctx->opt.tuning_table = nullptr;
    {
        DeviceGuard g(device);
        if (!g.ok) {
            delete ctx;
            return HD_ERR_CUDA;
        }
        e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
        int coop = 0;
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device);
        int ats = 0;
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ats, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device);
        if (e != cudaSuccess || !coop) {
            cudaGetLastError();
            if (ctx->stream) cudaStreamDestroy(ctx->stream);
            delete ctx;
            return HD_ERR_CUDA;
        }
        ctx->pageable_ats = ats;
        if (ctx->opt.record_timings)
            for (auto& ev : ctx->ev) cudaEventCreate(&ev);
    }
    if (!ctx->tuning_path.empty()) ctx->tune.load(ctx->tuning_path);
    *out = ctx;
    return HD_OK;
}

hd_status hd_context_destroy(hd_context* ctx) {
    if (!ctx) return HD_ERR_BAD_ARG;
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        DeviceGuard g(ctx->device);
        if (ctx->stream) cudaStreamSynchronize(ctx->stream);
        split_release(ctx);
        ctx->arena.release();
        for (DeviceArena& a : ctx->ws_arena) a.release();
        ctx->stamps.release();
        for (DeviceArena& a : ctx->part_stamps) a.release();
        ctx->pinned.release();
        for (int i = 0; i < hd_context::kAsyncSlots; ++i) {
            ctx->async_stage[i].release();
            if (ctx->async_done[i]) cudaEventDestroy(ctx->async_done[i]);
        }
        if (ctx->copy_stream) cudaStreamSynchronize(ctx->copy_stream);
        for (int i = 0; i < 2; ++i) {
            ctx->mask_stage[i].release();
            if (ctx->mask_ready[i]) cudaEventDestroy(ctx->mask_ready[i]);
            if (ctx->mask_free[i]) cudaEventDestroy(ctx->mask_free[i]);
        }
        if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
        for (auto& ev : ctx->ev)
            if (ev) cudaEventDestroy(ev);
        if (ctx->stream) cudaStreamDestroy(ctx->stream);
        ctx->stream = nullptr;
    }
    delete ctx;
    return HD_OK;
}

const char* hd_context_last_error(hd_context* ctx) { return ctx ? ctx->last_error.c_str() : ""; }

hd_status hd_context_last_timings(hd_context* ctx, hd_timings* out) {
    if (!ctx || !out) return HD_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (ctx->split.timed) {
        // the latest pipelined call on split SMs: its phases once complete
        DeviceGuard g(ctx->device);
        if (cudaEventQuery(ctx->split.ev[4]) != cudaSuccess) {
            cudaGetLastError();
            return HD_ERR_NOT_READY;
        }
        hd_timings T = ctx->split.shape;
        cudaEventElapsedTime(&T.pack_ms, ctx->split.ev[0], ctx->split.ev[1]);
        cudaEventElapsedTime(&T.setup_ms, ctx->split.ev[1], ctx->split.ev[2]);
        cudaEventElapsedTime(&T.solve_ms, ctx->split.ev[3], ctx->split.ev[4]);
        cudaEventElapsedTime(&T.total_ms, ctx->split.ev[0], ctx->split.ev[4]);
        T.iterations = -1;  // not read back by the enqueue-only entry
        ctx->split.timed = false;
        ctx->last_timings = T;
    }
    *out = ctx->last_timings;
    return HD_OK;
}

static hd_status metric_to_se(hd_context* ctx, int metric, int* se) {
    if (metric == HD_SE6) *se = 0;
    else if (metric == HD_SE18_FORBENCH) *se = 1;
    else return set_error(ctx, HD_ERR_BAD_ARG, "unknown metric %d", metric);
    return HD_OK;
}

hd_status hd_compute_u8(hd_context* ctx, const uint8_t* a, const uint8_t* b, int32_t W, int32_t H,
                        int32_t D, hd_metric metric, hd_result* out) {
    if (!ctx || !a || !b || !out) return HD_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    int se = 0;
    hd_status st = metric_to_se(ctx, metric, &se);
    if (st == HD_OK) st = check_dims(ctx, W, H, D);
    if (st != HD_OK) return st;
    DeviceGuard g(ctx->device);
    if (!g.ok) return set_error(ctx, HD_ERR_CUDA, "cannot select device %d", ctx->device);
    PairIn p{a, b, W, H, D, nullptr, nullptr};
    if (ctx->opt.zero_copy) {
        p.a = zero_copy_ptr(ctx, a);
        p.b = zero_copy_ptr(ctx, b);
    } else {
        p.a = p.b = nullptr;
    }
    if (!p.a) p.host_a = a;
    if (!p.b) p.host_b = b;
    RunOpts ro;
    ro.se = se;
    return run_pairs(ctx, &p, 1, ctx->stream, ro, out);
}

hd_status hd_compute_u8_device(hd_context* ctx, const uint8_t* d_a, const uint8_t* d_b, int32_t W,
                               int32_t H, int32_t D, hd_metric metric, void* stream, hd_result* out) {
    if (!ctx || !d_a || !d_b || !out) return HD_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    int se = 0;
    hd_status st = metric_to_se(ctx, metric, &se);
    if (st == HD_OK) st = check_dims(ctx, W, H, D);
    if (st != HD_OK) return st;
    DeviceGuard g(ctx->device);
    if (!g.ok) return set_error(ctx, HD_ERR_CUDA, "cannot select device %d", ctx->device);
    PairIn p{d_a, d_b, W, H, D, nullptr, nullptr};
    RunOpts ro;
    ro.se = se;
    return run_pairs(ctx, &p, 1, stream ? (cudaStream_t)stream : ctx->stream, ro, out);
}

hd_status hd_compute_u8_device_async(hd_context* ctx, const uint8_t* d_a, const uint8_t* d_b, int32_t W, int32_t H,
                                     int32_t D, hd_metric metric, void* stream, hd_result* d_out) {
    if (!ctx || !d_a || !d_b || !d_out) return HD_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    int se = 0;
    hd_status st = metric_to_se(ctx, metric, &se);
    if (st == HD_OK) st = check_dims(ctx, W, H, D);
    if (st != HD_OK) return st;
    DeviceGuard g(ctx->device);
    if (!g.ok) return set_error(ctx, HD_ERR_CUDA, "cannot select device %d", ctx->device);
    PairIn p{d_a, d_b, W, H, D, nullptr, nullptr};
    RunOpts ro;
    ro.se = se;
    ro.async_out = d_out;
    return run_pairs(ctx, &p, 1, stream ? (cudaStream_t)stream : ctx->stream, ro, nullptr);
}

hd_status hd_compute_u8_device_pipelined(hd_context* ctx, const uint8_t* d_a, const uint8_t* d_b, int32_t W,
                                         int32_t H, int32_t D, hd_metric metric, void* stream, hd_result* d_out) {
    if (!ctx || !d_a || !d_b || !d_out) return HD_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    int se = 0;
    hd_status st = metric_to_se(ctx, metric, &se);
    if (st == HD_OK) st = check_dims(ctx, W, H, D);
    if (st != HD_OK) return st;
    DeviceGuard g(ctx->device);
    if (!g.ok) return set_error(ctx, HD_ERR_CUDA, "cannot select device %d", ctx->device);
    PairIn p{d_a, d_b, W, H, D, nullptr, nullptr};
    RunOpts ro;
    ro.se = se;
    ro.async_out = d_out;
    ro.pipelined = true;
    return run_pairs(ctx, &p, 1, stream ? (cudaStream_t)stream : ctx->stream, ro, nullptr);
}

hd_status hd_pipeline_flush(hd_context* ctx, void* stream) {
    if (!ctx) return HD_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (!ctx->split.pending) return HD_OK;
    DeviceGuard g(ctx->device);
    if (!g.ok) return set_error(ctx, HD_ERR_CUDA, "cannot select device %d", ctx->device);
    // the dilations in each workspace run in order on one stream: the
    // latest of each covers them all
    const cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
    const cudaError_t e = wait_split_dilations(ctx, s);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "pipeline flush");
    ctx->split.pending = false;
    return HD_OK;
}

hd_status hd_compute_u8_async(hd_context* ctx, const uint8_t* a, const uint8_t* b, int32_t W, int32_t H, int32_t D,
                              hd_metric metric, void* stream, hd_result* d_out) {
    if (!ctx || !a || !b || !d_out) return HD_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    int se = 0;
    hd_status st = metric_to_se(ctx, metric, &se);
    if (st == HD_OK) st = check_dims(ctx, W, H, D);
    if (st != HD_OK) return st;
    DeviceGuard g(ctx->device);
    if (!g.ok) return set_error(ctx, HD_ERR_CUDA, "cannot select device %d", ctx->device);
    PairIn p{nullptr, nullptr, W, H, D, a, b};
    RunOpts ro;
    ro.se = se;
    ro.async_out = d_out;
    return run_pairs(ctx, &p, 1, stream ? (cudaStream_t)stream : ctx->stream, ro, nullptr);
}

hd_status hd_batch_compute(hd_context* ctx, const hd_pair_desc* pairs, int32_t n, hd_result* out) {
    if (!ctx || (n > 0 && (!pairs || !out)) || n < 0) return HD_ERR_BAD_ARG;
    if (n == 0) return HD_OK;
    std::lock_guard<std::mutex> lk(ctx->mu);
    for (int i = 0; i < n; ++i) {
        int se;
        if (!pairs[i].a || !pairs[i].b) return set_error(ctx, HD_ERR_BAD_ARG, "pair %d: null mask", i);
        hd_status st = metric_to_se(ctx, pairs[i].metric, &se);
        if (st == HD_OK) st = check_dims(ctx, pairs[i].W, pairs[i].H, pairs[i].D);
        if (st != HD_OK) return st;
    }
    DeviceGuard g(ctx->device);
    if (!g.ok) return set_error(ctx, HD_ERR_CUDA, "cannot select device %d", ctx->device);
    hd_status first = HD_OK;
    for (int se = 0; se < 2; ++se) {
        std::vector<PairIn> in;
        std::vector<int> idx;
        for (int i = 0; i < n; ++i) {
            const int pse = pairs[i].metric == HD_SE6 ? 0 : 1;
            if (pse != se) continue;
            PairIn p{pairs[i].a, pairs[i].b, pairs[i].W, pairs[i].H, pairs[i].D, nullptr, nullptr};
            if (!pairs[i].on_device) {
                p.a = ctx->opt.zero_copy ? zero_copy_ptr(ctx, pairs[i].a) : nullptr;
                p.b = ctx->opt.zero_copy ? zero_copy_ptr(ctx, pairs[i].b) : nullptr;
                if (!p.a) p.host_a = pairs[i].a;
                if (!p.b) p.host_b = pairs[i].b;
            }
            in.push_back(p);
            idx.push_back(i);
        }
        if (in.empty()) continue;
        std::vector<hd_result> res(in.size());
        RunOpts ro;
        ro.se = se;
        const hd_status st = run_pairs(ctx, in.data(), (int)in.size(), ctx->stream, ro, res.data());
        for (size_t j = 0; j < idx.size(); ++j) out[idx[j]] = res[j];
        if (st != HD_OK && st != HD_EMPTY_MASK) return st;
        if (first == HD_OK) first = st;
    }
    return first;
}

hd_status hd_profile_u8_device(hd_context* ctx, const uint8_t* d_a, const uint8_t* d_b, int32_t W,
                               int32_t H, int32_t D, hd_metric metric, hd_result* out,
                               uint64_t* tiles_ab, uint64_t* tiles_ba, int32_t len,
                               uint64_t* bricks_processed) {
    if (!ctx || !d_a || !d_b || !out || len < 0) return HD_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    int se = 0;
    hd_status st = metric_to_se(ctx, metric, &se);
    if (st == HD_OK) st = check_dims(ctx, W, H, D);
    if (st != HD_OK) return st;
    DeviceGuard g(ctx->device);
    if (!g.ok) return set_error(ctx, HD_ERR_CUDA, "cannot select device %d", ctx->device);
    PairIn p{d_a, d_b, W, H, D, nullptr, nullptr};
    RunOpts ro;
    ro.se = se;
    ro.stats = 1;
    ro.tiles_ab = tiles_ab;
    ro.tiles_ba = tiles_ba;
    ro.tiles_len = len;
    ro.bricks = bricks_processed;
    return run_pairs(ctx, &p, 1, ctx->stream, ro, out);
}

hd_status hd_distance_map_device(hd_context* ctx, const uint8_t* d_a, const uint8_t* d_b, int32_t W,
                                 int32_t H, int32_t D, hd_metric metric, int32_t* d_map_a,
                                 int32_t* d_map_b, hd_result* out) {
    if (!ctx || !d_a || !d_b || !out || !d_map_a || !d_map_b) return HD_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    int se = 0;
    hd_status st = metric_to_se(ctx, metric, &se);
    if (st == HD_OK) st = check_dims(ctx, W, H, D);
    if (st != HD_OK) return st;
    DeviceGuard g(ctx->device);
    if (!g.ok) return set_error(ctx, HD_ERR_CUDA, "cannot select device %d", ctx->device);
    PairIn p{d_a, d_b, W, H, D, nullptr, nullptr};
    RunOpts ro;
    ro.se = se;
    ro.map_a = d_map_a;
    ro.map_b = d_map_b;
    return run_pairs(ctx, &p, 1, ctx->stream, ro, out);
}

}  // extern "C"
