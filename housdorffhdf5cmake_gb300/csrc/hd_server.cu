// hd_server.cu -- continuous-batching request loop.
//
// No counterpart in the reference (it computes one pair per call).  Requests
// are admitted while device memory (a byte budget) and job slots allow; an
// admitted pair is packed and set up on the device and its two jobs join the
// resident persistent dilation loop at the next "tick" with their own step
// counter (Job::k0), so pairs that arrive while others are mid-flight overlap
// on the device.  A tick is one cooperative launch of the same dilation kernel
// as the single-pair path, bounded to tick_iterations steps; between ticks the
// scheduler thread reads the jobs' states, completes finished pairs, frees
// their memory and admits waiting ones.  Each pair's result depends only on
// its own masks, so it is identical alone and in any mix.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "hd/hd.h"
#include "hd_internal.h"
#include "hd_kernels.h"

using namespace hdh;
using hdk::Ctl;
using hdk::Job;
using hdk::JobState;
using hdk::PairDesc;
using hdk::PairInfo;

namespace {

enum ReqState { kWaiting = 0, kResident = 1, kDone = 2 };

struct Request {
    uint64_t ticket = 0;
    int32_t W = 0, H = 0, D = 0;
    const uint8_t* dev_a = nullptr;  // caller's device masks (on_device)
    const uint8_t* dev_b = nullptr;
    std::vector<uint8_t> host_a, host_b;  // copies of host masks
    ReqState state = kWaiting;
    bool cancel = false;
    hd_result result{};
    // resident resources
    int slot = -1;
    void* resident = nullptr;   // job buffers + histograms + info
    size_t resident_bytes = 0;
    size_t transient_bytes = 0;
    unsigned long long brick0 = 0, nbricks = 0;  // per job
    int kmax = 0;
    int wxf = 0;
    long long dom_words = 0;
    size_t off_hist = 0, off_info = 0, off_packed = 0;
};

// First-fit allocator over [0, cap) (brick ids).
struct RangeAlloc {
    std::map<unsigned long long, unsigned long long> free_;  // start -> length
    explicit RangeAlloc(unsigned long long cap = 0) {
        if (cap) free_[0] = cap;
    }
    bool alloc(unsigned long long n, unsigned long long* out) {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= n) {
                *out = it->first;
                const unsigned long long s = it->first + n, l = it->second - n;
                free_.erase(it);
                if (l) free_[s] = l;
                return true;
            }
        }
        return false;
    }
    void release(unsigned long long s, unsigned long long n) {
        auto it = free_.emplace(s, n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
};

inline size_t align_up(size_t x, size_t a = 256) { return (x + a - 1) / a * a; }

// How long the scheduler polls for new requests when it runs out of work
// before it sleeps on the condition variable, and how long hd_server_wait /
// hd_server_wait_any poll before they sleep (a wake-up through the
// condition variable adds tens of microseconds to a request's latency; the
// polls read one atomic count, not the server lock).
constexpr int kIdleSpinUs = 2000;
constexpr int kWaitSpinUs = 1000;
// Busy periods: single-pair kernel shape when at most kFewRequests wait as
// the server starts work; batch shape after a drain once more than
// kQueueForBatchMode wait.
constexpr int kFewRequests = 2;
constexpr int kQueueForBatchMode = 8;

}  // namespace

struct hd_server {
    hd_context* ctx = nullptr;
    hd_server_options opt{};
    int se = 0, grid = 0;
    // The dilation kernel's shape, chosen per busy period (the server is
    // empty when it changes: bricks of one shape cannot continue under
    // another): modes[0] the single-pair shape (more steps per barrier,
    // fewer barriers for a lone request), modes[1] the batch shape; `mode`
    // selects, and shape / solve_fn / grid are the selected mode's.
    struct Mode {
        Shape shape;
        const void* fn = nullptr;
        int grid = 0;
    } modes[2];
    int mode = 1;
    bool draining = false;  // single-pair mode with a queue building up: admit nothing until empty
    Shape shape;
    const void* solve_fn = nullptr;
    cudaStream_t stream = nullptr;
    std::thread worker;
    std::mutex mu;
    std::condition_variable cv;       // wakes the scheduler
    std::condition_variable done_cv;  // wakes waiters
    bool stop = false;
    uint64_t next_ticket = 1;
    std::deque<Request*> waiting;
    std::map<uint64_t, std::unique_ptr<Request>> reqs;
    std::vector<Request*> slots;      // resident pair per slot
    std::vector<int> free_slots;
    std::vector<int> quarantine;      // slots freed during the last tick
    std::vector<uint32_t> slot_epoch; // bumped on every admission into a slot and on every completion
    RangeAlloc bricks;
    unsigned long long brick_cap = 0;
    // persistent device state
    Job* d_jobs = nullptr;
    JobState* d_states = nullptr;
    Ctl* d_ctl = nullptr;
    unsigned long long* d_queue[3] = {nullptr, nullptr, nullptr};
    int32_t* d_stamps = nullptr;
    PairDesc* d_descs = nullptr;      // per-tick admission descriptors
    int max_admit = 256;
    cudaMemPool_t pool = nullptr;     // the pairs' buffers: a private pool that keeps what it has reserved
    void* h_pinned = nullptr;         // descriptors and retirements out, states and results in
    size_t h_pinned_bytes = 0;
    size_t off_h_results = 0, off_h_retire = 0, off_h_yield = 0;
    PairDesc* d_slot_descs = nullptr; // per slot: its pair's descriptor (info = null: unused)
    hd_result* d_results = nullptr;   // per slot: the result decoded by the launch that finished it
    uint32_t* d_retire = nullptr;     // (slot, epoch) pairs retired by a tick
    int32_t* d_yield = nullptr;       // yield generation, advanced by submissions during a tick
    cudaStream_t side = nullptr;      // posts the yield word while a tick runs
    cudaEvent_t ev_yield = nullptr;
    int32_t yield_gen = 0;            // last generation posted
    bool in_tick = false, yield_posted = false;
    std::deque<uint64_t> done_order;  // tickets in completion order (hd_server_wait_any)
    int g_next = 1;
    hd_server_stats stats{};
    std::string err;
    bool debug = false;  // HD_SERVER_DEBUG=1: one line per tick on stderr
    // Advanced (under the lock) by every submission, cancel and stop
    // (wake_seq) and by every completion (done_seq): the worker's idle poll
    // and the waiters' spin read them without the lock, which they take only
    // when a count has moved, so the polls do not compete with the tick and
    // with submissions for the lock.
    std::atomic<unsigned long long> wake_seq{0}, done_seq{0};
};

namespace {

hd_status cuda_err(hd_server* s, cudaError_t e, const char* where) {
    s->err = std::string(where) + ": " + cudaGetErrorString(e);
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? HD_ERR_OOM : HD_ERR_CUDA;
}

// Sizes of one request's device memory (resident part lives until completion,
// transient part only through packing and set-up).  Resident: three
// domain-sized buffers per job (both ping-pong buffers, and the
// uncovered-target array of the one-step kernel or a crop of one mask for
// the blocked kernel), histograms, counts, and the packed masks, which the
// blocked kernel reads in place as the single-pair path does (no crop copy
// in set-up).  Transient: the staged host masks.
void plan_request(hd_server* s, Request* r) {
    r->wxf = (r->W + 31) / 32;
    const long long pitch = (r->wxf + 3) / 4 * 4;
    r->dom_words = pitch * r->H * r->D;
    r->kmax = r->W + r->H + r->D;
    const size_t job_bytes = align_up(4ULL * r->dom_words);
    r->off_hist = 6 * job_bytes;
    r->off_info = align_up(r->off_hist + 2ULL * (r->kmax + 1) * sizeof(uint64_t));
    r->off_packed = align_up(r->off_info + sizeof(PairInfo));
    const size_t nb = (size_t)r->W * r->H * r->D;
    const size_t packed = align_up(4ULL * hdk::packed_pitch(r->W) * r->H * r->D);
    r->resident_bytes = r->off_packed + 2 * packed;
    r->transient_bytes = r->dev_a ? 0 : 2 * align_up(nb);
}

// Marks a request done (server lock held) and lists it for wait_any.
void mark_done(hd_server* s, Request* r) {
    r->state = kDone;
    s->done_seq.fetch_add(1, std::memory_order_release);
    // tickets taken by poll / wait leave the completion list from its front
    while (!s->done_order.empty() && !s->reqs.count(s->done_order.front())) s->done_order.pop_front();
    s->done_order.push_back(r->ticket);
}

void complete(hd_server* s, Request* r, hd_status st) {
    r->result.status = st;
    if (st != HD_OK && st != HD_EMPTY_MASK) r->result.hd = r->result.hd_ab = r->result.hd_ba = r->result.hd_robust = -1;
    s->stats.completed += 1;
    mark_done(s, r);
}

// One scheduler tick.  Called with the server lock NOT held.
void tick(hd_server* s) {
    using clk = std::chrono::steady_clock;
    const auto t_begin = clk::now();
    std::vector<Request*> admit;
    int32_t ygen = 0;
    int used_hi = 0;  // slots [0, used_hi) hold every resident pair
    {
        std::lock_guard<std::mutex> lk(s->mu);
        // cancelled waiting requests leave at once
        for (auto it = s->waiting.begin(); it != s->waiting.end();) {
            if ((*it)->cancel) {
                (*it)->result.status = HD_ERR_CANCELLED;
                mark_done(s, *it);
                s->stats.cancelled += 1;
                it = s->waiting.erase(it);
            } else {
                ++it;
            }
        }
        for (int q : s->quarantine) s->free_slots.push_back(q);
        s->quarantine.clear();
        // Kernel shape per busy period: a server that starts work with few
        // requests waiting takes the single-pair shape; once requests queue
        // up behind it, it admits nothing until the resident pairs are done
        // and then takes the batch shape.
        bool any_resident = false;
        for (auto* r : s->slots) any_resident = any_resident || r != nullptr;
        if (!any_resident && !s->waiting.empty()) {
            const int want = s->waiting.size() <= (size_t)kFewRequests ? 0 : 1;
            s->mode = want;
            s->shape = s->modes[want].shape;
            s->solve_fn = s->modes[want].fn;
            s->grid = s->modes[want].grid;
            s->draining = false;
        } else if (s->mode == 0 && s->waiting.size() > (size_t)kQueueForBatchMode) {
            s->draining = true;
        }
        while (!s->draining && !s->waiting.empty() && (int)admit.size() < s->max_admit && !s->free_slots.empty()) {
            Request* r = s->waiting.front();
            const size_t need = r->resident_bytes + r->transient_bytes;
            if (need > s->opt.hbm_budget_bytes) {  // can never fit
                s->waiting.pop_front();
                complete(s, r, HD_ERR_OOM);
                continue;
            }
            if (s->stats.bytes_in_use + need > s->opt.hbm_budget_bytes) break;
            r->nbricks = (unsigned long long)hdk::bricks_max(r->W, r->H, r->D, s->shape.bxw, s->shape.by, s->shape.bz);
            unsigned long long b0 = 0;
            if (!s->bricks.alloc(2 * r->nbricks, &b0)) break;
            s->waiting.pop_front();
            r->brick0 = b0;
            r->slot = s->free_slots.back();
            s->free_slots.pop_back();
            s->slots[r->slot] = r;
            r->state = kResident;
            s->stats.bytes_in_use += need;
            s->stats.bytes_peak = std::max(s->stats.bytes_peak, s->stats.bytes_in_use);
            admit.push_back(r);
        }
        // submissions from here on advance the yield word (once per tick):
        // this tick's launch then ends at its next barrier so that they are
        // admitted by the next tick
        s->in_tick = true;
        s->yield_posted = false;
        ygen = s->yield_gen;
        for (size_t sl = 0; sl < s->slots.size(); ++sl)
            if (s->slots[sl]) used_hi = (int)sl + 1;
        s->done_cv.notify_all();
    }
    cudaStream_t st = s->stream;
    cudaError_t e = cudaSuccess;
    // ---- admission: allocate, upload, pack, set up --------------------------
    std::vector<PairDesc> descs;
    std::vector<Request*> admitted;
    long long ptiles = 0, stiles = 0;
    // the blocked kernel reads the packed masks in place unless that adds a
    // brick column (then crops), like the single-pair path
    const int setup_mode = s->shape.kernel == 1 ? hdk::kSetupOneStep : hdk::kSetupBlocked;
    // the admitted pairs' transient buffers (staged host masks) in one block
    // for the tick, freed after the set-up; a block per pair for what lives
    // until the pair completes
    size_t transient_total = 0;
    for (Request* r : admit) transient_total += align_up(r->transient_bytes);
    void* tblock = nullptr;
    if (transient_total) {
        e = cudaMallocFromPoolAsync(&tblock, transient_total, s->pool, st);
        if (e != cudaSuccess) {
            cudaGetLastError();
            tblock = nullptr;
        }
    }
    size_t toff = 0;
    for (size_t i = 0; i < admit.size(); ++i) {
        Request* r = admit[i];
        void* res = nullptr;
        const bool t_ok = tblock != nullptr || transient_total == 0;
        if (t_ok) e = cudaMallocFromPoolAsync(&res, r->resident_bytes, s->pool, st);
        if (!t_ok || e != cudaSuccess) {
            cudaGetLastError();
            e = cudaSuccess;
            std::lock_guard<std::mutex> lk(s->mu);
            s->stats.bytes_in_use -= r->resident_bytes + r->transient_bytes;
            s->bricks.release(r->brick0, 2 * r->nbricks);
            s->slots[r->slot] = nullptr;
            s->quarantine.push_back(r->slot);
            complete(s, r, HD_ERR_OOM);
            continue;
        }
        r->resident = res;
        char* rb = (char*)res;
        char* tb = tblock ? (char*)tblock + toff : nullptr;
        toff += align_up(r->transient_bytes);
        const size_t nb = (size_t)r->W * r->H * r->D;
        const size_t packed = align_up(4ULL * hdk::packed_pitch(r->W) * r->H * r->D);
        PairDesc d{};
        if (r->dev_a) {
            d.a = r->dev_a;
            d.b = r->dev_b;
        } else {
            uint8_t* ia = (uint8_t*)tb;
            uint8_t* ib = ia + align_up(nb);
            cudaMemcpyAsync(ia, r->host_a.data(), nb, cudaMemcpyHostToDevice, st);
            cudaMemcpyAsync(ib, r->host_b.data(), nb, cudaMemcpyHostToDevice, st);
            d.a = ia;
            d.b = ib;
        }
        d.pa = (uint32_t*)(rb + r->off_packed);
        d.pb = (uint32_t*)(rb + r->off_packed + packed);
        const size_t job_bytes = align_up(4ULL * r->dom_words);
        for (int j = 0; j < 2; ++j) {
            for (int b = 0; b < 3; ++b) d.jb[j][b] = (uint32_t*)(rb + (3 * j + b) * job_bytes);
            d.hist[j] = (unsigned long long*)(rb + r->off_hist) + (size_t)j * (r->kmax + 1);
            d.brick0[j] = r->brick0 + (unsigned long long)j * r->nbricks;
        }
        d.W = r->W;
        d.H = r->H;
        d.D = r->D;
        d.wxf = r->wxf;
        d.se = s->se;
        d.aligned = ((((uintptr_t)d.a) | ((uintptr_t)d.b)) & 15) == 0;
        d.kmax = r->kmax;
        d.job0 = 2 * r->slot;
        d.epoch = ++s->slot_epoch[r->slot];
        d.tile0 = ptiles;
        d.stile0 = stiles;
        ptiles += hdk::pack_tiles_of(r->W, r->H, r->D);
        stiles += hdk::setup_tiles_of(r->W, r->H, r->D, setup_mode, s->shape.bxw, s->shape.by, s->shape.bz);
        d.info = (PairInfo*)(rb + r->off_info);
        descs.push_back(d);
        admitted.push_back(r);
    }
    if (!admitted.empty()) {
        // descriptors, then the pairs' count / bounding-box start values
        char* hp = (char*)s->h_pinned + align_up(sizeof(Ctl)) + align_up(sizeof(JobState) * 2 * s->slots.size());
        std::memcpy(hp, descs.data(), sizeof(PairDesc) * descs.size());
        e = cudaMemcpyAsync(s->d_descs, hp, sizeof(PairDesc) * descs.size(), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = hdk::launch_info_init(s->d_descs, (int)descs.size(), st, s->d_slot_descs);
        const int cap_ctas = std::max(s->ctx->sm_count * 8, 1);
        if (e == cudaSuccess)
            e = hdk::launch_pack(s->d_descs, (int)admitted.size(), ptiles, (int)std::min<long long>(cap_ctas, ptiles),
                                 s->ctx->opt.label, 0, st);
        if (e == cudaSuccess)
            e = hdk::launch_setup(s->d_descs, (int)admitted.size(), stiles, 0,
                                  s->d_jobs, s->d_states,
                                  s->d_queue[s->g_next % 3], s->d_ctl, s->g_next, s->shape.bxw, s->shape.by,
                                  s->shape.bz, setup_mode, st);
        // no wait here: the host masks' copies read the requests' own
        // buffers (alive until completion), the descriptors' staging area is
        // rewritten only after the end-of-tick synchronisation, and the
        // transient buffers below are freed in stream order
        if (e != cudaSuccess) {
            cuda_err(s, e, "admission");
        }
    }
    if (tblock) cudaFreeAsync(tblock, st);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        for (auto* r : admitted) s->stats.bytes_in_use -= r->transient_bytes;
    }
    const auto t_admitted = clk::now();
    // ---- one tick of the persistent dilation loop ---------------------------
    int resident = 0;
    for (auto* r : s->slots) resident += r != nullptr;
    const float pct = (s->ctx->opt.percentile > 0.f && s->ctx->opt.percentile <= 1.f) ? s->ctx->opt.percentile : 0.95f;
    if (resident > 0 && e == cudaSuccess) {
        hdk::SolveParams sp{};
        sp.jobs = s->d_jobs;
        sp.states = s->d_states;
        for (int q = 0; q < 3; ++q) sp.queue[q] = s->d_queue[q];
        sp.stamps = s->d_stamps;
        sp.ctl = s->d_ctl;
        sp.g0 = s->g_next;
        sp.max_iters = s->opt.tick_iterations;
        sp.timeout_ns = s->ctx->opt.barrier_timeout_ns > 0 ? s->ctx->opt.barrier_timeout_ns : 10000000000LL;
        // after its last barrier the launch decodes every pair that has
        // finished into its slot's result (the histograms stay on the device)
        sp.descs = s->d_slot_descs;
        sp.npairs = used_hi;
        sp.pct = pct;
        sp.out = s->d_results;
        sp.decode_done_only = 1;
        sp.yield = s->d_yield;
        sp.yield_gen = ygen;
        if (resident == 1 && s->shape.kernel == 2) {
            // a lone request: its two jobs are read from a per-CTA copy (the
            // jobs change only between ticks: set-up and retire run on this
            // stream before the launch)
            for (size_t i = 0; i < s->slots.size(); ++i)
                if (s->slots[i]) {
                    sp.job_cache = hdk::kJobCache;
                    sp.job_cache_base = 2 * (int32_t)i;
                }
        }
        void* args[] = {&sp};
        // yield words posted before this tick have landed
        e = cudaStreamWaitEvent(st, s->ev_yield, 0);
        if (e == cudaSuccess)
            e = cudaLaunchCooperativeKernel(s->solve_fn, dim3(s->grid), dim3(s->shape.threads), args,
                                            (size_t)s->shape.smem, st);
    }
    // ---- read back loop control, job states and results, in one wait ---------
    const size_t nst = 2 * (size_t)used_hi;
    char* hp = (char*)s->h_pinned;
    Ctl* hctl = (Ctl*)hp;
    JobState* hst = (JobState*)(hp + align_up(sizeof(Ctl)));
    hd_result* hres = (hd_result*)(hp + s->off_h_results);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hctl, s->d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && nst)
        e = cudaMemcpyAsync(hst, s->d_states, sizeof(JobState) * nst, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && used_hi)
        e = cudaMemcpyAsync(hres, s->d_results, sizeof(hd_result) * used_hi, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->in_tick = false;
    }
    int hard_err = 0;
    if (e != cudaSuccess) {
        cuda_err(s, e, "tick");
        hard_err = HD_ERR_CUDA;
    } else {
        if (resident > 0) s->g_next = std::max(s->g_next, hctl->g_end);
        hard_err = hctl->err;
    }
    if (s->debug) {
        const auto t_read = clk::now();
        std::fprintf(stderr,
                     "[hd_server] tick %llu admitted %zu resident %d g_next %d err %d(%s) jobs_active %d q %u/%u/%u "
                     "iters %d admission %.3f ms solve+readback %.3f ms\n",
                     (unsigned long long)s->stats.ticks, admitted.size(), resident, s->g_next, hctl->err,
                     e == cudaSuccess ? "ok" : cudaGetErrorString(e), hctl->jobs_active, hctl->qcount[0],
                     hctl->qcount[1], hctl->qcount[2], hctl->iters_run,
                     std::chrono::duration<double, std::milli>(t_admitted - t_begin).count(),
                     std::chrono::duration<double, std::milli>(t_read - t_admitted).count());
        for (size_t sl = 0; sl < s->slots.size() && sl < 4; ++sl)
            if (s->slots[sl])
                std::fprintf(stderr, "[hd_server]   slot %zu: active %d/%d remaining %llu/%llu hd %d/%d status %d/%d\n", sl,
                             hst[2 * sl].active, hst[2 * sl + 1].active, hst[2 * sl].remaining,
                             hst[2 * sl + 1].remaining, hst[2 * sl].hd, hst[2 * sl + 1].hd, hst[2 * sl].status,
                             hst[2 * sl + 1].status);
    }
    // A tick that admitted nothing and ran no step while jobs are still
    // active means their frontier is empty with targets left, which the
    // dilation cannot produce; fail those pairs rather than spin.
    const bool stalled = hard_err == 0 && e == cudaSuccess && resident > 0 && admitted.empty() &&
                         hctl->iters_run == 0 && hctl->jobs_active > 0;
    if (stalled && s->debug) std::fprintf(stderr, "[hd_server] no progress: failing active pairs\n");
    std::vector<Request*> finished;
    for (size_t sl = 0; sl < (size_t)used_hi; ++sl) {
        Request* r = s->slots[sl];
        if (!r) continue;
        const JobState& s0 = hst[2 * sl];
        const JobState& s1 = hst[2 * sl + 1];
        const bool fin = hard_err != 0 || stalled || r->cancel || (s0.active == 0 && s1.active == 0);
        if (fin) finished.push_back(r);
    }
    if (stalled) hard_err = HD_ERR_ITER_LIMIT;
    unsigned long long cancelled_active = 0;
    uint32_t* hretire = (uint32_t*)(hp + s->off_h_retire);
    int nretire = 0;
    for (Request* r : finished) {
        const size_t sl = (size_t)r->slot;
        const JobState s0 = hst[2 * sl], s1 = hst[2 * sl + 1];
        hd_status st_r = HD_OK;
        if (r->cancel) {
            st_r = HD_ERR_CANCELLED;
            cancelled_active += (s0.active != 0) + (s1.active != 0);
            r->result = hd_result{};
        } else if (hard_err) {
            r->result = hd_result{};
            st_r = (hd_status)hard_err;
        } else {
            // decoded on the device at the end of this tick's launch (the
            // rules of decode_result: statuses, exact sums, one division,
            // robust HD from the per-step histogram)
            r->result = hres[sl];
            st_r = (hd_status)r->result.status;
        }
        // Queue entries of the finished jobs may still be waiting for the
        // next step: a new epoch on the jobs makes the kernels drop them
        // before they read the buffers freed here (entries compare the low
        // 8 bits), and the slot's descriptor copy is marked unused.
        hretire[2 * nretire] = (uint32_t)sl;
        hretire[2 * nretire + 1] = ++s->slot_epoch[sl];
        ++nretire;
        cudaFreeAsync(r->resident, st);
        r->resident = nullptr;
        std::lock_guard<std::mutex> lk(s->mu);
        s->stats.bytes_in_use -= r->resident_bytes;
        s->bricks.release(r->brick0, 2 * r->nbricks);
        s->slots[sl] = nullptr;
        s->quarantine.push_back((int)sl);
        if (r->cancel) {
            r->result.status = HD_ERR_CANCELLED;
            mark_done(s, r);
            s->stats.cancelled += 1;
        } else {
            complete(s, r, st_r);
        }
    }
    if (!finished.empty()) {
        std::lock_guard<std::mutex> lk(s->mu);
        s->done_cv.notify_all();  // results first, clean-up after
    }
    if (nretire) {
        // the list is read before the next tick rewrites it (the end of
        // every tick waits for the stream)
        cudaError_t e3 = cudaMemcpyAsync(s->d_retire, hretire, sizeof(uint32_t) * 2 * nretire,
                                         cudaMemcpyHostToDevice, st);
        if (e3 == cudaSuccess) e3 = hdk::launch_retire(s->d_jobs, s->d_slot_descs, s->d_retire, nretire, st);
        if (e3 != cudaSuccess) cuda_err(s, e3, "retire");
    }
    if (cancelled_active || hard_err) {
        // Cancelled jobs leave the loop: mark them inactive and fix the
        // active-job count (no kernel runs between ticks).  After a device
        // error every resident pair has failed: reset the loop state.
        if (hard_err) {
            Ctl z{};
            cudaMemcpyAsync(s->d_ctl, &z, sizeof z, cudaMemcpyHostToDevice, st);
            s->g_next += 2;
        } else {
            for (Request* r : finished) {
                if (!r->cancel) continue;
                JobState off{};
                const size_t sl = (size_t)r->slot;
                cudaMemcpyAsync(s->d_states + 2 * sl, &off, sizeof off, cudaMemcpyHostToDevice, st);
                cudaMemcpyAsync(s->d_states + 2 * sl + 1, &off, sizeof off, cudaMemcpyHostToDevice, st);
            }
            Ctl c = *hctl;
            c.jobs_active -= (int)cancelled_active;
            cudaMemcpyAsync(&s->d_ctl->jobs_active, &c.jobs_active, sizeof(int32_t), cudaMemcpyHostToDevice, st);
        }
        cudaStreamSynchronize(st);
    }
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stats.ticks += 1;
        s->done_cv.notify_all();
    }
}

void worker_main(hd_server* s) {
    DeviceGuard g(s->ctx->device);
    auto has_work = [&] {
        if (s->stop) return true;
        if (!s->waiting.empty()) return true;
        for (auto* r : s->slots)
            if (r) return true;
        return false;
    };
    for (;;) {
        // idle: poll for a new request for a short while before sleeping
        // (a wake-up through the condition variable costs tens of
        // microseconds of a request's latency); the lock is taken only when
        // a submission, cancel or stop has moved wake_seq
        const auto t_idle = std::chrono::steady_clock::now();
        unsigned long long seen = s->wake_seq.load(std::memory_order_acquire);
        bool work = false;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            work = has_work();
        }
        while (!work && std::chrono::steady_clock::now() - t_idle < std::chrono::microseconds(kIdleSpinUs)) {
            const unsigned long long now_seq = s->wake_seq.load(std::memory_order_acquire);
            if (now_seq == seen) continue;
            seen = now_seq;
            std::lock_guard<std::mutex> lk(s->mu);
            work = has_work();
        }
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv.wait(lk, has_work);
            if (s->stop) return;
        }
        tick(s);
    }
}

// A wait's limit in ms, from 0 up to 2^40 (35 years: the deadline in the
// steady clock's nanoseconds cannot overflow).
int64_t clamp_timeout_ms(int64_t timeout_ms) { return std::min<int64_t>(std::max<int64_t>(timeout_ms, 0), int64_t(1) << 40); }

// Polls `ready` (server lock held by `lk`) for up to kWaitSpinUs, or
// timeout_ms if that is shorter; true once it holds.  Between checks the
// lock is released and only the completion count is read, without the
// lock, until it moves.  A result that lands within the window is picked up
// without the condition variable's wake-up latency.
template <class F>
bool spin_wait(hd_server* s, std::unique_lock<std::mutex>& lk, F ready, int64_t timeout_ms) {
    const auto lim = std::chrono::microseconds(
        timeout_ms >= 0 ? std::min<int64_t>(kWaitSpinUs, clamp_timeout_ms(timeout_ms) * 1000) : kWaitSpinUs);
    const auto t0 = std::chrono::steady_clock::now();
    while (!ready()) {
        const unsigned long long seen = s->done_seq.load(std::memory_order_acquire);
        lk.unlock();
        bool timed_out = false;
        while (s->done_seq.load(std::memory_order_acquire) == seen) {
            if (std::chrono::steady_clock::now() - t0 >= lim) {
                timed_out = true;
                break;
            }
        }
        lk.lock();
        if (timed_out) return ready();
    }
    return true;
}

}  // namespace

extern "C" {

void hd_server_options_init(hd_server_options* opt) {
    if (!opt) return;
    std::memset(opt, 0, sizeof *opt);
    opt->hbm_budget_bytes = 120ULL << 30;
    opt->max_queue = 4096;
    opt->tick_iterations = 64;
    opt->metric = HD_SE6;
}

hd_status hd_server_create(hd_context* ctx, const hd_server_options* opt, hd_server** out) {
    if (!ctx || !out) return HD_ERR_BAD_ARG;
    *out = nullptr;
    auto* s = new (std::nothrow) hd_server();
    if (!s) return HD_ERR_OOM;
    s->ctx = ctx;
    hd_server_options_init(&s->opt);
    if (opt) s->opt = *opt;
    if (!s->opt.hbm_budget_bytes) s->opt.hbm_budget_bytes = 120ULL << 30;
    if (s->opt.max_queue <= 0) s->opt.max_queue = 4096;
    if (s->opt.tick_iterations <= 0) s->opt.tick_iterations = 64;
    if (s->opt.metric != HD_SE6 && s->opt.metric != HD_SE18_FORBENCH) {
        delete s;
        return HD_ERR_BAD_ARG;
    }
    s->se = s->opt.metric == HD_SE6 ? 0 : 1;
    s->debug = std::getenv("HD_SERVER_DEBUG") != nullptr;
    int slots = s->opt.max_inflight > 0 ? s->opt.max_inflight : 1024;
    slots = std::min(slots, 16384);
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        DeviceGuard g(ctx->device);
        if (!g.ok) {
            delete s;
            return HD_ERR_CUDA;
        }
        PairIn typical{nullptr, nullptr, 256, 256, 160, nullptr, nullptr};
        unsigned long long brick_bytes = ~0ull;
        for (int m = 0; m < 2; ++m) {
            Shape sh = pick_shape(ctx, s->se, &typical, m == 0 ? 1 : 16);  // one pair / a batch-like mix
            const void* fn = solve_fn_of(s->se, sh);
            if (!fn) {
                delete s;
                return HD_ERR_BAD_ARG;
            }
            const int occ = occupancy_of(ctx, fn, sh.threads, sh.smem);
            if (occ <= 0) {
                delete s;
                return HD_ERR_CUDA;
            }
            const int cps = sh.ctas_per_sm;
            s->modes[m].shape = sh;
            s->modes[m].fn = fn;
            s->modes[m].grid = ctx->sm_count * (cps > 0 ? std::min(cps, occ) : occ);
            brick_bytes = std::min<unsigned long long>(brick_bytes, 4ULL * sh.bxw * sh.by * sh.bz);
        }
        s->mode = 1;
        s->shape = s->modes[1].shape;
        s->solve_fn = s->modes[1].fn;
        s->grid = s->modes[1].grid;
        // brick ids: one per 3 x (brick bytes) of budget (each job brick
        // spans 3 buffers) for the smaller brick of the two shapes, capped
        s->brick_cap = std::min<unsigned long long>(s->opt.hbm_budget_bytes / (3 * brick_bytes) + 4096, 1ULL << 26);
        s->bricks = RangeAlloc(s->brick_cap);
        cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) {
            // buffers come and go every tick: a pool that returns memory to
            // the device at each synchronisation would map and unmap it
            // every tick, so this one keeps up to the budget reserved
            cudaMemPoolProps props{};
            props.allocType = cudaMemAllocationTypePinned;
            props.handleTypes = cudaMemHandleTypeNone;
            props.location.type = cudaMemLocationTypeDevice;
            props.location.id = ctx->device;
            e = cudaMemPoolCreate(&s->pool, &props);
            uint64_t keep = s->opt.hbm_budget_bytes;
            if (e == cudaSuccess) e = cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
        if (e == cudaSuccess) e = cudaMalloc(&s->d_jobs, sizeof(Job) * 2 * slots);
        if (e == cudaSuccess) e = cudaMalloc(&s->d_states, sizeof(JobState) * 2 * slots);
        if (e == cudaSuccess) e = cudaMalloc(&s->d_ctl, sizeof(Ctl));
        for (int q = 0; q < 3 && e == cudaSuccess; ++q)
            e = cudaMalloc(&s->d_queue[q], sizeof(unsigned long long) * s->brick_cap);
        if (e == cudaSuccess) e = cudaMalloc(&s->d_stamps, sizeof(int32_t) * s->brick_cap);
        if (e == cudaSuccess) e = cudaMalloc(&s->d_descs, sizeof(PairDesc) * s->max_admit);
        if (e == cudaSuccess) e = cudaMalloc(&s->d_slot_descs, sizeof(PairDesc) * slots);
        if (e == cudaSuccess) e = cudaMalloc(&s->d_results, sizeof(hd_result) * slots);
        if (e == cudaSuccess) e = cudaMalloc(&s->d_retire, sizeof(uint32_t) * 2 * slots);
        if (e == cudaSuccess) e = cudaMalloc(&s->d_yield, sizeof(int32_t));
        if (e == cudaSuccess) e = cudaMemset(s->d_states, 0, sizeof(JobState) * 2 * slots);
        if (e == cudaSuccess) e = cudaMemset(s->d_ctl, 0, sizeof(Ctl));
        if (e == cudaSuccess) e = cudaMemset(s->d_stamps, 0, sizeof(int32_t) * s->brick_cap);
        if (e == cudaSuccess) e = cudaMemset(s->d_slot_descs, 0, sizeof(PairDesc) * slots);  // info = null: unused
        if (e == cudaSuccess) e = cudaMemset(s->d_yield, 0, sizeof(int32_t));
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_yield, cudaEventDisableTiming);
        // pinned: [Ctl][JobState x 2 slots][PairDesc x max_admit][hd_result x slots][retire list][yield word]
        s->off_h_results = align_up(align_up(sizeof(Ctl)) + align_up(sizeof(JobState) * 2 * slots) +
                                    sizeof(PairDesc) * s->max_admit);
        s->off_h_retire = align_up(s->off_h_results + sizeof(hd_result) * slots);
        s->off_h_yield = align_up(s->off_h_retire + sizeof(uint32_t) * 2 * slots);
        s->h_pinned_bytes = s->off_h_yield + sizeof(int32_t);
        if (e == cudaSuccess) e = cudaHostAlloc(&s->h_pinned, s->h_pinned_bytes, cudaHostAllocDefault);
        if (e != cudaSuccess) {
            cudaGetLastError();
            hd_server_destroy(s);
            return e == cudaErrorMemoryAllocation ? HD_ERR_OOM : HD_ERR_CUDA;
        }
    }
    s->slots.assign(slots, nullptr);
    s->slot_epoch.assign(slots, 0u);
    for (int i = slots - 1; i >= 0; --i) s->free_slots.push_back(i);
    s->worker = std::thread(worker_main, s);
    *out = s;
    return HD_OK;
}

hd_status hd_server_submit(hd_server* s, const hd_pair_desc* pair, uint64_t* ticket) {
    if (!s || !pair || !ticket || !pair->a || !pair->b) return HD_ERR_BAD_ARG;
    if ((pair->metric == HD_SE6 ? 0 : 1) != s->se) return HD_ERR_BAD_ARG;
    if (check_dims(nullptr, pair->W, pair->H, pair->D) != HD_OK) return HD_ERR_BAD_ARG;
    auto r = std::make_unique<Request>();
    r->W = pair->W;
    r->H = pair->H;
    r->D = pair->D;
    if (pair->on_device) {
        r->dev_a = pair->a;
        r->dev_b = pair->b;
    } else {
        const size_t nb = (size_t)pair->W * pair->H * pair->D;
        r->host_a.assign(pair->a, pair->a + nb);
        r->host_b.assign(pair->b, pair->b + nb);
    }
    plan_request(s, r.get());
    std::lock_guard<std::mutex> lk(s->mu);
    if ((int)s->waiting.size() >= s->opt.max_queue) return HD_ERR_BUSY;
    r->ticket = s->next_ticket++;
    *ticket = r->ticket;
    s->waiting.push_back(r.get());
    s->reqs[r->ticket] = std::move(r);
    s->stats.submitted += 1;
    if (s->in_tick && !s->yield_posted && !s->draining) {
        // a tick is running: advance the yield word so that its launch ends
        // at the next grid barrier and the next tick admits this request.
        // The copy may read a later (larger) generation than the one written
        // here, which ends the launch just the same.
        s->yield_posted = true;
        int32_t* hy = (int32_t*)((char*)s->h_pinned + s->off_h_yield);
        *hy = ++s->yield_gen;
        DeviceGuard g(s->ctx->device);
        cudaError_t e = cudaMemcpyAsync(s->d_yield, hy, sizeof(int32_t), cudaMemcpyHostToDevice, s->side);
        if (e == cudaSuccess) e = cudaEventRecord(s->ev_yield, s->side);
        if (e != cudaSuccess) cudaGetLastError();  // the tick then simply runs to its end
    }
    s->wake_seq.fetch_add(1, std::memory_order_release);
    s->cv.notify_all();
    return HD_OK;
}

hd_status hd_server_poll(hd_server* s, uint64_t ticket, hd_result* out) {
    if (!s || !out) return HD_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return HD_ERR_BAD_ARG;
    if (it->second->state != kDone) return HD_ERR_NOT_READY;
    *out = it->second->result;
    s->reqs.erase(it);
    return HD_OK;
}

hd_status hd_server_wait(hd_server* s, uint64_t ticket, int64_t timeout_ms, hd_result* out) {
    if (!s || !out) return HD_ERR_BAD_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return HD_ERR_BAD_ARG;
    Request* r = it->second.get();
    auto ready = [&] { return r->state == kDone; };
    // one deadline for the poll and the wait that follows it
    const auto deadline = std::chrono::steady_clock::now() + std::chrono::milliseconds(clamp_timeout_ms(timeout_ms));
    spin_wait(s, lk, ready, timeout_ms);
    if (timeout_ms < 0) {
        s->done_cv.wait(lk, ready);
    } else if (!s->done_cv.wait_until(lk, deadline, ready)) {
        return HD_ERR_NOT_READY;
    }
    *out = r->result;
    s->reqs.erase(ticket);
    return HD_OK;
}

hd_status hd_server_wait_any(hd_server* s, int64_t timeout_ms, uint64_t* ticket, hd_result* out) {
    if (!s || !ticket || !out) return HD_ERR_BAD_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    // one deadline for every round (a completion whose ticket another call
    // took sends the loop round again)
    const auto deadline = std::chrono::steady_clock::now() + std::chrono::milliseconds(clamp_timeout_ms(timeout_ms));
    for (;;) {
        // tickets already taken by hd_server_poll / hd_server_wait are skipped
        while (!s->done_order.empty() && !s->reqs.count(s->done_order.front())) s->done_order.pop_front();
        if (!s->done_order.empty()) break;
        auto ready = [&] { return !s->done_order.empty(); };
        int64_t left_ms = -1;
        if (timeout_ms >= 0) {
            left_ms = std::chrono::duration_cast<std::chrono::milliseconds>(deadline - std::chrono::steady_clock::now())
                          .count();
            if (left_ms < 0) return HD_ERR_NOT_READY;
        }
        if (spin_wait(s, lk, ready, left_ms)) continue;
        if (timeout_ms < 0) {
            s->done_cv.wait(lk, ready);
        } else if (!s->done_cv.wait_until(lk, deadline, ready)) {
            return HD_ERR_NOT_READY;
        }
    }
    const uint64_t t = s->done_order.front();
    s->done_order.pop_front();
    *ticket = t;
    *out = s->reqs[t]->result;
    s->reqs.erase(t);
    return HD_OK;
}

hd_status hd_server_cancel(hd_server* s, uint64_t ticket) {
    if (!s) return HD_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return HD_ERR_BAD_ARG;
    if (it->second->state == kDone) return HD_OK;
    it->second->cancel = true;
    s->wake_seq.fetch_add(1, std::memory_order_release);
    s->cv.notify_all();
    return HD_OK;
}

hd_status hd_server_get_stats(hd_server* s, hd_server_stats* out) {
    if (!s || !out) return HD_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->stats;
    out->waiting_pairs = s->waiting.size();
    unsigned long long res = 0;
    for (auto* r : s->slots) res += r != nullptr;
    out->resident_pairs = res;
    return HD_OK;
}

hd_status hd_server_destroy(hd_server* s) {
    if (!s) return HD_ERR_BAD_ARG;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->wake_seq.fetch_add(1, std::memory_order_release);
        s->cv.notify_all();
    }
    if (s->worker.joinable()) s->worker.join();
    {
        DeviceGuard g(s->ctx->device);
        for (auto* r : s->slots)
            if (r && r->resident) cudaFreeAsync(r->resident, s->stream);
        if (s->stream) cudaStreamSynchronize(s->stream);
        if (s->pool) cudaMemPoolDestroy(s->pool);
        cudaFree(s->d_jobs);
        cudaFree(s->d_states);
        cudaFree(s->d_ctl);
        for (auto* q : s->d_queue) cudaFree(q);
        cudaFree(s->d_stamps);
        cudaFree(s->d_descs);
        cudaFree(s->d_slot_descs);
        cudaFree(s->d_results);
        cudaFree(s->d_retire);
        cudaFree(s->d_yield);
        if (s->side) {
            cudaStreamSynchronize(s->side);
            cudaStreamDestroy(s->side);
        }
        if (s->ev_yield) cudaEventDestroy(s->ev_yield);
        if (s->h_pinned) cudaFreeHost(s->h_pinned);
        if (s->stream) cudaStreamDestroy(s->stream);
        cudaGetLastError();
    }
    delete s;
    return HD_OK;
}

}  // extern "C"
