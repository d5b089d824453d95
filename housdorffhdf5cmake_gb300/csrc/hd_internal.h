// hd_internal.h -- host-side context and the shared pair pipeline.
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "hd/hd.h"
#include "hd_device.cuh"

namespace hdh {

// Grow-only device allocation.
struct DeviceArena {
    void* ptr = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t n);
    void release();
};

// Grow-only pinned host allocation (staging for descriptors and results).
struct PinnedArena {
    void* ptr = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t n);
    void release();
};

// Dilation kernel and brick geometry.
//   kernel 1: one step per grid barrier, bricks bxw words x 32/bxw rows x bz planes
//   kernel 2: `steps` steps per grid barrier, bricks 4 words x (32 - 2 steps) rows x bz planes
struct Shape {  // default: the autotuner's choice on the 512x512x256, 512^3 and ragged-batch workloads
    int kernel = 2;
    int bxw = 4;
    int by = 28;
    int bz = 8;
    int steps = 2;
    int ctas_per_sm = 0;
    // queue schedule: pair order of a batch (0 = as given, 1 = largest
    // first: its bricks get the lowest ids and lead the first queue) and the
    // mapping of queue items to warps (0 = CTA-major: consecutive items on
    // the warps of one CTA, 1 = spread: consecutive items on different SMs)
    int order = 0;
    int spread = 0;
    int threads = 128;  // CTA size of the persistent launch
    int smem = 0;       // dynamic shared memory per CTA
    void finish() {
        if (kernel == 2) {
            // kTbWarps warps per CTA, each with a ring of streamed planes and
            // the brick's target rows in shared memory
            bxw = 4;
            by = hdk::tb_brick_rows(steps);
            threads = hdk::kTbWarps * 32;
            smem = hdk::kTbWarps * hdk::tb_warp_bytes(steps, bz);
        } else {
            by = 32 / bxw;
            steps = 1;
            threads = 256;
            smem = 0;
        }
    }
};

// One tuned shape per (element, volume class).
struct TuneEntry {
    Shape shape;
    double us = 0.0;  // measured time of the winner (informational)
};

struct TuneTable {
    std::map<std::string, TuneEntry> entries;
    bool load(const std::string& path);
    bool save(const std::string& path) const;
};

// Key of a workload class: element and log2 buckets of the mean volume and
// the pair count (1, 2-15, 16+).
std::string tune_key(int se, double mean_voxels, int npairs);

// Device switch for the duration of one call (restores the caller's device).
struct DeviceGuard {
    int prev = -1;
    bool ok = false;
    explicit DeviceGuard(int dev);
    ~DeviceGuard();
};

}  // namespace hdh

struct hd_context {
    int device = 0;
    hd_options opt{};
    std::string tuning_path;
    cudaStream_t stream = nullptr;
    int sm_count = 0;
    int pageable_ats = 0;  // device reads pageable host memory through the host page tables
    std::mutex mu;
    std::string last_error;
    int g_next = 1;  // global iteration counter, monotonic across calls (brick stamps rely on it)
    hdh::DeviceArena arena;   // per-call buffers
    hdh::DeviceArena stamps;  // per-brick queue stamps, never cleared
    static constexpr int kMaxDilationParts = 3;  // the split path's dilation partitions, at most
    // the stamps of the split path's dilation partitions 1, 2: their
    // dilations may run beside those of partition 0, which uses `stamps`
    // (same size and resets as stamps)
    hdh::DeviceArena part_stamps[kMaxDilationParts - 1];
    size_t stamp_slots = 0;
    hdh::PinnedArena pinned;
    std::map<const void*, int> occupancy;  // persistent kernel -> resident CTAs per SM
    hdh::TuneTable tune;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};  // record_timings: before pack/setup/solve, after solve
    hd_timings last_timings{};
    // asynchronous calls: descriptor staging buffers that stay untouched
    // until their upload has run (an event per buffer)
    static constexpr int kAsyncSlots = 4;
    hdh::PinnedArena async_stage[kAsyncSlots];
    cudaEvent_t async_done[kAsyncSlots] = {nullptr, nullptr, nullptr, nullptr};
    int async_next = 0;
    // asynchronous calls with host masks: two device buffers the masks are
    // copied into on a copy stream, so a pair's copy overlaps the previous
    // pair's kernels (ready: copy done; free: the packing that read it done)
    cudaStream_t copy_stream = nullptr;
    hdh::DeviceArena mask_stage[2];
    cudaEvent_t mask_ready[2] = {nullptr, nullptr}, mask_free[2] = {nullptr, nullptr};
    int mask_next = 0;
    // asynchronous single pairs on split SMs (green contexts): pairs are
    // packed and set up on a few SMs while earlier pairs dilate on the rest,
    // split in up to three groups that dilate consecutive pairs side by side;
    // the pairs take two workspaces per group in turn
    struct Split {
        int state = 0;                      // 0 not tried, 1 ready, -1 unavailable
        // CUgreenCtx: [0] packing and set-up, [1 + p] dilation partition p
        void* green[1 + kMaxDilationParts] = {};
        // solve[p]: the dilations of partition p; workspace i dilates on
        // partition i % parts
        cudaStream_t solve[kMaxDilationParts] = {}, prep = nullptr;
        int solve_sms[kMaxDilationParts] = {}, prep_sms = 0;
        int parts = 1;
        cudaEvent_t caller = nullptr, prep_done = nullptr;
        // workspaces in turn, two per dilation partition (a pair's packing
        // then need not wait for the dilation before last in its partition)
        static constexpr int kWorkspaces = 2 * kMaxDilationParts;
        int nws = 2;
        cudaEvent_t ws_free[kWorkspaces] = {};  // the dilation that last used workspace i
        int next = 0;
        bool pending = false;  // a dilation the caller's stream has not waited for yet
        // record_timings: events of the latest call on the split SMs, each on
        // the stream its kernel ran on (before pack, after pack, after
        // set-up; before and after the dilation); read by
        // hd_context_last_timings once they have completed
        cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
        bool timed = false;
        hd_timings shape{};  // the fields of hd_timings that are not times
    } split;
    hdh::DeviceArena ws_arena[Split::kWorkspaces - 1];  // the split path's workspaces 1, 2, ...
};

namespace hdh {

// One pair entering the pipeline: device-addressable mask pointers.
struct PairIn {
    const uint8_t* a;
    const uint8_t* b;
    int32_t W, H, D;
    const uint8_t* host_a;  // non-null: stage from this host buffer
    const uint8_t* host_b;
};

struct RunOpts {
    int se = 0;
    int stats = 0;
    int32_t* map_a = nullptr;
    int32_t* map_b = nullptr;
    uint64_t* tiles_ab = nullptr;
    uint64_t* tiles_ba = nullptr;
    int32_t tiles_len = 0;
    uint64_t* bricks = nullptr;
    bool force_shape = false;  // use `shape` as given (autotuner)
    Shape shape;
    hd_result* async_out = nullptr;  // device memory: enqueue only, results decoded on the device
    bool pipelined = false;          // with async_out: the result may complete after a later flush
    bool ordered = false;            // the pairs are already in the shape's order (internal)
};

hd_status set_error(hd_context* ctx, hd_status st, const char* fmt, ...);
hd_status cuda_fail(hd_context* ctx, cudaError_t e, const char* where);

// Validates sizes of one pair (limits of the 32-bit word offsets).
hd_status check_dims(hd_context* ctx, int32_t W, int32_t H, int32_t D);

// Host pointer -> device-addressable pointer when the kernels may read it in
// place (pinned / registered memory, or pageable memory on a device that
// walks the host page tables); nullptr if it must be staged.
const uint8_t* zero_copy_ptr(hd_context* ctx, const uint8_t* p);

// The pipeline: pack -> set-up -> one persistent dilation launch -> results.
// Caller holds ctx->mu and the device guard.
hd_status run_pairs(hd_context* ctx, const PairIn* pairs, int n, cudaStream_t s, const RunOpts& ro,
                    hd_result* out);

// Kernel and brick shape for a workload (options, then tuning table, then default).
Shape pick_shape(hd_context* ctx, int se, const PairIn* pairs, int n);

// Host stub of the persistent kernel of a shape (nullptr if not compiled in).
const void* solve_fn_of(int se, const Shape& sh);

// Pair result from the packing counts and the two jobs' states (s0 dilates A
// and covers B, s1 the reverse) and their per-step histograms.
hd_status decode_result(const hdk::PairInfo& I, const hdk::JobState& s0, const hdk::JobState& s1,
                        const uint64_t* hist_ab, const uint64_t* hist_ba, int kp1, int iters, int err,
                        float pct, hd_result* out);

// Resident CTAs per SM of a persistent kernel launched with `threads` threads
// and `smem` bytes of dynamic shared memory (cached per context; raises the
// kernel's dynamic shared memory limit first when needed).
int occupancy_of(hd_context* ctx, const void* fn, int threads, int smem);

// Split SMs for asynchronous single pairs (hd_context::Split): set up on
// first use; false when green contexts are unavailable.  split_release ends it.
bool split_ready(hd_context* ctx);
void split_release(hd_context* ctx);

// Percentile HD of one direction with the reference's float stopping rule.
int robust_k(const uint64_t* hist, int len, uint64_t total, float p);

}  // namespace hdh
