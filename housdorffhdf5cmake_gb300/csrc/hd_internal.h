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

// One tuned brick shape per (element, volume class).
struct TuneEntry {
    int bxw = 4;
    int bz = 8;
    int ctas_per_sm = 0;
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
    size_t stamp_slots = 0;
    hdh::PinnedArena pinned;
    std::map<const void*, int> occupancy;  // persistent kernel -> resident CTAs per SM
    hdh::TuneTable tune;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};  // record_timings: before pack/setup/solve, after solve
    hd_timings last_timings{};
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
    int bxw = 0, bz = 0, ctas_per_sm = 0;  // 0 = from options / tuning table
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

// Brick shape for a workload (options, then tuning table, then default).
void pick_shape(hd_context* ctx, int se, const PairIn* pairs, int n, int* bxw, int* bz, int* cps);

// Pair result from the packing counts and the two jobs' states (s0 dilates A
// and covers B, s1 the reverse) and their per-step histograms.
hd_status decode_result(const hdk::PairInfo& I, const hdk::JobState& s0, const hdk::JobState& s1,
                        const uint64_t* hist_ab, const uint64_t* hist_ba, int kp1, int iters, int err,
                        float pct, hd_result* out);

// Resident CTAs per SM of a persistent kernel (cached per context).
int occupancy_of(hd_context* ctx, const void* fn);

// Percentile HD of one direction with the reference's float stopping rule.
int robust_k(const uint64_t* hist, int len, uint64_t total, float p);

}  // namespace hdh
