// hd_device.cuh -- device-side data structures shared by the packing, set-up
// and dilation kernels and by the host orchestration.
//
// Layout in HBM (one pair):
//   a, b        uint8 masks, W x H x D, x fastest (caller's or staged copy)
//   pa, pb      the full volume bit-packed along x: 32 voxels per uint32,
//               bit i of word w of row (y, z) is voxel x = 32 w + i;
//               wxf = ceil(W / 32) words per row, rows padded with zero
//               words to a multiple of 4 (packed_pitch), word w of row
//               (y, z) at (z * H + y) * packed_pitch + w
//   per direction (a "job": dilate a source mask until it covers a target):
//     buf[0], buf[1]  ping-pong dilation state over the job's domain
//     U               target voxels not yet covered (one-step kernel; the
//                     blocked kernel finds newly covered voxels as target
//                     voxels in a step's result but not in its input)
//               domain layout [z][y][pitch] words, pitch = ceil(wx / 4) * 4,
//               pad words zero.  The domain is the bounding box of A u B with
//               x widened to whole words (6-neighbour element), widened by
//               one more word in x and one row and plane in y and z
//               (18-neighbour element: shortest paths may step one voxel
//               out of the box, see domain_box).  The blocked kernel reads its
//               first iteration's state and the target from the packed
//               masks in place when the domain can start on a multiple of 4
//               words without adding a brick column; else from crops of A
//               and B in the domain layout (in the U slots of the two jobs).
//   bricks      the unit of work of the persistent loop, one warp per brick:
//               one-step kernel (hd_solve.cuh): BXW words (x) x (32 / BXW)
//               rows (y) x BZ planes (z), lane (lx, ly) owns one word column
//               and walks z; blocked kernel (hd_solve_tb.cuh): 4 words x
//               (32 - 2T) rows x BZ planes, lane = one row.
#pragma once
#include <stdint.h>

#include "hd/hd.h"

namespace hdk {

constexpr int kMaxPairsPerLaunch = 65535;

// Bounding box and counts of one pair, accumulated by the packing kernel.
struct PairInfo {
    unsigned long long n_a, n_b, n_ab;
    int32_t bb[6];  // min / max x word, y, z of A u B (min = INT_MAX, max = -1 when empty)
    int32_t pad[2];
};

// Packing / set-up descriptor of one pair (host-written).
struct PairDesc {
    const uint8_t* a;
    const uint8_t* b;
    uint32_t* pa;      // full packed A, packed_pitch(W) * H * D words (16-byte aligned)
    uint32_t* pb;
    uint32_t* jb[2][3];  // per job: buf0, buf1, U (capacity: pitch_full * H * D words each)
    unsigned long long* hist[2];  // per job: kmax + 1 counters
    int32_t W, H, D, wxf;  // wxf = ceil(W / 32) words of a row (pitch: packed_pitch(W))
    int32_t se;          // 0: 6-neighbour, 1: 18-neighbour (forBench default)
    int32_t aligned;     // a and b are 16-byte aligned
    int32_t kmax;        // iteration cap per job
    int32_t job0;        // index of this pair's first job (jobs 2p, 2p+1)
    unsigned long long brick0[2];  // first global brick id of each job
    PairInfo* info;
    int32_t* tstamp[2];            // instrumented runs only (else null)
    unsigned long long* tcount[2];
    uint32_t epoch;                // queue-entry tag of this pair's jobs (slot reuse)
    uint32_t pad_;
    long long tile0;               // first packing tile of this pair
    long long stile0;              // first set-up tile of this pair
};

// Packing and set-up split every pair into tiles; one launch covers the
// tiles of all pairs.  Packing tiles are kPackTileWords words of the packed
// volume (wxf * H * D words), set-up tiles kTileWords words of the domain
// capacity (rows padded to 4 words: roundup(wxf, 4) * H * D).
constexpr long long kTileWords = 1024;
constexpr long long kPackTileWords = 1024;

// Temporally blocked dilation kernel (hd_solve_tb.cuh): each warp streams
// the BZ + 2T planes of its brick through a ring of shared-memory slots
// kTbPrefetch planes ahead of the one being computed; a plane stays until
// its final step has been compared with it, T planes later.  A lane holds
// tb_rows(T) consecutive rows of the brick (the warp 32 tb_rows(T) rows, 2T
// of them halo): a row's neighbours in y come from the lane's own registers
// but for the first and last row, which take one shuffle each.  Per warp:
// the slots (32 tb_rows rows x (16 B interior + 8 B halo words)) and the
// brick's target rows (BZ planes x 32 tb_rows rows x 16 B).  Resident CTAs
// of kTbWarps warps per SM: tb_min_ctas (the registers of the levels' state
// decide).
constexpr int kTbWarps = 4;
constexpr int kTbPrefetch = 2;
// One row per lane: two (half the shuffles per row, a 64-row block with 2T
// halo rows) measured slower on every workload (218 registers at 4 steps,
// 2 CTAs per SM: 512x512x256 0.129 against 0.113 ms, 512^3 5.7 against 3.8
// ms, the ragged batch 2.35 against 1.54 ms).
__host__ __device__ constexpr int tb_rows(int) { return 1; }
__host__ __device__ constexpr int tb_min_ctas(int T) {
    return tb_rows(T) == 1 ? (T <= 2 ? 4 : 3) : (T <= 2 ? 3 : 2);
}
__host__ __device__ constexpr int tb_brick_rows(int T) { return 32 * tb_rows(T) - 2 * T; }
__host__ __device__ constexpr int tb_ring_slots(int T, int BZ) {
    return T + 1 + kTbPrefetch >= BZ + 2 * T ? BZ + 2 * T : T + 1 + kTbPrefetch;
}
__host__ __device__ constexpr int tb_warp_bytes(int T, int BZ) {
    return (tb_ring_slots(T, BZ) * 32 * 24 + BZ * 32 * 16) * tb_rows(T);
}
__host__ __device__ __forceinline__ long long pack_words(int W, int H, int D) {
    return (long long)((W + 31) / 32) * H * D;
}
// Row pitch of the packed volumes (words): 16-byte aligned rows.
__host__ __device__ __forceinline__ int packed_pitch(int W) { return (((W + 31) / 32) + 3) & ~3; }
__host__ __device__ __forceinline__ long long domain_cap_words(int W, int H, int D) {
    return (long long)((((W + 31) / 32) + 3) & ~3) * H * D;
}
__host__ __device__ __forceinline__ long long tiles_of(long long words) { return (words + kTileWords - 1) / kTileWords; }
__host__ __device__ __forceinline__ long long pack_tiles_of(int W, int H, int D) {
    return (pack_words(W, H, D) + kPackTileWords - 1) / kPackTileWords;
}
// Bricks of the full volume's brick grid (an upper bound of any domain's).
__host__ __device__ __forceinline__ long long bricks_max(int W, int H, int D, int bxw, int by, int bz) {
    return (long long)((((W + 31) / 32) + bxw - 1) / bxw) * ((H + by - 1) / by) * ((D + bz - 1) / bz);
}

// Set-up modes: what the dilation kernel will read (see setup_kernel).
constexpr int kSetupBlocked = 0;         // blocked kernel: packed masks in place if that adds no brick column, else crops
constexpr int kSetupOneStep = 1;         // one-step kernel: cropped ping-pong buffers and uncovered target
constexpr int kSetupBlockedCrop = 2;     // blocked kernel: crops of A and B
constexpr int kSetupBlockedInPlace = 3;  // blocked kernel: packed masks in place
constexpr long long kSetupBricks = 2048; // bricks per set-up tile when nothing is copied

// Set-up tiles of one pair: kTileWords words of the domain capacity when
// the mode may copy, else kSetupBricks bricks of the largest brick grid.
__host__ __device__ __forceinline__ long long setup_tiles_of(int W, int H, int D, int mode, int bxw, int by, int bz) {
    if (mode != kSetupBlockedInPlace) return tiles_of(domain_cap_words(W, H, D));
    const long long b = bricks_max(W, H, D, bxw, by, bz);
    return b > 0 ? (b + kSetupBricks - 1) / kSetupBricks : 1;
}

// One direction of a pair, written by the set-up kernel.  The fields a
// queue item of the blocked kernel reads come first, within one 128-byte
// line (the rest serve the one-step kernel and instrumented runs).
struct __align__(128) Job {
    uint32_t* buf[2];
    // blocked kernel: the source (state of the first iteration) and the
    // target, read-only: either the packed masks pa / pb read in place
    // (domain rows start on 16-byte boundaries) or crops of them in the
    // domain layout; domain word (x, y, z) is at
    // vol + ((z + vz0) * vh + y + vy0) * vpitch + vx0 + x
    const uint32_t* vol[2];
    int32_t wx, h, d;          // domain: words per row, rows, planes
    int32_t pitch;             // row pitch (words)
    uint32_t tailmask;         // valid bits of a row's last word
    int32_t nbx, nby, nbz;     // brick grid
    int32_t k0;                // global iteration at which local step 1 runs
    int32_t kmax;              // local step cap
    uint32_t epoch;            // entries carrying another epoch belong to a previous user of the slot
    int32_t vpitch, vh;        // vol[]: row pitch (words) and rows per plane
    int32_t vx0, vy0, vz0;     // vol[]: domain origin (words, rows, planes)
    unsigned long long brick0;
    unsigned long long* hist;  // newly covered voxels per local step
    // ---- one-step kernel, instrumented runs
    uint32_t* U;
    int32_t wv;                // domain width in voxels
    int32_t ox, oy, oz;        // domain origin in the full volume (voxels)
    int32_t tw, th;            // full-volume 32^3 tile grid (x, y), instrumented runs
    int32_t* tstamp;           // instrumented runs: per full-volume tile, last marked step
    unsigned long long* tcount;  // instrumented runs: tiles per step
};
static_assert(__builtin_offsetof(Job, U) <= 128, "hot fields of a job within its first line");

// Queue entry: epoch (8 bits) | 1 (bit 55: an entry is never zero, so a
// cleared slot reads as empty) | job (23 bits) | local brick (32 bits).
constexpr unsigned kEntryJobMask = 0x7fffffu;
__host__ __device__ __forceinline__ unsigned long long make_entry(uint32_t epoch, uint32_t job, uint32_t lb) {
    return ((unsigned long long)(epoch & 0xffu) << 56) | (1ull << 55) |
           ((unsigned long long)(job & kEntryJobMask) << 32) | lb;
}

// Mutable per-job state.
struct JobState {
    unsigned long long sum;        // sum over covered target voxels of their step
    unsigned long long remaining;  // target voxels not yet covered
    unsigned long long bricks;     // bricks processed (instrumented runs)
    int32_t hd;                    // last step that covered something
    int32_t last_k;                // last local step run
    int32_t status;                // 0 ok, else hd_status
    int32_t active;                // 1 while the job takes part in the dilation loop
};

// Loop control shared by all CTAs of the persistent kernel.
struct Ctl {
    // barrier release word, written once per barrier by the last CTA to
    // arrive: generation (bits 32-63) | continue flag (bit 31) | length of
    // the next step's queue (bits 0-30)
    unsigned long long release;
    unsigned int bar_count;
    int32_t err;           // first error (hd_status), 0 = none
    int32_t jobs_active;   // jobs with uncovered target voxels
    unsigned int qcount[3];
    int32_t g_end;         // next global iteration (written at exit)
    int32_t iters_run;
    // blocked kernel: items of a step's queue handed out past its static
    // share (per step modulo 3; the barrier zeroes the next step's count)
    unsigned int claim[3];
    int32_t pad[3];
};

struct SolveParams {
    Job* jobs;
    JobState* states;
    unsigned long long* queue[3];  // entries, see make_entry
    int32_t* stamps;               // per global brick: last iteration it was queued for
    Ctl* ctl;
    int32_t* map[2];               // optional dense per-voxel distance maps (per pair: job 0 / 1)
    int32_t map_w, map_h, map_d;   // full-volume sizes for the maps
    int32_t g0;                    // first global iteration of this launch
    int32_t max_iters;             // iterations this launch may run
    int32_t stats;                 // instrumented run
    int32_t spread;                // queue item i goes to warp (i mod warps) numbered CTA-major (0) or SM-spread (1)
    long long timeout_ns;          // one barrier wait
    // device-side result decode at the end of the launch (asynchronous
    // entries; out == nullptr: the host decodes)
    const PairDesc* descs;
    int32_t npairs;
    float pct;                     // robust HD percentile
    hd_result* out;                // out[i] = result of pair i
    // serving: decode only pairs whose descriptor is live (info != null) and
    // whose jobs have both finished; the others' out[i] is left as it is
    int32_t decode_done_only;
    // serving: a word the host advances while a launch runs (requests
    // waiting for admission); once it differs from yield_gen the loop ends
    // at the next grid barrier (null: never)
    const int32_t* yield;
    int32_t yield_gen;
    // blocked kernel: jobs job_cache_base .. job_cache_base + job_cache - 1
    // (at most kJobCache: a single pair, or a server tick with one resident
    // request) are read from a per-CTA copy of their first line, taken at the
    // start of the launch (no kernel writes a job while the dilation runs);
    // job_cache 0: none
    int32_t job_cache;
    int32_t job_cache_base;
    // blocked kernel: the leading slots of each queue that are zero before a
    // step's entries are written (the set-up zeroes them; the kernel keeps
    // them so); a warp numbered below reads its first entry of the next
    // step before the grid barrier (see solve_tb_kernel); 0: never
    int32_t spec_first;
};
constexpr int kSpecSlots = 4096;  // at least the warps of any persistent grid
constexpr int kJobCache = 2;

}  // namespace hdk
