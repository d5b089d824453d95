// hd_noalloc.cu -- the one entry point that allocates nothing.
//
// Some callers cannot allocate GPU memory at the moment they need a distance:
// code running under a framework's allocator that owns all device memory, a
// real-time loop that must not call cudaMalloc / cudaFree (they can block and
// synchronise the device), or a host that has no free HBM to give.  For them,
// hd_compute_u8_device_noalloc computes one pair with every intermediate
// buffer (packed masks, the two dilation jobs' state, work queues, brick
// stamps, loop control) inside the fixed array g_scratch below, which lives in
// the library's device image: each GPU that loads the library holds it until
// the process exits.  Inputs and the result are the caller's device memory.
//
// Rules of use:
//   - sizes: the pair must fit g_scratch (kScratchBytes = 80 MiB, about one
//     byte per voxel; 512 x 512 x 256 fits); larger pairs are rejected with
//     HD_ERR_BAD_ARG before anything is launched;
//   - the first call on a device looks up g_scratch's device address
//     (cudaGetSymbolAddress) with that device current; make that first call
//     before any stream capture;
//   - all calls share g_scratch, which keeps the previous call's contents
//     (each call clears what must start at zero); calls that overlap on the
//     GPU, on different streams or from different threads, race on it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "hd/hd.h"
#include "hd_device.cuh"
#include "hd_kernels.h"

namespace {

constexpr size_t kScratchBytes = 80ull << 20;
constexpr int kMaxDevices = 64;
constexpr int kBxw = 4, kBz = 8;  // brick shape used by this entry point

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

struct DeviceSlot {
    bool ready = false;
    unsigned char* scratch = nullptr;  // device address of g_scratch on this device
    int sm_count = 0;
    int ctas_per_sm[2] = {0, 0};       // persistent kernel occupancy per element
};

std::mutex g_mu;
DeviceSlot g_slots[kMaxDevices];

inline size_t up256(size_t x) { return (x + 255) / 256 * 256; }

struct Layout {
    size_t ctl, states, info, desc, jobs, hist, queue[3], stamps, pa, pb, jb[2][3], total;
    int wxf, kmax;
    long long bricks, dom_words;
};

Layout plan(int W, int H, int D) {
    Layout L{};
    L.wxf = (W + 31) / 32;
    const long long pitch = (L.wxf + 3) / 4 * 4;
    L.dom_words = pitch * H * D;
    const int by = 32 / kBxw;
    L.bricks = (long long)((L.wxf + kBxw - 1) / kBxw) * ((H + by - 1) / by) * ((D + kBz - 1) / kBz);
    L.kmax = W + H + D;
    size_t cur = 0;
    auto take = [&](size_t n) { const size_t o = cur; cur = up256(cur + n); return o; };
    L.ctl = take(sizeof(hdk::Ctl));
    L.states = take(2 * sizeof(hdk::JobState));
    L.info = take(sizeof(hdk::PairInfo));
    L.desc = take(sizeof(hdk::PairDesc));
    L.jobs = take(2 * sizeof(hdk::Job));
    L.hist = take(2 * sizeof(unsigned long long) * (L.kmax + 1));
    for (auto& q : L.queue) q = take(sizeof(unsigned long long) * 2 * L.bricks);
    L.stamps = take(sizeof(int32_t) * 2 * L.bricks);
    const size_t full = 4ull * hdk::packed_pitch(W) * H * D;
    L.pa = take(full);
    L.pb = take(full);
    for (int j = 0; j < 2; ++j)
        for (int b = 0; b < 3; ++b) L.jb[j][b] = take(4ull * L.dom_words);
    L.total = cur;
    return L;
}

// Writes the pair descriptor, the packing counters' start values and a clean
// loop-control block into the scratch (one thread; no host-to-device copy).
__global__ void noalloc_prepare(unsigned char* base, Layout L, const uint8_t* a, const uint8_t* b, int W, int H,
                                int D, int se) {
    hdk::Ctl* ctl = (hdk::Ctl*)(base + L.ctl);
    memset(ctl, 0, sizeof(hdk::Ctl));
    hdk::PairInfo* I = (hdk::PairInfo*)(base + L.info);
    memset(I, 0, sizeof(hdk::PairInfo));
    I->bb[0] = I->bb[2] = I->bb[4] = 0x7fffffff;
    I->bb[1] = I->bb[3] = I->bb[5] = -1;
    hdk::PairDesc* P = (hdk::PairDesc*)(base + L.desc);
    memset(P, 0, sizeof(hdk::PairDesc));
    P->a = a;
    P->b = b;
    P->pa = (uint32_t*)(base + L.pa);
    P->pb = (uint32_t*)(base + L.pb);
    for (int j = 0; j < 2; ++j) {
        for (int k = 0; k < 3; ++k) P->jb[j][k] = (uint32_t*)(base + L.jb[j][k]);
        P->hist[j] = (unsigned long long*)(base + L.hist) + (size_t)j * (L.kmax + 1);
        P->brick0[j] = (unsigned long long)j * L.bricks;
    }
    P->W = W;
    P->H = H;
    P->D = D;
    P->wxf = L.wxf;
    P->se = se;
    P->aligned = ((((uintptr_t)a) | ((uintptr_t)b)) & 15) == 0;
    P->kmax = L.kmax;
    P->job0 = 0;
    P->info = I;
    P->tile0 = 0;
    P->stile0 = 0;
}

}  // namespace

extern "C" hd_status hd_compute_u8_device_noalloc(const uint8_t* d_a, const uint8_t* d_b, int32_t W, int32_t H,
                                                  int32_t D, hd_metric metric, void* stream, hd_result* d_out) {
    if (!d_a || !d_b || !d_out || W <= 0 || H <= 0 || D <= 0) return HD_ERR_BAD_ARG;
    if (metric != HD_SE6 && metric != HD_SE18_FORBENCH) return HD_ERR_BAD_ARG;
    if ((long long)W * H * D > (1LL << 31)) return HD_ERR_BAD_ARG;
    const Layout L = plan(W, H, D);
    if (L.total > kScratchBytes) return HD_ERR_BAD_ARG;  // does not fit the fixed scratch
    const int se = metric == HD_SE6 ? 0 : 1;
    const void* solve = hdk::solve_kernel_ptr(se, kBxw, kBz);
    if (!solve) return HD_ERR_BAD_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return HD_ERR_CUDA;
    }
    DeviceSlot* slot = &g_slots[dev];
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!slot->ready) {
            // once per device, with that device current: the scratch's device address
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
            if (e == cudaSuccess) e = cudaDeviceGetAttribute(&slot->sm_count, cudaDevAttrMultiProcessorCount, dev);
            for (int s = 0; s < 2 && e == cudaSuccess; ++s)
                e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&slot->ctas_per_sm[s], hdk::solve_kernel_ptr(s, kBxw, kBz),
                                                                  256, 0);
            if (e != cudaSuccess || p == nullptr) {
                cudaGetLastError();
                return HD_ERR_CUDA;
            }
            slot->scratch = (unsigned char*)p;
            slot->ready = true;
        }
    }
    cudaStream_t s = (cudaStream_t)stream;
    unsigned char* base = slot->scratch;
    // The layout moves with the volume's size, so the brick stamps may sit on
    // bytes of an earlier call: clear them and start the step count at 1.
    const int g0 = 1;
    cudaError_t e = cudaMemsetAsync(base + L.stamps, 0, sizeof(int32_t) * 2 * L.bricks, s);
    if (e == cudaSuccess) {
        noalloc_prepare<<<1, 1, 0, s>>>(base, L, d_a, d_b, W, H, D, se);
        e = cudaGetLastError();
    }
    const hdk::PairDesc* desc = (const hdk::PairDesc*)(base + L.desc);
    const long long ptiles = hdk::pack_tiles_of(W, H, D);
    const long long stiles = hdk::setup_tiles_of(W, H, D, hdk::kSetupOneStep, kBxw, 32 / kBxw, kBz);
    const int cap_ctas = std::max(slot->sm_count * 8, 1);
    if (e == cudaSuccess)  // nonzero bytes are foreground
        e = hdk::launch_pack(desc, 1, ptiles, (int)std::min<long long>(cap_ctas, ptiles), 0, 0, s);
    hdk::Job* jobs = (hdk::Job*)(base + L.jobs);
    hdk::JobState* states = (hdk::JobState*)(base + L.states);
    hdk::Ctl* ctl = (hdk::Ctl*)(base + L.ctl);
    unsigned long long* q[3] = {(unsigned long long*)(base + L.queue[0]), (unsigned long long*)(base + L.queue[1]),
                                (unsigned long long*)(base + L.queue[2])};
    if (e == cudaSuccess)
        e = hdk::launch_setup(desc, 1, stiles, 0, jobs, states, q[g0 % 3], ctl,
                              g0, kBxw, 32 / kBxw, kBz, hdk::kSetupOneStep, s);
    if (e == cudaSuccess) {
        hdk::SolveParams sp{};
        sp.jobs = jobs;
        sp.states = states;
        for (int i = 0; i < 3; ++i) sp.queue[i] = q[i];
        sp.stamps = (int32_t*)(base + L.stamps);
        sp.ctl = ctl;
        sp.map_w = W;
        sp.map_h = H;
        sp.map_d = D;
        sp.g0 = g0;
        sp.max_iters = L.kmax + 2;
        sp.timeout_ns = 10000000000LL;
        sp.descs = desc;  // the launch decodes the result into d_out
        sp.npairs = 1;
        sp.pct = 0.95f;
        sp.out = d_out;
        void* args[] = {&sp};
        e = cudaLaunchCooperativeKernel(solve, dim3(slot->sm_count * std::max(1, slot->ctas_per_sm[se])), dim3(256),
                                        args, 0, s);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return HD_ERR_CUDA;
    }
    return HD_OK;
}
