// ref_kernel.cpp -- runs the reference's own `dilate` kernel
// (forBench/HausdorffDistance.cu:21-98), compiled from the reference source to
// PTX by oracle/ref_kernel.py, through the CUDA driver API.
//
// TEST INFRASTRUCTURE ONLY: it produces golden HDs that pin the CPU oracle.
// The host loop below restates computeDistance's loop
// (forBench/HausdorffDistance.cu:146-172): set `finished` to 1, launch
// `dilate` over all voxels with 512-thread blocks (:110-111,156), copy Write
// to Read for both masks (:161-162), read `finished` back (:167), count.  It
// never feeds a pair with exactly one empty mask (the reference loops forever
// on it) and it stops after max_trips loop trips, so every launch ends.
#include <cuda.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

namespace {
#define CK(x)                                   \
    do {                                        \
        CUresult r_ = (x);                      \
        if (r_ != CUDA_SUCCESS) { rc = -(int)r_; goto done; } \
    } while (0)
}  // namespace

// Returns 0 and the HD in *hd_out, 1 if the pair has exactly one empty mask
// (not run), 2 if max_trips was reached, negative on a CUDA error.
extern "C" int ref_forbench_hd(const char* ptx_path, const uint8_t* a, const uint8_t* b, int W, int H,
                               int D, int max_trips, int* hd_out) {
    const size_t N = (size_t)W * H * D;
    size_t na = 0, nb = 0;
    for (size_t i = 0; i < N; ++i) { na += a[i] != 0; nb += b[i] != 0; }
    if ((na == 0) != (nb == 0)) return 1;
    std::ifstream f(ptx_path);
    if (!f) return -1000;
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string ptx = ss.str();
    std::vector<uint8_t> ha(N), hb(N);
    for (size_t i = 0; i < N; ++i) { ha[i] = a[i] != 0; hb[i] = b[i] != 0; }
    int rc = 0;
    CUdevice dev;
    CUcontext ctx = nullptr;
    CUmodule mod = nullptr;
    CUfunction fn;
    CUdeviceptr gW, gH, gD, gFin, d1 = 0, d2 = 0, r1 = 0, r2 = 0, w1 = 0, w2 = 0;
    size_t sz;
    int distance = -1, fin = 0, one = 1;
    const unsigned threads = 512, blocks = (unsigned)((N + threads - 1) / threads);
    void* args[6];
    CK(cuInit(0));
    CK(cuDeviceGet(&dev, 0));
    CK(cuDevicePrimaryCtxRetain(&ctx, dev));
    CK(cuCtxPushCurrent(ctx));
    CK(cuModuleLoadData(&mod, ptx.c_str()));
    CK(cuModuleGetFunction(&fn, mod, "_Z6dilatePKbS0_S0_S0_PbS1_"));
    CK(cuModuleGetGlobal(&gW, &sz, mod, "WIDTH"));
    CK(cuModuleGetGlobal(&gH, &sz, mod, "HEIGHT"));
    CK(cuModuleGetGlobal(&gD, &sz, mod, "DEPTH"));
    CK(cuModuleGetGlobal(&gFin, &sz, mod, "finished"));
    CK(cuMemcpyHtoD(gW, &W, sizeof W));
    CK(cuMemcpyHtoD(gH, &H, sizeof H));
    CK(cuMemcpyHtoD(gD, &D, sizeof D));
    CK(cuMemAlloc(&d1, N));
    CK(cuMemAlloc(&d2, N));
    CK(cuMemAlloc(&r1, N));
    CK(cuMemAlloc(&r2, N));
    CK(cuMemAlloc(&w1, N));
    CK(cuMemAlloc(&w2, N));
    CK(cuMemcpyHtoD(d1, ha.data(), N));
    CK(cuMemcpyHtoD(d2, hb.data(), N));
    CK(cuMemcpyDtoD(r1, d1, N));
    CK(cuMemcpyDtoD(r2, d2, N));
    CK(cuMemcpyDtoD(w1, d1, N));
    CK(cuMemcpyDtoD(w2, d2, N));
    args[0] = &d1; args[1] = &d2; args[2] = &r1; args[3] = &r2; args[4] = &w1; args[5] = &w2;
    while (!fin) {
        if (distance + 1 >= max_trips) { rc = 2; break; }
        CK(cuMemcpyHtoD(gFin, &one, sizeof one));
        CK(cuLaunchKernel(fn, blocks, 1, 1, threads, 1, 1, 0, nullptr, args, nullptr));
        CK(cuMemcpyDtoD(r1, w1, N));
        CK(cuMemcpyDtoD(r2, w2, N));
        CK(cuMemcpyDtoH(&fin, gFin, sizeof fin));
        ++distance;
    }
    if (rc == 0) *hd_out = distance;
done:
    if (d1) cuMemFree(d1);
    if (d2) cuMemFree(d2);
    if (r1) cuMemFree(r1);
    if (r2) cuMemFree(r2);
    if (w1) cuMemFree(w1);
    if (w2) cuMemFree(w2);
    if (mod) cuModuleUnload(mod);
    if (ctx) {
        CUcontext popped;
        cuCtxPopCurrent(&popped);
        cuDevicePrimaryCtxRelease(dev);
    }
    return rc;
}
