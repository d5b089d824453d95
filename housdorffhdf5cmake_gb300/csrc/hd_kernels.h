// hd_kernels.h -- launch wrappers of the device kernels, for the host
// orchestration in hd_api.cu.
#pragma once
#include <cuda_runtime.h>

#include "hd/hd.h"
#include "hd_device.cuh"

namespace hdk {

// Packing and set-up run over `ntiles` tiles (descs[i].tile0 / stile0 =
// first tile of pair i, increasing; per pair tiles_of(pack_words) and
// setup_tiles_of) with `grid` CTAs.  Brick geometry: bxw words x by rows x
// bz planes (both kernel families).
// label: 0 = every nonzero byte is foreground, 1..255 = bytes equal to label.
// sms (packing and set-up): SMs the stream's kernels run on (0: the
// device's); the grid is one resident wave of them.
cudaError_t launch_pack(const PairDesc* d_descs, int npairs, long long ntiles, int grid, int label, int sms,
                        cudaStream_t s);
// zq1 / zq2 (may be null): queues whose first nz slots are zeroed.
cudaError_t launch_setup(const PairDesc* d_descs, int npairs, long long ntiles, int sms, Job* jobs,
                         JobState* states, unsigned long long* queue0, Ctl* ctl, int g0, int bxw, int by, int bz,
                         int mode, cudaStream_t s, unsigned long long* zq1 = nullptr,
                         unsigned long long* zq2 = nullptr, int nz = 0);
// Start values of descs[i].info (counts 0, empty bounding box), i < npairs;
// with slot_descs, also copies descs[i] to slot_descs[descs[i].job0 / 2].
cudaError_t launch_info_init(const PairDesc* d_descs, int npairs, cudaStream_t s, PairDesc* slot_descs = nullptr);
// Serving: list = n (slot, epoch) pairs (device memory); each slot's jobs
// take the epoch and slot_descs[slot].info becomes null.
cudaError_t launch_retire(Job* jobs, PairDesc* slot_descs, const uint32_t* list, int n, cudaStream_t s);
cudaError_t launch_zero_i32(int32_t* p, long long n, cudaStream_t s);
cudaError_t launch_map_init(const PairDesc* d_descs, int32_t* map_a, int32_t* map_b, long long n, int label,
                            cudaStream_t s);

// The persistent dilation kernel for one (element, brick width, brick depth).
// Returns the kernel's host stub for cudaLaunchCooperativeKernel, or nullptr
// if that shape is not compiled in.  Compiled shapes: bxw in {2, 4, 8},
// bz in {4, 8, 16}, both elements.
const void* solve_kernel_ptr(int se, int bxw, int bz);
const void* solve_kernel_ptr_se6(int bxw, int bz);
const void* solve_kernel_ptr_se18(int bxw, int bz);

// The temporally blocked kernel (hd_solve_tb.cuh): `steps` dilation steps per
// grid barrier, bricks of 4 words x (32 - 2 steps) rows x bz planes.
// Compiled: steps 1, 2 with bz 8, 16; steps 3, 4, 5 with bz 8; both elements.
const void* solve_tb_kernel_ptr(int se, int steps, int bz);
const void* solve_tb_kernel_ptr_se6(int steps, int bz);
const void* solve_tb_kernel_ptr_se18(int steps, int bz);

}  // namespace hdk
