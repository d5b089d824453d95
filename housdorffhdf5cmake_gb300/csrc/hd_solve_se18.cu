// hd_solve_se18.cu -- instantiations of the persistent dilation kernel for the
// 18-neighbour structuring element (one file per element so the two compile
// in parallel).
#include "hd_kernels.h"
#include "hd_solve.cuh"

namespace hdk {

#define HD_SOLVE_CASE(BXW, BZ) \
    if (bxw == BXW && bz == BZ) return reinterpret_cast<const void*>(&solve_kernel<BXW, BZ, true>);

const void* solve_kernel_ptr_se18(int bxw, int bz) {
    HD_SOLVE_CASE(2, 4)
    HD_SOLVE_CASE(2, 8)
    HD_SOLVE_CASE(2, 16)
    HD_SOLVE_CASE(4, 4)
    HD_SOLVE_CASE(4, 8)
    HD_SOLVE_CASE(4, 16)
    HD_SOLVE_CASE(8, 4)
    HD_SOLVE_CASE(8, 8)
    HD_SOLVE_CASE(8, 16)
    return nullptr;
}

}  // namespace hdk
