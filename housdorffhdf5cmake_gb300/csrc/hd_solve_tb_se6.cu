// hd_solve_tb_se6.cu -- instantiations of the temporally blocked dilation
// kernel for the 6-neighbour structuring element.
#include "hd_kernels.h"
#include "hd_solve_tb.cuh"

namespace hdk {

#define HD_TB_CASE(T, BZ) \
    if (steps == T && bz == BZ) return reinterpret_cast<const void*>(&solve_tb_kernel<T, BZ, false>);

const void* solve_tb_kernel_ptr_se6(int steps, int bz) {
    HD_TB_CASE(1, 8)
    HD_TB_CASE(1, 16)
    HD_TB_CASE(2, 8)
    HD_TB_CASE(2, 16)
    HD_TB_CASE(3, 8)
    HD_TB_CASE(4, 8)
    HD_TB_CASE(5, 8)
    return nullptr;
}

}  // namespace hdk
