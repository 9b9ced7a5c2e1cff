// The persistent batch kernel (batch_kernel in oslg_interp.cuh) for every op
// family: one launch runs many groups from a device work list. Compiled in
// two objects (-DOSLG_BATCH_MAXT=256 / 512) so that the two launch-bound
// variants build in parallel.
#include "oslg_interp.cuh"

#ifndef OSLG_BATCH_MAXT
#error "compile with -DOSLG_BATCH_MAXT=256 or 512"
#endif

#define OSLG_CAT2(a, b) a##b
#define OSLG_CAT(a, b) OSLG_CAT2(a, b)

namespace oslg {

int OSLG_CAT(batch_launch_, OSLG_BATCH_MAXT)(bool smem, unsigned grid, unsigned block, size_t shmem, void* stream,
                                             const dev::BatchArgs& b) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (smem) dev::batch_kernel<true, 7, OSLG_BATCH_MAXT><<<grid, block, shmem, s>>>(b);
    else dev::batch_kernel<false, 7, OSLG_BATCH_MAXT><<<grid, block, shmem, s>>>(b);
    return (int)cudaGetLastError();
}

int OSLG_CAT(batch_occupancy_, OSLG_BATCH_MAXT)(bool smem, int block, size_t shmem, int* per_sm) {
    cudaError_t e = smem ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                               per_sm, dev::batch_kernel<true, 7, OSLG_BATCH_MAXT>, block, shmem)
                         : cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                               per_sm, dev::batch_kernel<false, 7, OSLG_BATCH_MAXT>, block, shmem);
    return (int)e;
}

int OSLG_CAT(batch_smem_limit_, OSLG_BATCH_MAXT)(int bytes) {
    cudaError_t e1 = cudaFuncSetAttribute(dev::batch_kernel<true, 7, OSLG_BATCH_MAXT>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaError_t e2 = cudaFuncSetAttribute(dev::batch_kernel<false, 7, OSLG_BATCH_MAXT>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    return (int)(e1 != cudaSuccess ? e1 : e2);
}

}  // namespace oslg
