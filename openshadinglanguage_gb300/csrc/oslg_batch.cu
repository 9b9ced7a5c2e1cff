// The persistent batch kernel (batch_kernel in oslg_interp.cuh) for every op
// family: one launch runs many groups from a device work list. One object
// per (launch bound, points per thread) pair, -DOSLG_BATCH_MAXT=256|512 and
// -DOSLG_BATCH_PPT=1|2|4, so the variants build in parallel; each carries
// both heap placements.
#include "oslg_interp.cuh"

#if !defined(OSLG_BATCH_MAXT) || !defined(OSLG_BATCH_PPT)
#error "compile with -DOSLG_BATCH_MAXT=256|512 -DOSLG_BATCH_PPT=1|2|4"
#endif

#define OSLG_NAME_(a, b, c) a##b##_##c
#define OSLG_NAME(a, b, c) OSLG_NAME_(a, b, c)

namespace oslg {

#define OSLG_KERNEL(S) dev::batch_kernel<S, 7, OSLG_BATCH_MAXT, OSLG_BATCH_PPT>

int OSLG_NAME(batch_launch_, OSLG_BATCH_MAXT, OSLG_BATCH_PPT)(bool smem, unsigned grid, unsigned block, size_t shmem,
                                                              void* stream, const dev::BatchArgs& b) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (smem) OSLG_KERNEL(true)<<<grid, block, shmem, s>>>(b);
    else OSLG_KERNEL(false)<<<grid, block, shmem, s>>>(b);
    return (int)cudaGetLastError();
}

int OSLG_NAME(batch_occupancy_, OSLG_BATCH_MAXT, OSLG_BATCH_PPT)(bool smem, int block, size_t shmem, int* per_sm) {
    cudaError_t e = smem ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, OSLG_KERNEL(true), block, shmem)
                         : cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, OSLG_KERNEL(false), block, shmem);
    return (int)e;
}

int OSLG_NAME(batch_smem_limit_, OSLG_BATCH_MAXT, OSLG_BATCH_PPT)(int bytes) {
    cudaError_t e1 = cudaFuncSetAttribute(OSLG_KERNEL(true), cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaError_t e2 = cudaFuncSetAttribute(OSLG_KERNEL(false), cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    return (int)(e1 != cudaSuccess ? e1 : e2);
}

}  // namespace oslg
