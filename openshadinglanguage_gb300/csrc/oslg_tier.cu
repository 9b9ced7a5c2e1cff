// One feature tier of the interpreter: compiled once per tier with
// -DOSLG_TIER=N (N = 0..7), each object carrying interp_kernel<smem, N> for
// both heap placements and the host entry points that launch it. Splitting
// the tiers keeps each kernel's code small (a program only touches the op
// families it uses) and lets the tiers compile in parallel.
#include "oslg_interp.cuh"

#ifndef OSLG_TIER
#error "compile with -DOSLG_TIER=<0..7>"
#endif

#define OSLG_CAT2(a, b) a##b
#define OSLG_CAT(a, b) OSLG_CAT2(a, b)

namespace oslg {

namespace {
int launch_impl(bool smem, unsigned grid, unsigned block, size_t shmem, void* stream, const dev::KArgs& k) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (smem) dev::interp_kernel<true, OSLG_TIER><<<grid, block, shmem, s>>>(k);
    else dev::interp_kernel<false, OSLG_TIER><<<grid, block, shmem, s>>>(k);
    return (int)cudaGetLastError();
}
int occupancy_impl(bool smem, int block, size_t shmem, int* per_sm) {
    cudaError_t e = smem ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, dev::interp_kernel<true, OSLG_TIER>,
                                                                       block, shmem)
                         : cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, dev::interp_kernel<false, OSLG_TIER>,
                                                                       block, shmem);
    return (int)e;
}
int smem_limit_impl(int bytes) {
    cudaError_t e1 = cudaFuncSetAttribute(dev::interp_kernel<true, OSLG_TIER>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaError_t e2 = cudaFuncSetAttribute(dev::interp_kernel<false, OSLG_TIER>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    return (int)(e1 != cudaSuccess ? e1 : e2);
}
}  // namespace

const TierFns& OSLG_CAT(tier_fns_, OSLG_TIER)() {
    static const TierFns f = { launch_impl, occupancy_impl, smem_limit_impl };
    return f;
}

}  // namespace oslg
