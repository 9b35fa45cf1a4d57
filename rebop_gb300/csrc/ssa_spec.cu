// Host side of the speculative kernel over the packed network descriptor.
#include <cuda_runtime.h>

#include <cstdlib>
#include <cstring>

#include "ssa_spec_body.cuh"

namespace rbg {

template <int MAXR, bool MACRO>
__global__ void __launch_bounds__(kSpecBlock, 1) ssa_spec_kernel(const __grid_constant__ SsaArgs a) {
    spec_body<TableOps<MAXR, MACRO>>(a);
}

// ------------------------------------------------------------------ host side

namespace {

template <int MAXR, bool MACRO>
int spec_launch(const SsaArgs &a, int block, int grid, size_t smem, cudaStream_t st) {
    auto kern = ssa_spec_kernel<MAXR, MACRO>;
    cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return (int)err;
    kern<<<grid, block, smem, st>>>(a);
    return (int)cudaGetLastError();
}

template <int MAXR, bool MACRO>
int spec_occupancy(int block, size_t smem) {
    int n = 0;
    auto kern = ssa_spec_kernel<MAXR, MACRO>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, block, smem);
    return n;
}

template <bool MACRO>
int spec_dispatch(const SsaArgs &a, int block, int grid, size_t smem, cudaStream_t st, int *occ) {
    if (a.R <= 8) return occ ? (*occ = spec_occupancy<8, MACRO>(block, smem), 0)
                             : spec_launch<8, MACRO>(a, block, grid, smem, st);
    return occ ? (*occ = spec_occupancy<16, MACRO>(block, smem), 0) : spec_launch<16, MACRO>(a, block, grid, smem, st);
}

}  // namespace

int ssa_spec_block() { return kSpecBlock; }

bool ssa_spec_supported(const SsaArgs &a, int max_order) {
    return a.R <= 16 && a.S < 65536 && max_order < 32768;
}

size_t ssa_spec_smem(const SsaArgs &a, int slots) {
    return spec_smem_bytes(a, slots);
}

int ssa_spec_slots(const SsaArgs &a, int grid, size_t smem_limit, int block) {
    // every warp owns the same number of slots (at least one per lane)
    const int warps = block / 32;
    if (spec_smem_bytes(a, block) > smem_limit) return 0;
    const int64_t want = (a.n_traj + grid - 1) / (grid > 0 ? grid : 1);
    int slots = block;
    while (slots < want && slots + warps <= kSpecMaxSlots &&
           spec_smem_bytes(a, slots + warps) <= smem_limit)
        slots += warps;
    return slots;
}

int ssa_spec_occupancy(const SsaArgs &a, int block, size_t smem) {
    int occ = 0;
    if (a.macro_mode) spec_dispatch<true>(a, block, 0, smem, nullptr, &occ);
    else spec_dispatch<false>(a, block, 0, smem, nullptr, &occ);
    return occ;
}

int launch_ssa_spec(const SsaArgs &a, int block, int grid, size_t smem, void *stream) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    return a.macro_mode ? spec_dispatch<true>(a, block, grid, smem, st, nullptr)
                        : spec_dispatch<false>(a, block, grid, smem, st, nullptr);
}

}  // namespace rbg
