// Chain-kernel instantiations with 32-128 threads per chain.
#include "achr_chain_kernel.cuh"

namespace achr {

cudaError_t launch_chain_cfg_small(int bd, int ept, const ChainArgs &a, cudaStream_t s, int max_ctas, int *per_sm) {
    switch (bd * 100 + ept) {
        case 32 * 100 + 4: return launch_cfg<32, 4>(a, s, max_ctas, per_sm);
        case 32 * 100 + 8: return launch_cfg<32, 8>(a, s, max_ctas, per_sm);
        case 64 * 100 + 4: return launch_cfg<64, 4>(a, s, max_ctas, per_sm);
        case 64 * 100 + 8: return launch_cfg<64, 8>(a, s, max_ctas, per_sm);
        case 128 * 100 + 4: return launch_cfg<128, 4>(a, s, max_ctas, per_sm);
        case 128 * 100 + 8: return launch_cfg<128, 8>(a, s, max_ctas, per_sm);
        case 128 * 100 + 16: return launch_cfg<128, 16>(a, s, max_ctas, per_sm);
        case 128 * 100 + 32: return launch_cfg<128, 32>(a, s, max_ctas, per_sm);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_chain_queue_small(int bd, int ept, const ChainQueue &q, cudaStream_t s, int grid, int *per_sm) {
    switch (bd * 100 + ept) {
        case 32 * 100 + 4: return launch_queue_cfg<32, 4>(q, s, grid, per_sm);
        case 32 * 100 + 8: return launch_queue_cfg<32, 8>(q, s, grid, per_sm);
        case 64 * 100 + 4: return launch_queue_cfg<64, 4>(q, s, grid, per_sm);
        case 64 * 100 + 8: return launch_queue_cfg<64, 8>(q, s, grid, per_sm);
        case 128 * 100 + 4: return launch_queue_cfg<128, 4>(q, s, grid, per_sm);
        case 128 * 100 + 8: return launch_queue_cfg<128, 8>(q, s, grid, per_sm);
        case 128 * 100 + 16: return launch_queue_cfg<128, 16>(q, s, grid, per_sm);
        case 128 * 100 + 32: return launch_queue_cfg<128, 32>(q, s, grid, per_sm);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace achr
