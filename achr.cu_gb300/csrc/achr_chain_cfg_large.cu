// Chain-kernel instantiations with 256-512 threads per chain.
#include "achr_chain_kernel.cuh"

namespace achr {

cudaError_t launch_chain_cfg_large(int bd, int ept, const ChainArgs &a, cudaStream_t s, int max_ctas, int *per_sm) {
    switch (bd * 100 + ept) {
        case 256 * 100 + 4: return launch_cfg<256, 4>(a, s, max_ctas, per_sm);
        case 256 * 100 + 8: return launch_cfg<256, 8>(a, s, max_ctas, per_sm);
        case 256 * 100 + 16: return launch_cfg<256, 16>(a, s, max_ctas, per_sm);
        case 512 * 100 + 4: return launch_cfg<512, 4>(a, s, max_ctas, per_sm);
        case 512 * 100 + 8: return launch_cfg<512, 8>(a, s, max_ctas, per_sm);
        case 512 * 100 + 16: return launch_cfg<512, 16>(a, s, max_ctas, per_sm);
        case 512 * 100 + 32: return launch_cfg<512, 32>(a, s, max_ctas, per_sm);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_chain_queue_large(int bd, int ept, const ChainQueue &q, cudaStream_t s, int grid, int *per_sm) {
    switch (bd * 100 + ept) {
        case 256 * 100 + 4: return launch_queue_cfg<256, 4>(q, s, grid, per_sm);
        case 256 * 100 + 8: return launch_queue_cfg<256, 8>(q, s, grid, per_sm);
        case 256 * 100 + 16: return launch_queue_cfg<256, 16>(q, s, grid, per_sm);
        case 512 * 100 + 4: return launch_queue_cfg<512, 4>(q, s, grid, per_sm);
        case 512 * 100 + 8: return launch_queue_cfg<512, 8>(q, s, grid, per_sm);
        case 512 * 100 + 16: return launch_queue_cfg<512, 16>(q, s, grid, per_sm);
        case 512 * 100 + 32: return launch_queue_cfg<512, 32>(q, s, grid, per_sm);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace achr
