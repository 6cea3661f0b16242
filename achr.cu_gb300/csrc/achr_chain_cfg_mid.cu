// Chain-kernel instantiations between the power-of-two lengths: 320 x 12 and
// 384 x 10 (3840 elements, two CTAs per SM), 512 x 12 (6144) and 512 x 15
// (7680, one CTA per SM), so that models of 4097-7680 reactions do not pad to
// 8192.
#include "achr_chain_kernel.cuh"

namespace achr {

cudaError_t launch_chain_cfg_mid(int bd, int ept, const ChainArgs &a, cudaStream_t s, int max_ctas, int *per_sm) {
    switch (bd * 100 + ept) {
        case 320 * 100 + 12: return launch_cfg<320, 12>(a, s, max_ctas, per_sm);
        case 384 * 100 + 10: return launch_cfg<384, 10>(a, s, max_ctas, per_sm);
        case 512 * 100 + 12: return launch_cfg<512, 12>(a, s, max_ctas, per_sm);
        case 512 * 100 + 15: return launch_cfg<512, 15>(a, s, max_ctas, per_sm);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_chain_queue_mid(int bd, int ept, const ChainQueue &q, cudaStream_t s, int grid, int *per_sm) {
    switch (bd * 100 + ept) {
        case 320 * 100 + 12: return launch_queue_cfg<320, 12>(q, s, grid, per_sm);
        case 384 * 100 + 10: return launch_queue_cfg<384, 10>(q, s, grid, per_sm);
        case 512 * 100 + 12: return launch_queue_cfg<512, 12>(q, s, grid, per_sm);
        case 512 * 100 + 15: return launch_queue_cfg<512, 15>(q, s, grid, per_sm);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace achr
