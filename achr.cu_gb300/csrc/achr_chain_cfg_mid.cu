// Chain-kernel instantiations with 320 and 384 threads per chain (two CTAs per SM).
#include "achr_chain_kernel.cuh"

namespace achr {

cudaError_t launch_chain_cfg_mid(int bd, int ept, const ChainArgs &a, cudaStream_t s, int max_ctas, int *per_sm) {
    switch (bd * 100 + ept) {
        case 320 * 100 + 12: return launch_cfg<320, 12>(a, s, max_ctas, per_sm);
        case 384 * 100 + 10: return launch_cfg<384, 10>(a, s, max_ctas, per_sm);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace achr
