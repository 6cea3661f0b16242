// Configuration ladder of the chain kernel and its dispatcher.
//
// A configuration is (threads per chain BD, elements per thread EPT); its
// padded length BD * EPT must hold the model's n reactions.  For each padded
// length there is a default configuration (used when threads_per_chain = 0)
// and alternatives that the autotuner may pick.
#include "achr_internal.h"

namespace achr {

cudaError_t launch_chain_cfg_small(int bd, int ept, const ChainArgs &a, cudaStream_t s, int max_ctas, int *per_sm);
cudaError_t launch_chain_cfg_large(int bd, int ept, const ChainArgs &a, cudaStream_t s, int max_ctas, int *per_sm);
cudaError_t launch_chain_cfg_mid(int bd, int ept, const ChainArgs &a, cudaStream_t s, int max_ctas, int *per_sm);
cudaError_t launch_chain_queue_small(int bd, int ept, const ChainQueue &q, cudaStream_t s, int grid, int *per_sm);
cudaError_t launch_chain_queue_mid(int bd, int ept, const ChainQueue &q, cudaStream_t s, int grid, int *per_sm);
cudaError_t launch_chain_queue_large(int bd, int ept, const ChainQueue &q, cudaStream_t s, int grid, int *per_sm);

namespace {

struct Cfg {
    int bd, ept;
    bool dflt;
};

// Ordered by padded length; the default for each length comes first.
// 320 x 12 and 384 x 10 (3840 elements) put 20 or 24 warps on an SM with two
// chains each, against 16 for 256 x 16, at the cost of fewer registers per
// thread; 384 x 10 is the default up to 3840 reactions (2.04e7 against 1.95e7
// chain-steps/s for 256 x 16 on a 2766 x 3742 model).  512 x 12 and 512 x 15
// cut the padding of 4097-7680 reactions (a 7440-reaction model pads to 7680,
// not 8192: 3 % of the FP64 work on padding instead of 10 %).
const Cfg kLadder[] = {
    {32, 4, true},    {64, 4, true},    {32, 8, false},   {128, 4, true},  {64, 8, false},
    {128, 8, true},   {256, 4, false},  {256, 8, true},   {128, 16, false}, {512, 4, false},
    {320, 12, false}, {384, 10, true},  {256, 16, true},  {512, 8, false},  {128, 32, false},
    {512, 12, true},  {512, 15, true},  {512, 16, true},  {512, 32, true},
};

const Cfg *find_cfg(int n, int threads_per_chain) {
    for (const Cfg &c : kLadder) {
        if (c.bd * c.ept < n) continue;
        if (threads_per_chain == 0 ? c.dflt : c.bd == threads_per_chain) return &c;
    }
    return nullptr;
}

}  // namespace

int chain_padded_length(int n, int threads_per_chain) {
    const Cfg *c = find_cfg(n, threads_per_chain);
    return c ? c->bd * c->ept : 0;
}

int chain_block_size(int n, int threads_per_chain) {
    const Cfg *c = find_cfg(n, threads_per_chain);
    return c ? c->bd : 0;
}

int chain_alloc_length(int n) {
    const int np = chain_padded_length(n, 0);
    if (np == 0) return 0;
    return np * 2 > 16384 ? np : np * 2;
}

int chain_candidates(int n, int max_np, int *bds, int cap) {
    const int np0 = chain_padded_length(n, 0);
    int k = 0;
    for (const Cfg &c : kLadder) {
        const int np = c.bd * c.ept;
        if (np < n || np > max_np || np > 2 * np0) continue;
        bool dup = false;
        for (int j = 0; j < k; ++j) dup |= bds[j] == c.bd;
        if (dup || chain_padded_length(n, c.bd) != np) continue;
        if (k < cap) bds[k++] = c.bd;
    }
    return k;
}

size_t chain_smem_bytes(int n, int d, int ldw, int block) {
    (void)ldw;
    (void)d;
    const int np = chain_padded_length(n, block);
    return sizeof(double) * 3 * (size_t)np + 24 * 64 + 2 * 1792 + 128;
}

bool chain_config(int n, int threads_per_chain, int *bd, int *ept) {
    const Cfg *c = find_cfg(n, threads_per_chain);
    if (!c) return false;
    *bd = c->bd;
    *ept = c->ept;
    return true;
}

cudaError_t launch_chain_queue(int bd, int ept, const ChainQueue &q, cudaStream_t stream, int grid, int *per_sm) {
    if (bd <= 128) return launch_chain_queue_small(bd, ept, q, stream, grid, per_sm);
    if (bd == 320 || bd == 384 || (bd == 512 && (ept == 12 || ept == 15)))
        return launch_chain_queue_mid(bd, ept, q, stream, grid, per_sm);
    return launch_chain_queue_large(bd, ept, q, stream, grid, per_sm);
}

cudaError_t launch_chains(const ChainArgs &a, int threads_per_chain, cudaStream_t stream, int max_ctas,
                          int *per_sm) {
    const Cfg *c = find_cfg(a.n, threads_per_chain);
    if (!c || c->bd * c->ept > a.np) return cudaErrorInvalidValue;
    if (a.P <= 0 && !per_sm) return cudaSuccess;
    if (c->bd <= 128) return launch_chain_cfg_small(c->bd, c->ept, a, stream, max_ctas, per_sm);
    if (c->bd == 320 || c->bd == 384 || (c->bd == 512 && (c->ept == 12 || c->ept == 15)))
        return launch_chain_cfg_mid(c->bd, c->ept, a, stream, max_ctas, per_sm);
    return launch_chain_cfg_large(c->bd, c->ept, a, stream, max_ctas, per_sm);
}

}  // namespace achr
