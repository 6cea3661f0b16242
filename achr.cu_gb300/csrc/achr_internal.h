// Internal declarations shared by the sampler translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>

namespace achr {

// Counters kept in device memory while a sampling launch runs.
enum CounterSlot {
    CNT_ACCEPTED = 0,
    CNT_REJECTED = 1,
    CNT_CHECKS = 2,
    CNT_REPROJ = 3,
    CNT_STUCK = 4,
    CNT_EXACT = 5,
    CNT_FINAL_PROJ = 6,
    CNT_MAXRES_BITS = 7,   // max ||S v||_inf of emitted points, as the bits of a non-negative double
    CNT_MAXVIOL_BITS = 8,  // max bound violation of emitted points, same encoding
    CNT_ERROR = 9,         // bit flags, ERR_*
    CNT_PASSES = 10,       // deferred reprojection: chain-passes (one chain through one batched pass)
    CNT_GEMMS = 11,        // deferred reprojection: tensor-core GEMMs that ran (not skipped by their gate)
    CNT_SLOTS = 16
};

enum DeviceError : unsigned long long {
    ERR_TMA_TIMEOUT = 1ull,
    ERR_TC_TIMEOUT = 2ull,  // a tensor-core GEMM pipeline wait expired
    ERR_DEFER_DIVERGED = 4ull,  // a deferred reprojection ended with max|S x| > residual_tol
};

// Everything one chain-sampling launch reads (device pointers) and its scalars.
struct ChainArgs {
    int n, m, W, d;
    int np;                     // length the per-element arrays are padded to (>= block size x elements per thread)
    int ldw;                    // leading dimension of the warmup matrix in doubles (even)
    int P, T;
    const double *warmup;       // ldw x W, column j = warmup point j
    const double *c0;           // np: start point and initial centre (zero padding)
    const double *A0;           // np: (W + centre_offset) * c0, the centre accumulator at step 0
    const double2 *lbub;        // np: (lb, ub) in FP64; padding (0, 0)
    const float2 *bnd;          // np: (lb, ub) rounded to FP32, infinite bounds as -+3e38; padding (-1, 1)
    float bound_err;            // max |lb - float(lb)|, |ub - float(ub)| over finite bounds, rounded up
    float dtol_hi, dtol_lo;     // FP32 brackets of d_tol (1 +- 2^-20)
    float utol32, mmt32;        // u_tol and max_min_tol in FP32
    // merged_ab = 1: the FP32 ratio-test brackets are formed in the same pass as
    // d, before the block knows ||d||, with the candidacy threshold bounded by
    // uthr_max >= u_tol ||d|| (from the box or the direction pool); the kernel
    // falls back to a separate bracket pass on any step whose threshold exceeds it.
    int merged_ab;
    float uthr_max;
    const int *row_ptr;         // CSR of S (m + 1)
    const int *col_idx;
    const double *val;
    // Sliced ELL copy of the same rows (groups of 32 rows, slot t of lane l of
    // group g at sell_off[g] + 32 t + l, zero padding); sell_off NULL: use CSR.
    const int *sell_off;
    const int *sell_col;
    const double *sell_val;
    int sell_groups;
    // Residual-form reprojection x <- x - S^T (S S^T)^+ S x: the pseudo-inverse
    // in FP32 (m x m, device row order) and the CSC of S; pinv32 NULL: N (N^T x).
    const float *pinv32;
    const int *csc_ptr;
    const int *csc_row;
    const double *csc_val;
    const double *N;            // n x d column-major null-space basis (ld = n)
    double *out;                // n x P row-major block: out[i * ld_out + p]
    long long ld_out;
    int step0;                  // global index of the first step of this launch (resumed chains)
    const double *x_in;         // NULL: chains start at the centre; else n x P points to resume from (ld_state)
    const double *A_in;         // with x_in: n x P centre accumulators (W + step0 + offset) c
    double *A_out;              // NULL or n x P: centre accumulators after the last step (ld_state)
    long long ld_state;
    unsigned long long seed, chain_offset;
    int check_period, max_attempts, centre_offset, exact_ratio;
    int final_project;          // 1: project+clip emitted points whose residual exceeds feasibility_tol
    int hit_and_run;            // 1: `warmup` holds directions; d = column r, no centre (A stays as loaded)
    double residual_tol, max_min_tol, u_tol, d_tol, feasibility_tol;
    unsigned long long *counters;  // CNT_SLOTS entries
    unsigned long long wait_ns;    // limit of the wait for a staged column (0: the default, 2 s)
    int wait_never;                // 1: that wait is on a barrier nothing completes (tests the timeout)
    // Segmented sampling (achr_defer.cu): the reference's per-chain reprojection
    // is deferred to a batched pass between launches.  A launch runs the steps
    // [step0, step0 + T) of every chain; a check step ends the chain's launch
    // right after x <- x + t u: the kernel writes S x (in FP64 and as BF16
    // hi/lo, rows in the device order) for a chain whose residual exceeds
    // residual_tol, and
    // the point and centre accumulator to chain-major state; the next launch
    // (after the batched reprojection has updated the points) clips the point
    // and adds it to the accumulator before its first step, as the reference
    // does after reprojecting (ACHRCuda.cu:338-350).
    int seg;                       // 1: segmented launch
    int seg_final;                 // 1: this launch holds the run's last step (emit points, diagnostics)
    double *seg_x, *seg_A;         // P x ld_seg chain-major points and centre accumulators
    long long ld_seg;
    unsigned *seg_flags;           // per chain, SEG_* bits
    unsigned long long *seg_any;   // set to 1 when a chain of this launch needs a reprojection
    unsigned short *seg_Rh, *seg_Rl;  // P x kpad BF16 bits: hi and lo parts of S x (device row order)
    int kpad;
    double *seg_rd;                // P x ld_r: S x at the check (FP64), device row order
    long long ld_r;
    const float *seg_dxh, *seg_dxl;  // P x ld_seg: the passes' correction (double-float), subtracted next launch
};

// Work queue of a persistent multi-model launch (achr_chain_queue_kernel):
// items (model, first chain, end chain) taken in order by the CTAs.
struct ChainQueue {
    const ChainArgs *args;        // one per model (device)
    const int4 *items;            // (model, p0, p1, 0)
    int n_items;
    int *next;                    // the next item to take (zero before the launch)
    int *chains_done;             // per model, zero before the launch
    unsigned long long *done_ns;  // per model: globaltimer when its last chain finished
    size_t extra_smem;            // shared memory for (S S^T)^+ r (m floats) of the residual-form models
    unsigned long long *cta_ns;   // NULL or one per CTA: globaltimer when the CTA found the queue empty
};

// Per-chain state bits of segmented sampling.
enum SegFlag : unsigned {
    SEG_STARTED = 1u,   // the chain-major state holds the chain's point and accumulator
    SEG_ACCEPTED = 2u,  // at least one step accepted
    SEG_STUCK = 4u,     // stopped after max_attempts rejections
    SEG_PENDING = 8u,   // the last launch ended after a check step's update: clip and add to the centre next
    SEG_REPROJ = 16u,   // that check found max|S x| > residual_tol: the batched passes reproject the point
    SEG_CORR = 32u,     // the next launch subtracts the passes' accumulated correction from the point
};

// FP32 rounding of a double toward +inf / -inf (host side).
inline float f32_up(double v) {
    float f = (float)v;
    if ((double)f < v) f = nextafterf(f, __builtin_huge_valf());
    return f;
}
inline float f32_down(double v) {
    float f = (float)v;
    if ((double)f > v) f = nextafterf(f, -__builtin_huge_valf());
    return f;
}

// Upper bound of the FP32 candidacy threshold u_tol ||d|| (times its margin)
// for the ratio-test brackets formed before the block norm is known, from a
// bound on ||d||; without a finite bound the brackets keep their own pass.
inline void set_merged_bound(ChainArgs &a, double u_tol, double dnorm_max) {
    const double t = u_tol * dnorm_max * 1.01;
    if (t == t && t > 0.0 && t < 1e30) {
        a.uthr_max = f32_up(t);
        a.merged_ab = 1;
    } else {
        a.uthr_max = 0.0f;
        a.merged_ab = 0;
    }
}

// Launch the persistent chain kernel; threads_per_chain = 0 picks the default
// configuration for n.  max_ctas > 0 caps the grid; per_sm (if non-NULL)
// receives the resident CTAs per SM of the configuration.  a.np is the length
// the per-reaction arrays were padded to (>= the configuration's BD * EPT).
cudaError_t launch_chains(const ChainArgs &a, int threads_per_chain, cudaStream_t stream, int max_ctas = 0,
                          int *per_sm = nullptr);

// Configuration ladder: threads per chain and padded element count for n
// reactions (threads_per_chain = 0: default); 0 if no configuration fits.
int chain_block_size(int n, int threads_per_chain);
// Configuration (threads, elements per thread) the model of n reactions runs with.
bool chain_config(int n, int threads_per_chain, int *bd, int *ept);
// Persistent work-queue launch of the configuration (bd, ept); see ChainQueue.
cudaError_t launch_chain_queue(int bd, int ept, const ChainQueue &q, cudaStream_t stream, int grid, int *per_sm);
int chain_padded_length(int n, int threads_per_chain);
// Length to pad per-reaction arrays to: twice the default padded length (so
// every autotuning candidate fits), at most 16384.
int chain_alloc_length(int n);
// Threads-per-chain values worth timing for n (padded length within max_np).
int chain_candidates(int n, int max_np, int *bds, int cap);
size_t chain_smem_bytes(int n, int d, int ldw, int block);

// Tensor-core GEMM (achr_tc_gemm.cu): C (M x N, FP32, row-major, ldc) =
// A0 B0^T (nsplit 1) or A0 B0^T + A0 B1^T + A1 B0^T (nsplit 3); operands BF16
// row-major with K contiguous, K a multiple of 64, lda/ldb multiples of 8.
struct TcGemm {
    int M, N, K, nsplit;
    const void *A0, *A1;
    long long lda;
    const void *B0, *B1;
    long long ldb;
    float *C;
    long long ldc;
    const unsigned long long *gate = nullptr;  // device word: the launch does nothing when *gate <= gate_max
    unsigned long long gate_max = 0;
};
const char *tc_gemm_check(const TcGemm &g);  // nullptr when the shapes are supported
cudaError_t launch_tc_gemm(const TcGemm &g, unsigned long long *err, cudaStream_t stream);
double tc_gemm_flops(const TcGemm &g);

}  // namespace achr
