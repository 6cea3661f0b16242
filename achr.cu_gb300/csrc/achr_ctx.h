// Sampler context shared by the C-ABI translation units.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <vector>

#include "../../include/achr.h"
#include "achr_internal.h"

namespace achr {

// Device buffer that frees itself.
template <class T>
struct DevBuf {
    T *p = nullptr;
    size_t count = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { reset(); }
    void reset() {
        if (p) cudaFree(p);
        p = nullptr;
        count = 0;
    }
    cudaError_t alloc(size_t n) {
        reset();
        if (n == 0) n = 1;
        cudaError_t e = cudaMalloc(&p, n * sizeof(T));
        if (e == cudaSuccess) count = n;
        else p = nullptr;
        return e;
    }
    cudaError_t upload(const T *h, size_t n) {
        cudaError_t e = alloc(n);
        if (e != cudaSuccess) return e;
        if (n) e = cudaMemcpy(p, h, n * sizeof(T), cudaMemcpyHostToDevice);
        return e;
    }
};

// Operator of the batched reprojection x <- x - S^T B S x, B = (S S^T)^+
// (achr_reproject.cu), built on first use.
struct ReprojState {
    int m = 0, n = 0, kpad = 0, rank = 0, device = 0;
    double lam_max = 0.0, lam_min = 0.0;
    DevBuf<__nv_bfloat16> Bh, Bl;  // m x kpad row-major: (S S^T)^+ split into hi + lo
    DevBuf<int> rp, ci, cp, ri;    // CSR and CSC of S (original row order)
    DevBuf<double> rv, cv;
    DevBuf<__nv_bfloat16> Rh, Rl;  // chunk x kpad: residuals of a chunk of chains, hi + lo
    DevBuf<float> Z;               // m x chunk: B r for the chunk
    int chunk_cap = 0;
    DevBuf<unsigned long long> flags;  // [1] max|Sx| bits after, [2] device error bits, [8 + r * chunks + c] round r, chunk c
};
void reproj_free(ReprojState *r);  // achr_reproject.cu

struct DeferState;
void defer_free(DeferState *d);  // achr_defer.cu

}  // namespace achr

struct achr_ctx;
namespace achr {
// (S S^T)^+ in FP32, rows and columns in the device row order, into ctx->pinv32
// (achr_reproject.cu; builds the batched-reprojection operator on the way).
achr_status build_pinv32(achr_ctx *ctx);
// The batched-reprojection operator of the context, built on first use.
achr_status ensure_reproj(achr_ctx *ctx);
// Segmented sampling with the per-chain reprojections deferred to a batched
// pass (achr_defer.cu): runs the launch described by `a` (a.P chains of a.T
// steps from step 0) on `stream`.
achr_status defer_sample(achr_ctx *ctx, const ChainArgs &a, int threads_per_chain, cudaStream_t stream,
                         bool timed);
// After the stream of a timed defer_sample has completed: device time of its
// chain-kernel launches and of its batched passes, and the chains per sweep.
achr_status defer_times(achr_ctx *ctx, double *chain_ms, double *pass_ms, double *chains_per_sweep);
// Whether sampling with these options takes the deferred path.
bool defer_selected(const achr_ctx *ctx);
}  // namespace achr

struct achr_ctx {
    int n = 0, m = 0, W = 0, d = 0, ldw = 0, np = 0;
    float bound_err = 0.0f;
    // sqrt(sum_i max(lb_i^2, ub_i^2)): every point and centre of a chain lies in
    // the box, so ||w - c|| <= 2 box_norm (inf when a bound is infinite)
    double box_norm = 0.0;
    double dir_norm_max = 0.0;  // largest norm of a hit-and-run direction
    double tuned_rate = 0.0;  // chain-steps per ms on the whole GPU with the tuned configuration (0: not measured)
    int device = 0;
    achr_options opt{};
    std::vector<double> h_lb, h_ub;
    std::vector<int> h_rowptr, h_colidx;  // CSR of S in the model's row order (duplicates summed)
    std::vector<double> h_val;
    achr::DevBuf<double> warmup, c0, A0, val, N, points;
    achr::DevBuf<double2> lbub;
    achr::DevBuf<float2> bnd;
    achr::DevBuf<int> rowptr, colidx;  // device CSR: rows sorted longest first
    achr::DevBuf<int> sell_off, sell_col;  // the same rows as sliced ELL (32-row groups)
    achr::DevBuf<double> sell_val;
    int sell_groups = 0;
    std::vector<int> h_row_order;          // device row q is model row h_row_order[q]
    achr::DevBuf<int> csc_ptr, csc_row;    // CSC of S with device (sorted) row indices
    achr::DevBuf<double> csc_val;
    achr::DevBuf<float> pinv32;            // (S S^T)^+ in FP32, device row order, m x m (empty: not built)
    achr::DevBuf<unsigned long long> counters;
    achr::ReprojState *reproj = nullptr;  // batched reprojection operator, built on first use
    achr::DeferState *defer = nullptr;    // buffers of segmented sampling, built on first use
    double warmup_residual = 0.0;         // max |S w|_inf over the warmup points (as sampled)
    double kappa_sst = 1.0;               // condition number of S S^T on its range (from the null-space set-up)
    long long last_segments = 0;          // chain-kernel launches of the last deferred-reprojection run
    long long last_launches = 0;          // all kernels that run launched
    achr::DevBuf<double> dirs;   // hit-and-run direction pool, n x n_dirs (leading dimension ldw)
    int n_dirs = 0;              // 0: ACHR directions (warmup point minus centre)
    achr::DevBuf<double> zeros;  // np zeros: the (unused) centre accumulator of hit-and-run chains
    // Basis of the directions the polytope spans: the null space of S with the
    // reactions that are fixed across all warmup points also held fixed
    // (n x d_act, column-major); built on first use by the preconditioner.
    achr::DevBuf<double> Nact;
    int d_act = -1, n_frozen = 0;
};
