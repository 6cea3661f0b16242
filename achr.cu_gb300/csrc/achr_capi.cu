// C ABI of the sampler: context set-up (model upload, null space, centre) and
// sampling launches.  Replaces the set-up half of the reference's main()
// (ACHRcu/ACHRCuda.cu:642-729) and its per-file launch (:736-743).
#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <cusolverDn.h>

#include <algorithm>
#include <cmath>
#include <atomic>
#include <map>
#include <mutex>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/achr.h"
#include "achr_ctx.h"
#include "achr_queue_plan.h"

using achr::ChainArgs;
using achr::DevBuf;

namespace {

thread_local std::string g_last_error;

achr_status fail(achr_status st, const std::string &msg) {
    g_last_error = msg;
    return st;
}

achr_status cuda_fail(cudaError_t e, const char *what) {
    return fail(ACHR_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define ACHR_CUDA_TRY(expr)                                     \
    do {                                                        \
        cudaError_t e_ = (expr);                                \
        if (e_ != cudaSuccess) return cuda_fail(e_, #expr);     \
    } while (0)

// FP32 image of a bound for the chain kernel's brackets: round to nearest, an
// infinite bound becomes a finite stand-in (keeps the bracket arithmetic free
// of inf - inf); err is the conversion error rounded up (0 for infinities).
void f32_bound(double v, float &f, float &err) {
    if (std::isinf(v)) {
        f = v > 0 ? 3.0e38f : -3.0e38f;
        err = 0.0f;
        return;
    }
    f = (float)v;
    const double e = std::fabs(v - (double)f);
    float ef = (float)e;
    if ((double)ef < e) ef = std::nextafter(ef, INFINITY);
    err = ef;
}

using achr::f32_down;
using achr::f32_up;

// Writes the global nanosecond timer (used to time each model's branch of a
// batched graph).
__global__ void stamp_kernel(unsigned long long *slot) {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    *slot = t;
}

__global__ void centre_kernel(int n, int W, int ldw, const double *__restrict__ warmup, int centre_offset,
                              double *__restrict__ c0, double *__restrict__ A0) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double acc = 0.0;
    for (int j = 0; j < W; ++j) acc += warmup[(size_t)j * (size_t)ldw + i];
    // c = (1/W) * sum_j w_j (reference createCenterPt, ACHRCuda.cu:414-434)
    const double c = (1.0 / (double)W) * acc;
    c0[i] = c;
    A0[i] = (double)(W + centre_offset) * c;
}

// Largest |S w|_inf over the warmup points (one block per point, a thread per
// row of the device CSR), as the bits of a non-negative double, maxed into *out_bits.
__global__ void warmup_residual_kernel(int m, int ldw, const double *__restrict__ warmup, const int *__restrict__ rp,
                                       const int *__restrict__ ci, const double *__restrict__ rv,
                                       unsigned long long *out_bits) {
    __shared__ unsigned long long part[32];
    const double *w = warmup + (size_t)blockIdx.x * (size_t)ldw;
    unsigned long long mx = 0;
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        double acc = 0.0;
        for (int q = rp[i]; q < rp[i + 1]; ++q) acc = fma(rv[q], w[ci[q]], acc);
        mx = max(mx, (unsigned long long)__double_as_longlong(acc) & 0x7FFFFFFFFFFFFFFFull);
    }
    for (int o = 16; o; o >>= 1) mx = max(mx, (unsigned long long)__shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < (int)(blockDim.x >> 5); ++k) mx = max(mx, part[k]);
        atomicMax(out_bits, mx);
    }
}

// Largest column norm of an n x K column-major matrix (one block per column),
// as the bits of a non-negative double, maxed into *out_bits.
__global__ void col_norm_max_kernel(int n, long long ld, const double *__restrict__ M,
                                    unsigned long long *out_bits) {
    __shared__ double part[32];
    const double *col = M + (size_t)blockIdx.x * (size_t)ld;
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s = fma(col[i], col[i], s);
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[w];
        atomicMax(out_bits, (unsigned long long)__double_as_longlong(sqrt(t)));
    }
}

}  // namespace

extern "C" {

void achr_default_options(achr_options *opt) {
    if (!opt) return;
    std::memset(opt, 0, sizeof(*opt));
    opt->mode = ACHR_MODE_REFERENCE;
    opt->null_space = ACHR_NULL_SVD_STS;
    opt->check_period = 10;
    opt->max_attempts = 100000;
    opt->centre_offset = 0;
    opt->exact_ratio = 0;
    opt->threads_per_chain = 0;
    opt->residual_tol = 1e-9;
    opt->max_min_tol = 1e-9;
    opt->u_tol = 1e-9;
    opt->d_tol = 1e-14;
    opt->feasibility_tol = 1e-8;
}

const char *achr_last_error(void) { return g_last_error.c_str(); }

void achr_io_set_error(const char *msg) { g_last_error = msg ? msg : ""; }

int32_t achr_version(void) { return 100; }

}  // extern "C"

namespace {

achr_status validate_options(const achr_options &o) {
    if (o.mode != ACHR_MODE_REFERENCE && o.mode != ACHR_MODE_FEASIBLE) return fail(ACHR_ERR_INVALID, "unknown mode");
    if (o.null_space != ACHR_NULL_SVD_STS && o.null_space != ACHR_NULL_SVD_S && o.null_space != ACHR_NULL_FIXED)
        return fail(ACHR_ERR_INVALID, "unknown null_space method");
    if (o.check_period < 0) return fail(ACHR_ERR_INVALID, "check_period must be >= 0 (0: no in-loop checks)");
    if (o.max_attempts <= 0) return fail(ACHR_ERR_INVALID, "max_attempts must be positive");
    if (o.reproject_form < 0 || o.reproject_form > 3) return fail(ACHR_ERR_INVALID, "reproject_form must be 0..3");
    if (o.reprojection_passes < 0 || o.reprojection_passes > 8)
        return fail(ACHR_ERR_INVALID, "reprojection_passes must be 0..8");
    if (o.centre_offset != 0 && o.centre_offset != 1) return fail(ACHR_ERR_INVALID, "centre_offset must be 0 or 1");
    if (o.bracket_pass != 0 && o.bracket_pass != 1) return fail(ACHR_ERR_INVALID, "bracket_pass must be 0 or 1");
    if (o.threads_per_chain != 0 && o.threads_per_chain != 32 && o.threads_per_chain != 64 &&
        o.threads_per_chain != 128 && o.threads_per_chain != 256 && o.threads_per_chain != 320 &&
        o.threads_per_chain != 384 && o.threads_per_chain != 512)
        return fail(ACHR_ERR_INVALID, "threads_per_chain must be 0, 32, 64, 128, 256, 320, 384 or 512");
    if (!(o.residual_tol >= 0) || !(o.max_min_tol >= 0) || !(o.u_tol >= 0) || !(o.d_tol >= 0) ||
        !(o.feasibility_tol >= 0))
        return fail(ACHR_ERR_INVALID, "tolerances must be non-negative");
    return ACHR_OK;
}

// Null space of S by the reference's rule: eigen-decomposition of S^T S
// (symmetric, so its SVD and eigen-decomposition share the spectrum), cutoff
// n * sigma_0 * 2.2204e-16; the basis is every eigenvector whose eigenvalue
// magnitude is below the cutoff (ACHRCuda.cu:459-489).  If no value falls
// below the cutoff the reference keeps istart = 0 and uses all n columns.
achr_status null_space_sts(int n, int m, const std::vector<double> &denseS, std::vector<double> &N, int &d,
                           double &kappa) {
    DevBuf<double> dS, dStS, dW, work;
    DevBuf<int> info;
    ACHR_CUDA_TRY(dS.upload(denseS.data(), (size_t)m * n));
    ACHR_CUDA_TRY(dStS.alloc((size_t)n * n));
    ACHR_CUDA_TRY(dW.alloc(n));
    ACHR_CUDA_TRY(info.alloc(1));
    cublasHandle_t cb = nullptr;
    if (cublasCreate(&cb) != CUBLAS_STATUS_SUCCESS) return fail(ACHR_ERR_CUDA, "cublasCreate failed");
    const double one = 1.0, zero = 0.0;
    cublasStatus_t bs = cublasDgemm(cb, CUBLAS_OP_T, CUBLAS_OP_N, n, n, m, &one, dS.p, m, dS.p, m, &zero, dStS.p, n);
    cublasDestroy(cb);
    if (bs != CUBLAS_STATUS_SUCCESS) return fail(ACHR_ERR_CUDA, "cublasDgemm (S^T S) failed");
    cusolverDnHandle_t sh = nullptr;
    if (cusolverDnCreate(&sh) != CUSOLVER_STATUS_SUCCESS) return fail(ACHR_ERR_CUDA, "cusolverDnCreate failed");
    int lwork = 0;
    cusolverStatus_t ss =
        cusolverDnDsyevd_bufferSize(sh, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, dStS.p, n, dW.p, &lwork);
    if (ss == CUSOLVER_STATUS_SUCCESS) {
        cudaError_t e = work.alloc((size_t)(lwork > 0 ? lwork : 1));
        if (e != cudaSuccess) {
            cusolverDnDestroy(sh);
            return cuda_fail(e, "cudaMalloc(syevd work)");
        }
        ss = cusolverDnDsyevd(sh, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, dStS.p, n, dW.p, work.p, lwork,
                              info.p);
    }
    cusolverDnDestroy(sh);
    if (ss != CUSOLVER_STATUS_SUCCESS) return fail(ACHR_ERR_NUMERIC, "cusolverDnDsyevd failed");
    int h_info = 0;
    std::vector<double> lam(n), V((size_t)n * n);
    ACHR_CUDA_TRY(cudaMemcpy(&h_info, info.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (h_info != 0) return fail(ACHR_ERR_NUMERIC, "syevd did not converge (info=" + std::to_string(h_info) + ")");
    ACHR_CUDA_TRY(cudaMemcpy(lam.data(), dW.p, sizeof(double) * n, cudaMemcpyDeviceToHost));
    ACHR_CUDA_TRY(cudaMemcpy(V.data(), dStS.p, sizeof(double) * (size_t)n * n, cudaMemcpyDeviceToHost));
    double smax = 0.0;
    for (int i = 0; i < n; ++i) smax = std::max(smax, std::fabs(lam[i]));
    const double tol = (double)n * smax * 2.2204e-16;
    std::vector<int> cols;
    double lkept = 0.0;  // smallest eigenvalue above the cutoff
    for (int i = 0; i < n; ++i) {
        if (std::fabs(lam[i]) < tol) cols.push_back(i);
        else if (lkept == 0.0 || std::fabs(lam[i]) < lkept) lkept = std::fabs(lam[i]);
    }
    // condition number of S S^T on its range (the same non-zero spectrum as S^T S)
    kappa = lkept > 0.0 ? smax / lkept : 1.0;
    if (cols.empty())
        for (int i = 0; i < n; ++i) cols.push_back(i);
    d = (int)cols.size();
    N.assign((size_t)n * d, 0.0);
    for (int j = 0; j < d; ++j)
        std::memcpy(N.data() + (size_t)j * n, V.data() + (size_t)cols[j] * n, sizeof(double) * n);
    return ACHR_OK;
}

// Null space from the SVD of S^T (n x m, n >= m as cuSOLVER's gesvd needs):
// left singular vectors beyond the numerical rank span null(S).  Cutoff
// max(m,n) * sigma_0 * 2.2204e-16 on the singular values of S.
achr_status null_space_svd_s(int n, int m, const std::vector<double> &denseS, std::vector<double> &N, int &d,
                             double &kappa) {
    if (n < m) return fail(ACHR_ERR_UNSUPPORTED, "ACHR_NULL_SVD_S needs n_rxns >= n_mets");
    std::vector<double> St((size_t)n * m);
    for (int i = 0; i < m; ++i)
        for (int j = 0; j < n; ++j) St[(size_t)i * n + j] = denseS[(size_t)j * m + i];
    DevBuf<double> dA, dSig, dU, dVT, work, rwork;
    DevBuf<int> info;
    ACHR_CUDA_TRY(dA.upload(St.data(), St.size()));
    ACHR_CUDA_TRY(dSig.alloc(m));
    ACHR_CUDA_TRY(dU.alloc((size_t)n * n));
    ACHR_CUDA_TRY(dVT.alloc((size_t)m * m));
    ACHR_CUDA_TRY(info.alloc(1));
    ACHR_CUDA_TRY(rwork.alloc(m));
    cusolverDnHandle_t sh = nullptr;
    if (cusolverDnCreate(&sh) != CUSOLVER_STATUS_SUCCESS) return fail(ACHR_ERR_CUDA, "cusolverDnCreate failed");
    int lwork = 0;
    cusolverStatus_t ss = cusolverDnDgesvd_bufferSize(sh, n, m, &lwork);
    if (ss == CUSOLVER_STATUS_SUCCESS) {
        cudaError_t e = work.alloc((size_t)(lwork > 0 ? lwork : 1));
        if (e != cudaSuccess) {
            cusolverDnDestroy(sh);
            return cuda_fail(e, "cudaMalloc(gesvd work)");
        }
        signed char jobu = 'A', jobvt = 'N';
        ss = cusolverDnDgesvd(sh, jobu, jobvt, n, m, dA.p, n, dSig.p, dU.p, n, dVT.p, m, work.p, lwork, rwork.p,
                              info.p);
    }
    cusolverDnDestroy(sh);
    if (ss != CUSOLVER_STATUS_SUCCESS) return fail(ACHR_ERR_NUMERIC, "cusolverDnDgesvd failed");
    int h_info = 0;
    ACHR_CUDA_TRY(cudaMemcpy(&h_info, info.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (h_info != 0) return fail(ACHR_ERR_NUMERIC, "gesvd did not converge (info=" + std::to_string(h_info) + ")");
    std::vector<double> sig(m), U((size_t)n * n);
    ACHR_CUDA_TRY(cudaMemcpy(sig.data(), dSig.p, sizeof(double) * m, cudaMemcpyDeviceToHost));
    ACHR_CUDA_TRY(cudaMemcpy(U.data(), dU.p, sizeof(double) * U.size(), cudaMemcpyDeviceToHost));
    const double tol = (double)std::max(n, m) * (m > 0 ? sig[0] : 0.0) * 2.2204e-16;
    int rank = 0;
    for (int i = 0; i < m; ++i)
        if (sig[i] >= tol && sig[i] > 0.0) ++rank;
    kappa = rank > 0 ? (sig[0] / sig[(size_t)rank - 1]) * (sig[0] / sig[(size_t)rank - 1]) : 1.0;
    d = n - rank;
    N.assign((size_t)n * (d > 0 ? d : 0), 0.0);
    for (int j = 0; j < d; ++j)
        std::memcpy(N.data() + (size_t)j * n, U.data() + (size_t)(rank + j) * n, sizeof(double) * n);
    return ACHR_OK;
}

achr_status upload_null_space(achr_ctx *ctx, const double *N, int d) {
    ctx->d = d;
    ACHR_CUDA_TRY(ctx->N.upload(N, (size_t)ctx->n * (size_t)(d > 0 ? d : 0)));
    return ACHR_OK;
}

// FEASIBLE mode: project the warmup points onto the span of N in FP64,
// W <- N (N^T W) (cuBLAS), then recompute the centre.  %f-rounded warmup CSVs
// carry |S w| ~ 1e-6; after this the sampling loop starts on null(S).
achr_status prepare_warmup_and_centre(achr_ctx *ctx) {
    const int n = ctx->n, W = ctx->W, d = ctx->d;
    if (ctx->opt.mode == ACHR_MODE_FEASIBLE && d > 0) {
        cublasHandle_t cb = nullptr;
        if (cublasCreate(&cb) != CUBLAS_STATUS_SUCCESS) return fail(ACHR_ERR_CUDA, "cublasCreate failed");
        const double one = 1.0, zero = 0.0;
        const int chunk = 4096;  // warmup columns per GEMM pair (bounds the d x chunk temporary)
        DevBuf<double> Y;
        cudaError_t e = Y.alloc((size_t)d * (size_t)std::min(chunk, W));
        if (e != cudaSuccess) {
            cublasDestroy(cb);
            return cuda_fail(e, "cudaMalloc(projection temporary)");
        }
        for (int j0 = 0; j0 < W; j0 += chunk) {
            const int nc = std::min(chunk, W - j0);
            double *Wj = ctx->warmup.p + (size_t)j0 * ctx->ldw;
            cublasStatus_t bs = cublasDgemm(cb, CUBLAS_OP_T, CUBLAS_OP_N, d, nc, n, &one, ctx->N.p, n, Wj, ctx->ldw,
                                            &zero, Y.p, d);
            if (bs == CUBLAS_STATUS_SUCCESS)
                bs = cublasDgemm(cb, CUBLAS_OP_N, CUBLAS_OP_N, n, nc, d, &one, ctx->N.p, n, Y.p, d, &zero, Wj,
                                 ctx->ldw);
            if (bs != CUBLAS_STATUS_SUCCESS) {
                cublasDestroy(cb);
                return fail(ACHR_ERR_CUDA, "cublasDgemm (warmup projection) failed");
            }
        }
        cublasDestroy(cb);
    }
    ACHR_CUDA_TRY(cudaMemset(ctx->c0.p, 0, sizeof(double) * ctx->np));
    ACHR_CUDA_TRY(cudaMemset(ctx->A0.p, 0, sizeof(double) * ctx->np));
    centre_kernel<<<(n + 127) / 128, 128>>>(n, W, ctx->ldw, ctx->warmup.p, ctx->opt.centre_offset, ctx->c0.p,
                                            ctx->A0.p);
    ACHR_CUDA_TRY(cudaGetLastError());
    // The residual the warmup points carry as they will be sampled (a %f CSV
    // leaves about 1e-6; it decides where reprojections run, see defer_selected).
    ctx->warmup_residual = 0.0;
    if (ctx->m > 0) {
        DevBuf<unsigned long long> rb;
        ACHR_CUDA_TRY(rb.alloc(1));
        ACHR_CUDA_TRY(cudaMemset(rb.p, 0, sizeof(unsigned long long)));
        warmup_residual_kernel<<<W, 128>>>(ctx->m, ctx->ldw, ctx->warmup.p, ctx->rowptr.p, ctx->colidx.p, ctx->val.p,
                                           rb.p);
        ACHR_CUDA_TRY(cudaGetLastError());
        unsigned long long bits = 0;
        ACHR_CUDA_TRY(cudaMemcpy(&bits, rb.p, sizeof bits, cudaMemcpyDeviceToHost));
        std::memcpy(&ctx->warmup_residual, &bits, sizeof(double));
    }
    ACHR_CUDA_TRY(cudaDeviceSynchronize());
    return ACHR_OK;
}

ChainArgs chain_args(const achr_ctx *ctx, uint64_t seed, uint64_t chain_offset, int32_t n_points, int32_t n_steps,
                     double *d_points_out, int64_t ld_out);

achr_status read_counters(achr_ctx *ctx, achr_stats *stats, float ms);

// The deferred-reprojection part of the statistics (after the stream has completed).
achr_status deferred_stats(achr_ctx *ctx, bool deferred, achr_stats *stats) {
    stats->chain_ms = stats->kernel_ms;
    stats->kernel_launches = 1;
    if (!deferred) return ACHR_OK;
    stats->segments = ctx->last_segments;
    stats->kernel_launches = ctx->last_launches;
    double cm = 0.0, pm = 0.0, per_sweep = 0.0;
    achr_status st = achr::defer_times(ctx, &cm, &pm, &per_sweep);
    if (st != ACHR_OK) return st;
    stats->chain_ms = cm;
    stats->reprojection_ms = pm;
    const int kpad = (ctx->m + 63) / 64 * 64;
    stats->reprojection_flops = (double)stats->reprojection_gemms * 2.0 * per_sweep * ctx->m * kpad * 3.0;
    return ACHR_OK;
}

achr_status read_counters(achr_ctx *ctx, achr_stats *stats, float ms) {
    unsigned long long c[achr::CNT_SLOTS];
    ACHR_CUDA_TRY(cudaMemcpy(c, ctx->counters.p, sizeof(c), cudaMemcpyDeviceToHost));
    if (c[achr::CNT_ERROR] & achr::ERR_TMA_TIMEOUT)
        return fail(ACHR_ERR_TIMEOUT, "a warmup-column copy did not complete within its wait limit");
    if (c[achr::CNT_ERROR] & achr::ERR_TC_TIMEOUT)
        return fail(ACHR_ERR_TIMEOUT, "a tensor-core pipeline wait of the batched reprojection expired");
    if (c[achr::CNT_ERROR] & achr::ERR_DEFER_DIVERGED)
        return fail(ACHR_ERR_NUMERIC, "a deferred reprojection left max|S x| above residual_tol after its last pass");
    if (stats) {
        stats->accepted = (int64_t)c[achr::CNT_ACCEPTED];
        stats->rejected = (int64_t)c[achr::CNT_REJECTED];
        stats->checks = (int64_t)c[achr::CNT_CHECKS];
        stats->reprojections = (int64_t)c[achr::CNT_REPROJ];
        stats->stuck_chains = (int64_t)c[achr::CNT_STUCK];
        stats->exact_evals = (int64_t)c[achr::CNT_EXACT];
        stats->final_projections = (int64_t)c[achr::CNT_FINAL_PROJ];
        double r, v;
        std::memcpy(&r, &c[achr::CNT_MAXRES_BITS], sizeof(double));
        std::memcpy(&v, &c[achr::CNT_MAXVIOL_BITS], sizeof(double));
        stats->max_residual = r;
        stats->max_bound_violation = v;
        stats->kernel_ms = ms;
        stats->segments = 0;
        stats->reprojection_passes = (int64_t)c[achr::CNT_PASSES];
        stats->reprojection_gemms = (int64_t)c[achr::CNT_GEMMS];
        stats->chain_ms = ms;
        stats->reprojection_ms = 0.0;
        stats->reprojection_flops = 0.0;
        stats->kernel_launches = 1;
    }
    return ACHR_OK;
}

}  // namespace

extern "C" {

achr_status achr_create(const achr_model *model, const double *warmup, int32_t n_warmup, const achr_options *opt_in,
                        achr_ctx **out) {
    if (!out) return fail(ACHR_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (!model || !warmup) return fail(ACHR_ERR_INVALID, "model or warmup is NULL");
    achr_options opt;
    if (opt_in) opt = *opt_in;
    else achr_default_options(&opt);
    achr_status st = validate_options(opt);
    if (st != ACHR_OK) return st;
    const int n = model->n_rxns, m = model->n_mets;
    if (n <= 0 || m < 0) return fail(ACHR_ERR_INVALID, "model needs n_rxns > 0 and n_mets >= 0");
    if (n > 16384) return fail(ACHR_ERR_UNSUPPORTED, "n_rxns > 16384 is not supported by the chain kernel");
    if (n_warmup <= 0) return fail(ACHR_ERR_INVALID, "need at least one warmup point");
    if (model->nnz < 0 || (model->nnz > 0 && (!model->row || !model->col || !model->val)))
        return fail(ACHR_ERR_INVALID, "bad COO arrays");
    if (!model->lb || !model->ub) return fail(ACHR_ERR_INVALID, "bounds are NULL");

    achr_ctx *ctx = new (std::nothrow) achr_ctx();
    if (!ctx) return fail(ACHR_ERR_NOMEM, "context allocation failed");
    struct Guard {
        achr_ctx *&c;
        ~Guard() { delete c; }
    };
    achr_ctx *owned = ctx;
    Guard guard{owned};

    ctx->n = n;
    ctx->m = m;
    ctx->W = n_warmup;
    ctx->opt = opt;
    cudaGetDevice(&ctx->device);
    ctx->h_lb.assign(model->lb, model->lb + n);
    ctx->h_ub.assign(model->ub, model->ub + n);

    // COO -> CSR, duplicates summed, explicit zeros dropped (the reference's
    // dense-scan COO keeps only non-zeros, ACHRCuda.cu:647-655).
    std::vector<int64_t> order((size_t)model->nnz);
    for (int64_t k = 0; k < model->nnz; ++k) {
        const int r = model->row[k], c = model->col[k];
        if (r < 0 || r >= m || c < 0 || c >= n) return fail(ACHR_ERR_INVALID, "COO index out of range");
        order[(size_t)k] = k;
    }
    std::sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
        if (model->row[a] != model->row[b]) return model->row[a] < model->row[b];
        return model->col[a] < model->col[b];
    });
    ctx->h_rowptr.assign((size_t)m + 1, 0);
    for (size_t q = 0; q < order.size();) {
        const int r = model->row[order[q]], c = model->col[order[q]];
        double v = 0.0;
        while (q < order.size() && model->row[order[q]] == r && model->col[order[q]] == c) v += model->val[order[q++]];
        if (v != 0.0) {
            ctx->h_colidx.push_back(c);
            ctx->h_val.push_back(v);
            ctx->h_rowptr[(size_t)r + 1]++;
        }
    }
    for (int r = 0; r < m; ++r) ctx->h_rowptr[(size_t)r + 1] += ctx->h_rowptr[(size_t)r];

    // Per-reaction arrays are padded to the kernel's block size x elements per
    // thread; padding entries are fixed at 0 (lb = ub = 0) and never move.
    const int np_cfg = achr::chain_padded_length(n, opt.threads_per_chain);
    if (np_cfg == 0) return fail(ACHR_ERR_UNSUPPORTED, "no chain-kernel configuration for n_rxns with this threads_per_chain");
    const int np = std::max(np_cfg, achr::chain_alloc_length(n));  // room for every autotuning candidate
    ctx->np = np;
    // Padding reactions have lb = ub = 0 in FP64 and the FP32 box (-1, 1), so
    // their (zero) coordinate is never a candidate and never needs a clip.
    std::vector<float2> b32((size_t)np, make_float2(-1.0f, 1.0f));
    std::vector<double2> lu((size_t)np, make_double2(0.0, 0.0));
    float berr = 0.0f;
    for (int i = 0; i < n; ++i) {
        if (!(model->lb[i] <= model->ub[i])) return fail(ACHR_ERR_INVALID, "lb > ub or NaN bound at reaction " + std::to_string(i));
        float lf, le, uf, ue;
        f32_bound(model->lb[i], lf, le);
        f32_bound(model->ub[i], uf, ue);
        b32[i] = make_float2(lf, uf);
        berr = std::max(berr, std::max(le, ue));
        lu[i] = make_double2(model->lb[i], model->ub[i]);
    }
    ctx->bound_err = berr;
    {
        double bsq = 0.0;
        for (int i = 0; i < n; ++i) bsq += std::max(model->lb[i] * model->lb[i], model->ub[i] * model->ub[i]);
        ctx->box_norm = std::sqrt(bsq);
    }
    for (int64_t k = 0; k < (int64_t)n * n_warmup; ++k)
        if (!std::isfinite(warmup[k])) return fail(ACHR_ERR_INVALID, "warmup points must be finite");

    ACHR_CUDA_TRY(ctx->lbub.upload(lu.data(), np));
    ACHR_CUDA_TRY(ctx->bnd.upload(b32.data(), np));
    {
        // The device copy of S lists rows longest first, so the 32 rows a warp
        // sums together in the residual check have similar lengths; max|S x|
        // does not depend on the row order.
        std::vector<int> order_r((size_t)m);
        for (int r = 0; r < m; ++r) order_r[(size_t)r] = r;
        std::stable_sort(order_r.begin(), order_r.end(), [&](int a, int b) {
            return ctx->h_rowptr[(size_t)a + 1] - ctx->h_rowptr[a] > ctx->h_rowptr[(size_t)b + 1] - ctx->h_rowptr[b];
        });
        std::vector<int> rp((size_t)m + 1, 0), ci;
        std::vector<double> vv;
        ci.reserve(ctx->h_colidx.size());
        vv.reserve(ctx->h_val.size());
        for (int q = 0; q < m; ++q) {
            const int r = order_r[(size_t)q];
            for (int t = ctx->h_rowptr[r]; t < ctx->h_rowptr[(size_t)r + 1]; ++t) {
                ci.push_back(ctx->h_colidx[t]);
                vv.push_back(ctx->h_val[t]);
            }
            rp[(size_t)q + 1] = (int)ci.size();
        }
        ACHR_CUDA_TRY(ctx->rowptr.upload(rp.data(), rp.size()));
        ACHR_CUDA_TRY(ctx->colidx.upload(ci.data(), ci.size()));
        ACHR_CUDA_TRY(ctx->val.upload(vv.data(), vv.size()));
        // Sliced ELL: groups of 32 consecutive (sorted) rows, each group padded
        // to its longest row with (column 0, value 0) and stored slot-major,
        // so a warp's 32 lanes read one nonzero slot as one coalesced segment.
        const int groups = (m + 31) / 32;
        std::vector<int> so((size_t)groups + 1, 0), sc;
        std::vector<double> sv;
        for (int g = 0; g < groups; ++g) {
            int len = 0;
            for (int l = 0; l < 32 && 32 * g + l < m; ++l)
                len = std::max(len, rp[(size_t)(32 * g + l) + 1] - rp[(size_t)(32 * g + l)]);
            so[(size_t)g + 1] = so[(size_t)g] + 32 * len;
            for (int t = 0; t < len; ++t)
                for (int l = 0; l < 32; ++l) {
                    const int row = 32 * g + l;
                    const bool real = row < m && t < rp[(size_t)row + 1] - rp[(size_t)row];
                    sc.push_back(real ? ci[(size_t)rp[(size_t)row] + t] : 0);
                    sv.push_back(real ? vv[(size_t)rp[(size_t)row] + t] : 0.0);
                }
        }
        ctx->sell_groups = groups;
        ACHR_CUDA_TRY(ctx->sell_off.upload(so.data(), so.size()));
        ACHR_CUDA_TRY(ctx->sell_col.upload(sc.data(), sc.size()));
        ACHR_CUDA_TRY(ctx->sell_val.upload(sv.data(), sv.size()));
        // CSC over the same (sorted) rows, for the transposed product S^T z.
        ctx->h_row_order = order_r;
        std::vector<int> cp((size_t)n + 1, 0), cr(ci.size());
        std::vector<double> cv(ci.size());
        for (int c : ci) cp[(size_t)c + 1]++;
        for (int j = 0; j < n; ++j) cp[(size_t)j + 1] += cp[(size_t)j];
        {
            std::vector<int> fill(cp.begin(), cp.end() - 1);
            for (int q = 0; q < m; ++q)
                for (int t = rp[(size_t)q]; t < rp[(size_t)q + 1]; ++t) {
                    const int dst = fill[(size_t)ci[(size_t)t]]++;
                    cr[(size_t)dst] = q;
                    cv[(size_t)dst] = vv[(size_t)t];
                }
        }
        ACHR_CUDA_TRY(ctx->csc_ptr.upload(cp.data(), cp.size()));
        ACHR_CUDA_TRY(ctx->csc_row.upload(cr.data(), cr.size()));
        ACHR_CUDA_TRY(ctx->csc_val.upload(cv.data(), cv.size()));
    }
    ACHR_CUDA_TRY(ctx->counters.alloc(achr::CNT_SLOTS));

    // Warmup matrix with an even leading dimension so every column starts on a
    // 16-byte boundary (a TMA bulk-copy requirement).
    ctx->ldw = (n + 1) & ~1;
    ACHR_CUDA_TRY(ctx->warmup.alloc((size_t)ctx->ldw * n_warmup));
    ACHR_CUDA_TRY(cudaMemset(ctx->warmup.p, 0, sizeof(double) * (size_t)ctx->ldw * n_warmup));
    ACHR_CUDA_TRY(cudaMemcpy2D(ctx->warmup.p, sizeof(double) * ctx->ldw, warmup, sizeof(double) * n,
                               sizeof(double) * n, n_warmup, cudaMemcpyHostToDevice));

    // Null space (computeKernelCuda, ACHRCuda.cu:436-502).
    std::vector<double> denseS((size_t)m * n, 0.0);
    for (int r = 0; r < m; ++r)
        for (int q = ctx->h_rowptr[r]; q < ctx->h_rowptr[(size_t)r + 1]; ++q)
            denseS[(size_t)ctx->h_colidx[q] * m + r] = ctx->h_val[q];
    std::vector<double> Nh;
    int d = 0;
    if (m == 0) {
        // No constraints: the reference's rule keeps every column (identity basis).
        d = n;
        Nh.assign((size_t)n * n, 0.0);
        for (int i = 0; i < n; ++i) Nh[(size_t)i * n + i] = 1.0;
    } else if (opt.null_space == ACHR_NULL_FIXED) {
        // S with a unit row for every fixed reaction (lb == ub): those reactions are held too.
        std::vector<int> fixed;
        for (int i = 0; i < n; ++i)
            if (model->lb[i] == model->ub[i]) fixed.push_back(i);
        const int ma = m + (int)fixed.size();
        std::vector<double> Sa((size_t)ma * n, 0.0);
        for (int j = 0; j < n; ++j)
            std::memcpy(Sa.data() + (size_t)j * ma, denseS.data() + (size_t)j * m, sizeof(double) * m);
        for (size_t k = 0; k < fixed.size(); ++k) Sa[(size_t)fixed[k] * ma + (size_t)m + k] = 1.0;
        double kappa_aug = 1.0;
        st = null_space_sts(n, ma, Sa, Nh, d, kappa_aug);
        if (st != ACHR_OK) return st;
        ctx->kappa_sst = INFINITY;  // the deferred projector (built from S alone) would not match this basis
    } else {
        st = (opt.null_space == ACHR_NULL_SVD_S) ? null_space_svd_s(n, m, denseS, Nh, d, ctx->kappa_sst)
                                                 : null_space_sts(n, m, denseS, Nh, d, ctx->kappa_sst);
        if (st != ACHR_OK) return st;
    }
    st = upload_null_space(ctx, Nh.data(), d);
    if (st != ACHR_OK) return st;
    // Large models reproject a chain through (S S^T)^+ on the residual (about
    // m^2 FP32 operations) instead of N (N^T x) (4 n d FP64 operations).
    const bool want_residual_form =
        opt.reproject_form == 2 || (opt.reproject_form == 0 && (double)n * (double)d >= 4.0e6);
    if (want_residual_form && m > 0 && m <= std::min(np, 8192)) {
        st = achr::build_pinv32(ctx);
        if (st != ACHR_OK) return st;
    }

    // Centre of the warmup points and the centre accumulator (after the
    // FEASIBLE-mode projection of the warmup points).
    ACHR_CUDA_TRY(ctx->c0.alloc(np));
    ACHR_CUDA_TRY(ctx->A0.alloc(np));
    st = prepare_warmup_and_centre(ctx);
    if (st != ACHR_OK) return st;

    owned = nullptr;  // release from the guard
    *out = ctx;
    g_last_error.clear();
    return ACHR_OK;
}

achr_status achr_set_null_space(achr_ctx *ctx, const double *N, int32_t d) {
    if (!ctx || (!N && d > 0) || d < 0 || d > ctx->n) return fail(ACHR_ERR_INVALID, "bad null-space arguments");
    achr_status st = upload_null_space(ctx, N, d);
    if (st != ACHR_OK || ctx->opt.mode != ACHR_MODE_FEASIBLE) return st;
    return prepare_warmup_and_centre(ctx);  // re-project the warmup points onto the new basis
}

achr_status achr_get_null_space_dim(const achr_ctx *ctx, int32_t *d) {
    if (!ctx || !d) return fail(ACHR_ERR_INVALID, "NULL argument");
    *d = ctx->d;
    return ACHR_OK;
}

achr_status achr_get_null_space(const achr_ctx *ctx, double *N_out) {
    if (!ctx || !N_out) return fail(ACHR_ERR_INVALID, "NULL argument");
    if (ctx->d > 0)
        ACHR_CUDA_TRY(cudaMemcpy(N_out, ctx->N.p, sizeof(double) * (size_t)ctx->n * ctx->d, cudaMemcpyDeviceToHost));
    return ACHR_OK;
}

achr_status achr_get_centre(const achr_ctx *ctx, double *centre_out) {
    if (!ctx || !centre_out) return fail(ACHR_ERR_INVALID, "NULL argument");
    ACHR_CUDA_TRY(cudaMemcpy(centre_out, ctx->c0.p, sizeof(double) * ctx->n, cudaMemcpyDeviceToHost));
    return ACHR_OK;
}

achr_status achr_sample_device(achr_ctx *ctx, uint64_t seed, uint64_t chain_offset, int32_t n_points, int32_t n_steps,
                               double *d_points_out, int64_t ld_out, void *stream, achr_stats *stats) {
    if (!ctx) return fail(ACHR_ERR_INVALID, "ctx is NULL");
    if (n_points < 0 || n_steps < 0) return fail(ACHR_ERR_INVALID, "n_points and n_steps must be >= 0");
    if (n_points > 0 && (!d_points_out || ld_out < n_points)) return fail(ACHR_ERR_INVALID, "bad output buffer");
    if (chain_offset + (uint64_t)n_points < chain_offset) return fail(ACHR_ERR_INVALID, "chain ids overflow");
    cudaStream_t s = (cudaStream_t)stream;
    const ChainArgs a = chain_args(ctx, seed, chain_offset, n_points, n_steps, d_points_out, ld_out);
    ACHR_CUDA_TRY(cudaMemsetAsync(ctx->counters.p, 0, sizeof(unsigned long long) * achr::CNT_SLOTS, s));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (stats) {
        ACHR_CUDA_TRY(cudaEventCreate(&e0));
        ACHR_CUDA_TRY(cudaEventCreate(&e1));
        ACHR_CUDA_TRY(cudaEventRecord(e0, s));
    }
    // Reprojections either inside the chain kernel, or deferred to a batched
    // tensor-core pass between segmented launches (achr_defer.cu).
    const bool deferred = achr::defer_selected(ctx) && n_points > 0 && n_steps > 0;
    if (ctx->opt.reproject_form == 3 && !deferred && n_points > 0 && n_steps > 0 && ctx->opt.check_period > 0 &&
        ctx->m > 0) {
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        return fail(ACHR_ERR_UNSUPPORTED,
                    "deferred reprojection needs n_mets <= the chain kernel's padded length and a condition number "
                    "of S S^T of at most 2e4 (its BF16-split passes converge only then)");
    }
    cudaError_t e = cudaSuccess;
    achr_status dst = ACHR_OK;
    if (deferred) dst = achr::defer_sample(ctx, a, ctx->opt.threads_per_chain, s, stats != nullptr);
    else e = achr::launch_chains(a, ctx->opt.threads_per_chain, s);
    if (e != cudaSuccess || dst != ACHR_OK) {
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        return dst != ACHR_OK ? dst : cuda_fail(e, "chain kernel launch");
    }
    if (!stats) return ACHR_OK;
    ACHR_CUDA_TRY(cudaEventRecord(e1, s));
    ACHR_CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    achr_status rst = read_counters(ctx, stats, ms);
    if (rst == ACHR_OK) rst = deferred_stats(ctx, deferred, stats);
    return rst;
}

}  // extern "C"

namespace {

using achr::set_merged_bound;

ChainArgs chain_args(const achr_ctx *ctx, uint64_t seed, uint64_t chain_offset, int32_t n_points, int32_t n_steps,
                     double *d_points_out, int64_t ld_out) {
    ChainArgs a{};
    a.n = ctx->n;
    a.m = ctx->m;
    a.W = ctx->W;
    a.d = ctx->d;
    a.np = ctx->np;
    a.ldw = ctx->ldw;
    a.P = n_points;
    a.T = n_steps;
    a.warmup = ctx->warmup.p;
    a.c0 = ctx->c0.p;
    a.A0 = ctx->A0.p;
    a.lbub = ctx->lbub.p;
    a.bnd = ctx->bnd.p;
    a.bound_err = ctx->bound_err;
    a.dtol_hi = f32_up(ctx->opt.d_tol) * (1.0f + 9.5367431640625e-07f);
    a.dtol_lo = f32_down(ctx->opt.d_tol) * (1.0f - 9.5367431640625e-07f);
    a.utol32 = (float)ctx->opt.u_tol;
    a.mmt32 = (float)ctx->opt.max_min_tol;
    set_merged_bound(a, ctx->opt.u_tol, ctx->opt.bracket_pass == 1 ? INFINITY
                                        : ctx->n_dirs > 0           ? ctx->dir_norm_max
                                                                    : 2.0 * ctx->box_norm);
    a.row_ptr = ctx->rowptr.p;
    a.col_idx = ctx->colidx.p;
    a.val = ctx->val.p;
    a.pinv32 = ctx->pinv32.p;
    a.csc_ptr = ctx->csc_ptr.p;
    a.csc_row = ctx->csc_row.p;
    a.csc_val = ctx->csc_val.p;
    a.sell_off = ctx->sell_groups > 0 ? ctx->sell_off.p : nullptr;
    a.sell_col = ctx->sell_col.p;
    a.sell_val = ctx->sell_val.p;
    a.sell_groups = ctx->sell_groups;
    a.N = ctx->N.p;
    a.out = d_points_out;
    a.ld_out = ld_out;
    a.seed = seed;
    a.chain_offset = chain_offset;
    a.check_period = ctx->opt.check_period > 0 ? ctx->opt.check_period : 0x7fffffff;
    a.max_attempts = ctx->opt.max_attempts;
    a.centre_offset = ctx->opt.centre_offset;
    a.exact_ratio = ctx->opt.exact_ratio;
    a.final_project = ctx->opt.mode == ACHR_MODE_FEASIBLE ? 1 : 0;
    a.residual_tol = ctx->opt.residual_tol;
    a.max_min_tol = ctx->opt.max_min_tol;
    a.u_tol = ctx->opt.u_tol;
    a.d_tol = ctx->opt.d_tol;
    a.feasibility_tol = ctx->opt.feasibility_tol;
    a.counters = ctx->counters.p;
    a.step0 = 0;
    a.x_in = nullptr;
    a.A_in = nullptr;
    a.A_out = nullptr;
    a.ld_state = 0;
    a.hit_and_run = 0;
    const long long wl = ctx->opt.wait_limit_ns;
    a.wait_ns = wl != 0 ? (unsigned long long)(wl < 0 ? -wl : wl) : 0ull;
    a.wait_never = wl < 0 ? 1 : 0;
    if (ctx->n_dirs > 0) {
        a.warmup = ctx->dirs.p;
        a.W = ctx->n_dirs;
        a.A0 = ctx->zeros.p;
        a.hit_and_run = 1;
    }
    return a;
}

}  // namespace

extern "C" {

achr_status achr_set_directions(achr_ctx *ctx, const double *dirs, int64_t ld, int32_t n_dirs) {
    if (!ctx) return fail(ACHR_ERR_INVALID, "ctx is NULL");
    if (n_dirs < 0 || (n_dirs > 0 && (!dirs || ld < ctx->n))) return fail(ACHR_ERR_INVALID, "bad direction pool");
    if (n_dirs == 0) {
        ctx->dirs.reset();
        ctx->zeros.reset();
        ctx->n_dirs = 0;
        return ACHR_OK;
    }
    ctx->n_dirs = 0;
    ACHR_CUDA_TRY(ctx->dirs.alloc((size_t)ctx->ldw * n_dirs));
    ACHR_CUDA_TRY(cudaMemset(ctx->dirs.p, 0, sizeof(double) * (size_t)ctx->ldw * n_dirs));
    // host or device source (unified addressing decides the direction)
    ACHR_CUDA_TRY(cudaMemcpy2D(ctx->dirs.p, sizeof(double) * ctx->ldw, dirs, sizeof(double) * ld,
                               sizeof(double) * ctx->n, n_dirs, cudaMemcpyDefault));
    ACHR_CUDA_TRY(ctx->zeros.alloc((size_t)ctx->np));
    ACHR_CUDA_TRY(cudaMemset(ctx->zeros.p, 0, sizeof(double) * (size_t)ctx->np));
    {
        // the longest direction bounds ||d|| for the brackets formed in phase A
        DevBuf<unsigned long long> nb;
        ACHR_CUDA_TRY(nb.alloc(1));
        ACHR_CUDA_TRY(cudaMemset(nb.p, 0, sizeof(unsigned long long)));
        col_norm_max_kernel<<<n_dirs, 256>>>(ctx->n, ctx->ldw, ctx->dirs.p, nb.p);
        ACHR_CUDA_TRY(cudaGetLastError());
        unsigned long long bits = 0;
        ACHR_CUDA_TRY(cudaMemcpy(&bits, nb.p, sizeof bits, cudaMemcpyDeviceToHost));
        double nm;
        std::memcpy(&nm, &bits, sizeof nm);
        ctx->dir_norm_max = nm;
    }
    ctx->n_dirs = n_dirs;
    return ACHR_OK;
}

achr_status achr_get_directions(const achr_ctx *ctx, double *dirs_out) {
    if (!ctx || !dirs_out) return fail(ACHR_ERR_INVALID, "NULL argument");
    if (ctx->n_dirs == 0) return ACHR_OK;
    ACHR_CUDA_TRY(cudaMemcpy2D(dirs_out, sizeof(double) * ctx->n, ctx->dirs.p, sizeof(double) * ctx->ldw,
                               sizeof(double) * ctx->n, ctx->n_dirs, cudaMemcpyDefault));
    return ACHR_OK;
}

int32_t achr_get_n_directions(const achr_ctx *ctx) { return ctx ? ctx->n_dirs : 0; }

achr_status achr_sample_resume(achr_ctx *ctx, uint64_t seed, uint64_t chain_offset, int32_t n_points, int32_t step0,
                               int32_t n_steps, int32_t resume, double *d_points, double *d_centre_acc, int64_t ld,
                               void *stream, achr_stats *stats) {
    if (!ctx) return fail(ACHR_ERR_INVALID, "ctx is NULL");
    if (n_points < 0 || n_steps < 0 || step0 < 0 || (!resume && step0 != 0))
        return fail(ACHR_ERR_INVALID, "bad step range (a fresh start begins at step 0)");
    if ((int64_t)step0 + n_steps > 2147483647LL) return fail(ACHR_ERR_INVALID, "step index overflow");
    if (n_points > 0 && (!d_points || !d_centre_acc || ld < n_points))
        return fail(ACHR_ERR_INVALID, "bad state buffers");
    cudaStream_t s = (cudaStream_t)stream;
    ChainArgs a = chain_args(ctx, seed, chain_offset, n_points, n_steps, d_points, ld);
    a.step0 = step0;
    a.x_in = resume ? d_points : nullptr;
    a.A_in = resume ? d_centre_acc : nullptr;
    a.A_out = d_centre_acc;
    a.ld_state = ld;
    ACHR_CUDA_TRY(cudaMemsetAsync(ctx->counters.p, 0, sizeof(unsigned long long) * achr::CNT_SLOTS, s));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (stats) {
        ACHR_CUDA_TRY(cudaEventCreate(&e0));
        ACHR_CUDA_TRY(cudaEventCreate(&e1));
        ACHR_CUDA_TRY(cudaEventRecord(e0, s));
    }
    const bool deferred = achr::defer_selected(ctx) && n_points > 0 && n_steps > 0;
    cudaError_t e = cudaSuccess;
    achr_status dst = ACHR_OK;
    if (deferred) dst = achr::defer_sample(ctx, a, ctx->opt.threads_per_chain, s, stats != nullptr);
    else e = achr::launch_chains(a, ctx->opt.threads_per_chain, s);
    if (e != cudaSuccess || dst != ACHR_OK) {
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        return dst != ACHR_OK ? dst : cuda_fail(e, "chain kernel launch");
    }
    if (!stats) return ACHR_OK;
    ACHR_CUDA_TRY(cudaEventRecord(e1, s));
    ACHR_CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    achr_status rst = read_counters(ctx, stats, ms);
    if (rst == ACHR_OK) rst = deferred_stats(ctx, deferred, stats);
    return rst;
}

achr_status achr_sample(achr_ctx *ctx, uint64_t seed, uint64_t chain_offset, int32_t n_points, int32_t n_steps,
                        double *points_out, achr_stats *stats) {
    if (!ctx) return fail(ACHR_ERR_INVALID, "ctx is NULL");
    if (n_points < 0 || n_steps < 0) return fail(ACHR_ERR_INVALID, "n_points and n_steps must be >= 0");
    if (n_points > 0 && !points_out) return fail(ACHR_ERR_INVALID, "points_out is NULL");
    const size_t need = (size_t)ctx->n * (size_t)n_points;
    if (ctx->points.count < need) ACHR_CUDA_TRY(ctx->points.alloc(need));
    achr_stats local;
    achr_status st = achr_sample_device(ctx, seed, chain_offset, n_points, n_steps, ctx->points.p, n_points, nullptr,
                                        stats ? stats : &local);
    if (st != ACHR_OK) return st;
    if (need) ACHR_CUDA_TRY(cudaMemcpy(points_out, ctx->points.p, sizeof(double) * need, cudaMemcpyDeviceToHost));
    return ACHR_OK;
}

void achr_destroy(achr_ctx *ctx) {
    if (!ctx) return;
    achr::defer_free(ctx->defer);
    achr::reproj_free(ctx->reproj);
    delete ctx;
}

}  // extern "C"

namespace {

// Autotuning results per (default padded length, device): threads per chain.
std::mutex g_tune_mutex;
std::map<std::pair<int, int>, int> g_tune_cache;
// Guided self-scheduling of the batched work queues: an item holds the work
// queued behind it divided by (this x the queue's CTAs); set by
// achr_set_batch_tiles or achr_autotune_batch.
std::atomic<int> g_batch_tiles{4};

struct StreamSet {
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t> events;
    ~StreamSet() {
        for (cudaStream_t s : streams) cudaStreamDestroy(s);
        for (cudaEvent_t e : events) cudaEventDestroy(e);
    }
};

}  // namespace

extern "C" {

achr_status achr_autotune(achr_ctx *ctx, int32_t *threads_per_chain_out) {
    if (!ctx) return fail(ACHR_ERR_INVALID, "ctx is NULL");
    int dev = 0;
    ACHR_CUDA_TRY(cudaGetDevice(&dev));
    const std::pair<int, int> key(achr::chain_padded_length(ctx->n, 0), dev);
    int cand[8];
    int nc = 0;
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {  // known size: time only the cached choice (its rate feeds batching)
            cand[0] = it->second;
            nc = 1;
        }
    }
    if (nc == 0) nc = achr::chain_candidates(ctx->n, ctx->np, cand, 8);
    if (nc == 0) return fail(ACHR_ERR_UNSUPPORTED, "no chain-kernel configuration to tune");
    int sms = 0;
    ACHR_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    // A short run that fills the GPU a few times over: 4 chains per SM, 32 steps.
    const int P = 4 * sms, T = 32;
    const size_t need = (size_t)ctx->n * (size_t)P;
    if (ctx->points.count < need) ACHR_CUDA_TRY(ctx->points.alloc(need));
    const int saved = ctx->opt.threads_per_chain;
    int best = cand[0];
    double best_ms = 1e300;
    for (int c = 0; c < nc; ++c) {
        ctx->opt.threads_per_chain = cand[c];
        achr_stats st;
        achr_status r = achr_sample_device(ctx, 0x5eedull, 0, P, 4, ctx->points.p, P, nullptr, &st);  // warm-up
        if (r == ACHR_OK) r = achr_sample_device(ctx, 0x5eedull, 0, P, T, ctx->points.p, P, nullptr, &st);
        if (r != ACHR_OK) {
            ctx->opt.threads_per_chain = saved;
            return r;
        }
        if (st.kernel_ms < best_ms) {
            best_ms = st.kernel_ms;
            best = cand[c];
        }
    }
    ctx->opt.threads_per_chain = best;
    ctx->tuned_rate = best_ms > 0 ? (double)P * T / best_ms : 0.0;
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        g_tune_cache[key] = best;
    }
    if (threads_per_chain_out) *threads_per_chain_out = best;
    return ACHR_OK;
}

achr_status achr_sample_batch(achr_ctx *const *ctxs, int32_t n_models, const int32_t *n_points, int32_t n_steps,
                              uint64_t seed, double *const *d_points_out, const int64_t *ld_out, void *stream,
                              achr_batch_stats *stats, double *model_ms_out) {
    if (!ctxs || !n_points || !d_points_out || !ld_out || n_models <= 0 || n_steps < 0)
        return fail(ACHR_ERR_INVALID, "bad batch arguments");
    int dev = 0, sms = 0;
    ACHR_CUDA_TRY(cudaGetDevice(&dev));
    ACHR_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    // Per model: its configuration, its launch arguments and the predicted time of one chain.
    std::vector<ChainArgs> args((size_t)n_models);
    std::vector<double> chain_time((size_t)n_models);
    std::vector<int> cfg_key((size_t)n_models);
    uint64_t off = 0;
    for (int k = 0; k < n_models; ++k) {
        achr_ctx *c = ctxs[k];
        if (!c || n_points[k] < 0 || (n_points[k] > 0 && (!d_points_out[k] || ld_out[k] < n_points[k])))
            return fail(ACHR_ERR_INVALID, "bad batch entry " + std::to_string(k));
        int bd = 0, ept = 0;
        if (!achr::chain_config(c->n, c->opt.threads_per_chain, &bd, &ept) || bd * ept > c->np)
            return fail(ACHR_ERR_UNSUPPORTED, "no chain-kernel configuration for batch entry " + std::to_string(k));
        cfg_key[(size_t)k] = bd * 100 + ept;
        // disjoint chain ids: model k uses ids off .. off + P_k - 1
        args[(size_t)k] = chain_args(c, seed, off, n_points[k], n_steps, d_points_out[k], ld_out[k]);
        off += (uint64_t)n_points[k];
        // measured by the autotuner (whole-GPU rate), else padded elements x steps
        chain_time[(size_t)k] = c->tuned_rate > 0 ? (double)n_steps / c->tuned_rate
                                                  : (double)n_steps * (double)(bd * ept) * 1e-9;
    }
    // One work queue per configuration, its items from plan_queue
    // (achr_queue_plan.h) with `tiles` = 4 unless tuned.
    const int tiles = g_batch_tiles.load();
    struct Group {
        int bd, ept, grid = 0;
        std::vector<int> models;
        std::vector<int4> items;
        double work = 0.0;
        size_t extra = 0;
    };
    std::vector<Group> groups;
    for (int k = 0; k < n_models; ++k) {
        size_t g = 0;
        while (g < groups.size() && groups[g].bd * 100 + groups[g].ept != cfg_key[(size_t)k]) ++g;
        if (g == groups.size()) {
            Group ng;
            ng.bd = cfg_key[(size_t)k] / 100;
            ng.ept = cfg_key[(size_t)k] % 100;
            groups.push_back(ng);
        }
        groups[g].models.push_back(k);
        groups[g].work += (double)n_points[k] * chain_time[(size_t)k];
    }
    size_t total_items = 0;
    for (Group &G : groups) {
        // The residual-form reprojection keeps (S S^T)^+ r in shared memory: the
        // group keeps it only if that costs no resident CTA per SM.
        size_t extra = 0;
        for (int k : G.models) {
            ChainArgs &a = args[(size_t)k];
            if (a.pinv32 && a.m > a.ldw) a.pinv32 = nullptr;  // the residual stays below the column's padding
            if (a.pinv32) extra = std::max(extra, ((size_t)a.m * sizeof(float) + 15) & ~(size_t)15);
        }
        achr::ChainQueue probe{};
        int per_sm = 0, per_sm_z = 0;
        cudaError_t e = achr::launch_chain_queue(G.bd, G.ept, probe, nullptr, 0, &per_sm);
        if (e != cudaSuccess) return cuda_fail(e, "work-queue kernel configuration");
        if (extra) {
            probe.extra_smem = extra;
            e = achr::launch_chain_queue(G.bd, G.ept, probe, nullptr, 0, &per_sm_z);
            if (e != cudaSuccess || per_sm_z < per_sm) {
                (void)cudaGetLastError();
                extra = 0;
                for (int k : G.models) args[(size_t)k].pinv32 = nullptr;
            }
        }
        G.extra = extra;
        G.grid = sms * per_sm;
        for (const achr::QueueItem &q : achr::plan_queue(G.models, n_points, chain_time.data(), G.grid, tiles))
            G.items.push_back(make_int4(q.model, q.p0, q.p1, 0));
        total_items += G.items.size();
    }
    std::stable_sort(groups.begin(), groups.end(), [](const Group &x, const Group &y) { return x.work > y.work; });

    // Device copies: the models' arguments, the items of every group, and the
    // queue heads, per-model done counts and finish stamps (zeroed in the graph).
    DevBuf<ChainArgs> d_args;
    DevBuf<int4> d_items;
    DevBuf<int> d_ints;  // [0, groups): queue heads, [groups, groups + n_models): chains done
    DevBuf<unsigned long long> stamps;
    ACHR_CUDA_TRY(d_args.upload(args.data(), args.size()));
    {
        std::vector<int4> all;
        all.reserve(total_items);
        for (const Group &G : groups) all.insert(all.end(), G.items.begin(), G.items.end());
        ACHR_CUDA_TRY(d_items.upload(all.data(), all.size()));
    }
    const size_t n_ints = groups.size() + (size_t)n_models;
    ACHR_CUDA_TRY(d_ints.alloc(n_ints));
    size_t n_ctas = 0;
    for (Group &G : groups) {
        G.grid = (int)std::min<size_t>((size_t)G.grid, G.items.size());
        n_ctas += (size_t)G.grid;
    }
    // [0, n_models): each model's finish, [n_models]: graph start, then one per CTA: its exit
    ACHR_CUDA_TRY(stamps.alloc((size_t)n_models + 1 + n_ctas));

    cudaStream_t main = (cudaStream_t)stream;
    StreamSet ss;
    if (main == nullptr) {  // the legacy default stream cannot be captured: use a private stream
        cudaStream_t own = nullptr;
        ACHR_CUDA_TRY(cudaStreamCreateWithFlags(&own, cudaStreamNonBlocking));
        ss.streams.push_back(own);
        main = own;
    }
    const size_t first = ss.streams.size();
    ss.streams.resize(first + groups.size(), nullptr);
    ss.events.resize(groups.size() + 3, nullptr);
    for (size_t q = first; q < ss.streams.size(); ++q)
        ACHR_CUDA_TRY(cudaStreamCreateWithFlags(&ss.streams[q], cudaStreamNonBlocking));
    for (auto &ev : ss.events) ACHR_CUDA_TRY(cudaEventCreate(&ev));
    const size_t ng = groups.size();
    cudaEvent_t fork = ss.events[ng], t0 = ss.events[ng + 1], t1 = ss.events[ng + 2];
    // One graph: zero the queue state and every model's counters, fork, one
    // persistent work-queue kernel per configuration (largest total work
    // first) on its own stream, join.
    cudaGraph_t graph = nullptr;
    ACHR_CUDA_TRY(cudaStreamBeginCapture(main, cudaStreamCaptureModeThreadLocal));
    cudaError_t ce = cudaMemsetAsync(d_ints.p, 0, sizeof(int) * n_ints, main);
    for (int k = 0; k < n_models && ce == cudaSuccess; ++k)
        ce = cudaMemsetAsync(ctxs[k]->counters.p, 0, sizeof(unsigned long long) * achr::CNT_SLOTS, main);
    if (ce == cudaSuccess) {
        stamp_kernel<<<1, 1, 0, main>>>(stamps.p + n_models);
        ce = cudaGetLastError();
    }
    if (ce == cudaSuccess) ce = cudaEventRecord(fork, main);
    size_t item0 = 0, cta0 = (size_t)n_models + 1;
    for (size_t g = 0; g < ng && ce == cudaSuccess; ++g) {
        const Group &G = groups[g];
        cudaStream_t sg = ss.streams[first + g];
        achr::ChainQueue q{};
        q.args = d_args.p;
        q.items = d_items.p + item0;
        q.n_items = (int)G.items.size();
        q.next = d_ints.p + g;
        q.chains_done = d_ints.p + ng;
        q.done_ns = stamps.p;
        q.extra_smem = G.extra;
        q.cta_ns = stamps.p + cta0;
        item0 += G.items.size();
        cta0 += (size_t)G.grid;
        ce = cudaStreamWaitEvent(sg, fork, 0);
        if (ce == cudaSuccess) ce = achr::launch_chain_queue(G.bd, G.ept, q, sg, G.grid, nullptr);
        if (ce == cudaSuccess) ce = cudaEventRecord(ss.events[g], sg);
        if (ce == cudaSuccess) ce = cudaStreamWaitEvent(main, ss.events[g], 0);
    }
    cudaError_t ee = cudaStreamEndCapture(main, &graph);
    if (ce != cudaSuccess || ee != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return cuda_fail(ce != cudaSuccess ? ce : ee, "batched graph capture");
    }
    cudaGraphExec_t exec = nullptr;
    ce = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaGraphInstantiate");
    ce = cudaEventRecord(t0, main);
    if (ce == cudaSuccess) ce = cudaGraphLaunch(exec, main);
    if (ce == cudaSuccess) ce = cudaEventRecord(t1, main);
    if (ce == cudaSuccess) ce = cudaEventSynchronize(t1);
    cudaGraphExecDestroy(exec);
    if (ce != cudaSuccess) return cuda_fail(ce, "batched graph launch");
    float total_ms = 0.0f;
    ACHR_CUDA_TRY(cudaEventElapsedTime(&total_ms, t0, t1));
    std::vector<unsigned long long> ts((size_t)n_models + 1 + n_ctas);
    ACHR_CUDA_TRY(cudaMemcpy(ts.data(), stamps.p, sizeof(unsigned long long) * ts.size(), cudaMemcpyDeviceToHost));
    achr_batch_stats bs{};
    for (int k = 0; k < n_models; ++k) {
        const float mk = n_points[k] > 0 ? (float)((double)(ts[(size_t)k] - ts[(size_t)n_models]) * 1e-6) : 0.0f;
        if (model_ms_out) model_ms_out[k] = mk;
        achr_stats st;
        achr_status r = read_counters(ctxs[k], &st, mk);
        if (r != ACHR_OK) return r;
        bs.accepted += st.accepted;
        bs.rejected += st.rejected;
        bs.reprojections += st.reprojections;
        bs.stuck_chains += st.stuck_chains;
        bs.max_residual = std::max(bs.max_residual, st.max_residual);
        bs.max_bound_violation = std::max(bs.max_bound_violation, st.max_bound_violation);
    }
    // Idle share of each queue's CTA slots at its end: (max - mean) / max of
    // the exit times of its CTAs (when each found the queue empty), averaged
    // over the queues weighted by their predicted work.
    double imb = 0.0, wsum = 0.0;
    size_t c0 = (size_t)n_models + 1;
    for (const Group &G : groups) {
        double cmax = 0.0, cmean = 0.0;
        for (int c = 0; c < G.grid; ++c) {
            const double t = (double)(ts[c0 + (size_t)c] - ts[(size_t)n_models]) * 1e-6;
            cmax = std::max(cmax, t);
            cmean += t;
        }
        c0 += (size_t)G.grid;
        if (G.grid > 0 && cmax > 0.0) {
            cmean /= (double)G.grid;
            imb += G.work * (cmax - cmean) / cmax;
            wsum += G.work;
        }
    }
    bs.graph_ms = total_ms;
    bs.load_imbalance = wsum > 0.0 ? imb / wsum : 0.0;
    if (stats) *stats = bs;
    return ACHR_OK;
}

achr_status achr_set_batch_tiles(int32_t tiles) {
    if (tiles < 1 || tiles > 1024) return fail(ACHR_ERR_INVALID, "tiles must be in [1, 1024]");
    g_batch_tiles.store(tiles);
    return ACHR_OK;
}

int32_t achr_get_batch_tiles(void) { return g_batch_tiles.load(); }

achr_status achr_autotune_batch(achr_ctx *const *ctxs, int32_t n_models, const int32_t *n_points, int32_t n_steps,
                                uint64_t seed, double *const *d_points_out, const int64_t *ld_out, void *stream,
                                int32_t *tiles_out) {
    static const int kCand[] = {1, 2, 4, 8, 16};
    const int saved = g_batch_tiles.load();
    int best = saved;
    double best_ms = 1e300;
    for (int c : kCand) {
        g_batch_tiles.store(c);
        achr_batch_stats st;
        achr_status r = achr_sample_batch(ctxs, n_models, n_points, n_steps, seed, d_points_out, ld_out, stream, &st,
                                          nullptr);
        if (r != ACHR_OK) {
            g_batch_tiles.store(saved);
            return r;
        }
        if (st.graph_ms < best_ms) {
            best_ms = st.graph_ms;
            best = c;
        }
    }
    g_batch_tiles.store(best);
    if (tiles_out) *tiles_out = best;
    return ACHR_OK;
}

}  // extern "C"
