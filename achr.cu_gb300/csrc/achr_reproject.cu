// Batched null-space reprojection of many chains on the tensor cores, and the
// periodic-reprojection sampling driver built on it.
//
// The reference reprojects one chain at a time, x <- N (N^T x), as two FP64
// GEMVs (reprojectPoint / reprojectPoint2, ACHRcu/ACHRCuda.cu:208-230,
// triggered at :338-343).  Here all chains of a block are reprojected at
// once with the same orthogonal projector written through S:
//
//     N N^T = I - S^T (S S^T)^+ S,   so   x <- x - S^T (B (S x)),  B = (S S^T)^+.
//
//   1. r = S x for every chain, FP64 sparse (exact to rounding; |r| is the
//      small infeasibility the chain has accumulated), split into BF16 hi + lo;
//   2. z = B r as one tensor-core GEMM over all chains, with B split the same
//      way and the three leading split products (Bh rh + Bh rl + Bl rh)
//      accumulated in FP32 (achr_tc_gemm.cu);
//   3. x <- clip(x - S^T z) in FP64 sparse, the same clip the reference applies
//      after reprojecting (correctBounds, :193-206, :347-350), and the chain's
//      centre accumulator follows the point.
//
// The low-precision GEMM only ever sees the residual, so its relative error
// (about 2^-16 times the condition number of S S^T on its range) multiplies
// |S x|, not |x|: one pass takes a residual of 1e-9 to ~1e-11 while the
// point moves by no more than the residual's preimage.  Applying N N^T to x
// itself in BF16 would move every coordinate by ~1e-5 |x| and leave |S x|
// near 1e-2 for fluxes of size 1000.
#include <cublas_v2.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cusolverDn.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "achr_ctx.h"

extern "C" void achr_io_set_error(const char *msg);

namespace achr {

void reproj_free(ReprojState *r) { delete r; }

namespace {

constexpr int kRowChunk = 64;   // residual rows per staging tile (one 128-byte BF16 row per chain)
constexpr int kResWarps = 4;
constexpr int kStageStride = 72;  // BF16 entries per chain row of the staging tile (144 B: 16-byte aligned)
constexpr int kCorrWarps = 8;
constexpr int kMaxChunk = 65536;  // chains per GEMM

achr_status set_err(achr_status st, const std::string &msg) {
    achr_io_set_error(msg.c_str());
    return st;
}

achr_status cuda_err(cudaError_t e, const char *what) {
    return set_err(ACHR_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define REPROJ_TRY(expr)                                      \
    do {                                                      \
        cudaError_t e_ = (expr);                              \
        if (e_ != cudaSuccess) return achr::cuda_err(e_, #expr); \
    } while (0)

__device__ __forceinline__ unsigned long long abs_bits64(double v) {
    return (unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull;
}

// r = S x for 32 chains per block column (lane = chain, so every load of x is
// one coalesced 256-byte row segment) and 64-row chunks per warp.  With SPLIT
// the residuals go out as BF16 hi/lo rows of R (chain-major, K = metabolite
// contiguous, the layout the GEMM's TMA maps read), staged through shared
// memory so every chain row is written as 16-byte pieces.  Always: the
// largest |r| (as non-negative double bits) goes to *maxbits.
template <bool SPLIT>
__global__ void __launch_bounds__(kResWarps * 32)
    residual_kernel(int m, int kpad, int P, const double *__restrict__ X, long long ldx,
                    const int *__restrict__ rp, const int *__restrict__ ci, const double *__restrict__ rv,
                    __nv_bfloat16 *__restrict__ Rh, __nv_bfloat16 *__restrict__ Rl,
                    unsigned long long *maxbits, const unsigned long long *prev, unsigned long long tol_bits) {
    // A chunk whose previous round found it within tolerance was not corrected,
    // so its residual is unchanged: carry the value over and skip the pass.
    if (prev && *prev <= tol_bits) {
        if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) *maxbits = *prev;
        return;
    }
    __shared__ __align__(16) __nv_bfloat16 stage[SPLIT ? kResWarps : 1][2][32 * kStageStride];
    __shared__ unsigned long long wmax[kResWarps];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int p0 = blockIdx.x * 32;
    const int p = p0 + lane;
    const bool live = p < P;
    const double *xp = X + (live ? p : 0);
    unsigned long long mx = 0;
    const int nchunks = kpad / kRowChunk;
    for (int c = blockIdx.y * kResWarps + warp; c < nchunks; c += gridDim.y * kResWarps) {
        for (int r = 0; r < kRowChunk; ++r) {
            const int i = c * kRowChunk + r;
            double acc = 0.0;
            if (i < m) {
                const int q1 = __ldg(rp + i + 1);
                for (int q = __ldg(rp + i); q < q1; ++q) {
                    const double xv = live ? xp[(long long)__ldg(ci + q) * ldx] : 0.0;
                    acc = fma(__ldg(rv + q), xv, acc);
                }
            }
            mx = max(mx, abs_bits64(acc));
            if (SPLIT) {
                const __nv_bfloat16 hi = __double2bfloat16(acc);
                const __nv_bfloat16 lo = __double2bfloat16(acc - (double)__bfloat162float(hi));
                stage[SPLIT ? warp : 0][0][lane * kStageStride + r] = hi;
                stage[SPLIT ? warp : 0][1][lane * kStageStride + r] = lo;
            }
        }
        if (SPLIT) {
            __syncwarp();
            for (int t = lane; t < 32 * (kRowChunk / 8); t += 32) {
                const int row = t / (kRowChunk / 8), part = t % (kRowChunk / 8);
                const int pp = p0 + row;
                if (pp < P) {
                    const size_t off = (size_t)pp * (size_t)kpad + (size_t)c * kRowChunk + (size_t)part * 8;
                    *reinterpret_cast<uint4 *>(Rh + off) =
                        *reinterpret_cast<const uint4 *>(&stage[SPLIT ? warp : 0][0][row * kStageStride + part * 8]);
                    *reinterpret_cast<uint4 *>(Rl + off) =
                        *reinterpret_cast<const uint4 *>(&stage[SPLIT ? warp : 0][1][row * kStageStride + part * 8]);
                }
            }
            __syncwarp();
        }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) mx = max(mx, (unsigned long long)__shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) wmax[warp] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < kResWarps; ++w) mx = max(mx, wmax[w]);
        if (mx) atomicMax(maxbits, mx);
    }
}

// x_j <- clip(x_j - sum_i S_ij z_i, lb_j, ub_j) for 32 chains per block column
// (lane = chain: loads of z and x are coalesced rows); the centre accumulator
// moves with the point.
__global__ void __launch_bounds__(kCorrWarps * 32)
    correct_kernel(int n, int P, double *__restrict__ X, long long ldx, double *__restrict__ Acc, long long lda,
                   const int *__restrict__ cp, const int *__restrict__ ri, const double *__restrict__ cv,
                   const float *__restrict__ Z, long long ldz, const double2 *__restrict__ lbub,
                   const unsigned long long *gate, unsigned long long tol_bits) {
    if (*gate <= tol_bits) return;  // this chunk's residual is already within tolerance
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int p = blockIdx.x * 32 + lane;
    if (p >= P) return;
    for (int j = blockIdx.y * kCorrWarps + warp; j < n; j += gridDim.y * kCorrWarps) {
        double dl = 0.0;
        const int q1 = __ldg(cp + j + 1);
        for (int q = __ldg(cp + j); q < q1; ++q)
            dl = fma(__ldg(cv + q), (double)__ldg(Z + (long long)__ldg(ri + q) * ldz + p), dl);
        double *xp = X + (long long)j * ldx + p;
        const double xo = *xp;
        const double2 lu = lbub[j];
        double xn = xo - dl;
        xn = xn < lu.x ? lu.x : (xn > lu.y ? lu.y : xn);
        *xp = xn;
        if (Acc) Acc[(long long)j * lda + p] += xn - xo;
    }
}

// Column k of the eigenvector matrix scaled by 1 / lambda_k (kept columns only).
__global__ void scale_columns(int m, int r, const double *__restrict__ U, const double *__restrict__ lam,
                              double *__restrict__ V) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)m * r) return;
    const int k = (int)(t / m);
    V[t] = U[t] / lam[k];
}

// B (m x m, symmetric, column-major) -> row-major BF16 hi/lo with zero K padding.
__global__ void split_matrix(int m, int kpad, const double *__restrict__ B, __nv_bfloat16 *__restrict__ Bh,
                             __nv_bfloat16 *__restrict__ Bl) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)m * kpad) return;
    const int i = (int)(t / kpad), k = (int)(t % kpad);
    const double v = k < m ? B[(long long)k * m + i] : 0.0;  // B[i][k] = B[k][i]
    const __nv_bfloat16 hi = __double2bfloat16(v);
    Bh[t] = hi;
    Bl[t] = __double2bfloat16(v - (double)__bfloat162float(hi));
}

// (S S^T)^+ (column-major FP64) to FP32, rows and columns permuted to the
// device row order of the chain kernel's S.
__global__ void pinv32_kernel(int m, const int *__restrict__ order, const double *__restrict__ B,
                              float *__restrict__ out) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)m * m) return;
    const int i = (int)(t / m), k = (int)(t % m);
    out[t] = (float)B[(long long)order[k] * m + order[i]];  // B symmetric, column-major
}

achr_status build_reproj(achr_ctx *ctx, ReprojState &R, bool want_pinv32 = false) {
    const int m = ctx->m, n = ctx->n;
    R.m = m;
    R.n = n;
    R.kpad = (m + kRowChunk - 1) / kRowChunk * kRowChunk;
    REPROJ_TRY(cudaGetDevice(&R.device));
    // CSR (as stored) and CSC of S.
    const std::vector<int> &rp = ctx->h_rowptr, &ci = ctx->h_colidx;
    const std::vector<double> &rv = ctx->h_val;
    std::vector<int> cp((size_t)n + 1, 0), ri(ci.size());
    std::vector<double> cv(ci.size());
    for (int c : ci) cp[(size_t)c + 1]++;
    for (int j = 0; j < n; ++j) cp[(size_t)j + 1] += cp[(size_t)j];
    {
        std::vector<int> fill(cp.begin(), cp.end() - 1);
        for (int i = 0; i < m; ++i)
            for (int q = rp[(size_t)i]; q < rp[(size_t)i + 1]; ++q) {
                const int dst = fill[(size_t)ci[(size_t)q]]++;
                ri[(size_t)dst] = i;
                cv[(size_t)dst] = rv[(size_t)q];
            }
    }
    REPROJ_TRY(R.rp.upload(rp.data(), rp.size()));
    REPROJ_TRY(R.ci.upload(ci.data(), ci.size()));
    REPROJ_TRY(R.rv.upload(rv.data(), rv.size()));
    REPROJ_TRY(R.cp.upload(cp.data(), cp.size()));
    REPROJ_TRY(R.ri.upload(ri.data(), ri.size()));
    REPROJ_TRY(R.cv.upload(cv.data(), cv.size()));

    // B = (S S^T)^+ from the eigen-decomposition of S S^T, eigenvalues below
    // m * lambda_max * 2.2204e-16 dropped (the reference's null-space cutoff
    // rule, ACHRCuda.cu:478-487, applied to S S^T).
    std::vector<double> dS((size_t)m * n, 0.0);
    for (int i = 0; i < m; ++i)
        for (int q = rp[(size_t)i]; q < rp[(size_t)i + 1]; ++q) dS[(size_t)ci[(size_t)q] * m + i] = rv[(size_t)q];
    DevBuf<double> S, G, lam, V, B;
    DevBuf<int> info;
    REPROJ_TRY(S.upload(dS.data(), dS.size()));
    dS.clear();
    dS.shrink_to_fit();
    REPROJ_TRY(G.alloc((size_t)m * m));
    REPROJ_TRY(lam.alloc((size_t)m));
    REPROJ_TRY(info.alloc(1));
    cublasHandle_t cb = nullptr;
    cusolverDnHandle_t sh = nullptr;
    if (cublasCreate(&cb) != CUBLAS_STATUS_SUCCESS) return set_err(ACHR_ERR_CUDA, "cublasCreate failed");
    struct Guard {
        cublasHandle_t &cb;
        cusolverDnHandle_t &sh;
        ~Guard() {
            if (sh) cusolverDnDestroy(sh);
            if (cb) cublasDestroy(cb);
        }
    } guard{cb, sh};
    const double one = 1.0, zero = 0.0;
    if (cublasDgemm(cb, CUBLAS_OP_N, CUBLAS_OP_T, m, m, n, &one, S.p, m, S.p, m, &zero, G.p, m) !=
        CUBLAS_STATUS_SUCCESS)
        return set_err(ACHR_ERR_CUDA, "cublasDgemm (S S^T) failed");
    S.reset();
    if (cusolverDnCreate(&sh) != CUSOLVER_STATUS_SUCCESS) return set_err(ACHR_ERR_CUDA, "cusolverDnCreate failed");
    int lwork = 0;
    if (cusolverDnDsyevd_bufferSize(sh, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, m, G.p, m, lam.p, &lwork) !=
        CUSOLVER_STATUS_SUCCESS)
        return set_err(ACHR_ERR_NUMERIC, "syevd workspace query failed");
    {
        DevBuf<double> work;
        REPROJ_TRY(work.alloc((size_t)std::max(lwork, 1)));
        if (cusolverDnDsyevd(sh, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, m, G.p, m, lam.p, work.p, lwork,
                             info.p) != CUSOLVER_STATUS_SUCCESS)
            return set_err(ACHR_ERR_NUMERIC, "cusolverDnDsyevd (S S^T) failed");
        int h_info = 0;
        REPROJ_TRY(cudaMemcpy(&h_info, info.p, sizeof(int), cudaMemcpyDeviceToHost));
        if (h_info != 0) return set_err(ACHR_ERR_NUMERIC, "syevd of S S^T did not converge");
    }
    std::vector<double> h_lam((size_t)m);
    REPROJ_TRY(cudaMemcpy(h_lam.data(), lam.p, sizeof(double) * m, cudaMemcpyDeviceToHost));
    const double lmax = h_lam.back();
    const double tol = (double)m * lmax * 2.2204e-16;
    int k0 = 0;
    while (k0 < m && !(h_lam[(size_t)k0] > tol)) ++k0;
    const int r = m - k0;
    R.rank = r;
    R.lam_max = lmax;
    R.lam_min = r > 0 ? h_lam[(size_t)k0] : 0.0;
    REPROJ_TRY(B.alloc((size_t)m * m));
    if (r > 0) {
        REPROJ_TRY(V.alloc((size_t)m * r));
        const long long cnt = (long long)m * r;
        scale_columns<<<(unsigned)((cnt + 255) / 256), 256>>>(m, r, G.p + (size_t)k0 * m, lam.p + k0, V.p);
        REPROJ_TRY(cudaGetLastError());
        if (cublasDgemm(cb, CUBLAS_OP_N, CUBLAS_OP_T, m, m, r, &one, V.p, m, G.p + (size_t)k0 * m, m, &zero, B.p,
                        m) != CUBLAS_STATUS_SUCCESS)
            return set_err(ACHR_ERR_CUDA, "cublasDgemm (pseudo-inverse) failed");
    } else {
        REPROJ_TRY(cudaMemset(B.p, 0, sizeof(double) * (size_t)m * m));
    }
    REPROJ_TRY(R.Bh.alloc((size_t)m * R.kpad));
    REPROJ_TRY(R.Bl.alloc((size_t)m * R.kpad));
    const long long cnt = (long long)m * R.kpad;
    split_matrix<<<(unsigned)((cnt + 255) / 256), 256>>>(m, R.kpad, B.p, R.Bh.p, R.Bl.p);
    REPROJ_TRY(cudaGetLastError());
    if (want_pinv32) {
        DevBuf<int> ord;
        REPROJ_TRY(ord.upload(ctx->h_row_order.data(), ctx->h_row_order.size()));
        REPROJ_TRY(ctx->pinv32.alloc((size_t)m * m));
        const long long mm = (long long)m * m;
        pinv32_kernel<<<(unsigned)((mm + 255) / 256), 256>>>(m, ord.p, B.p, ctx->pinv32.p);
        REPROJ_TRY(cudaGetLastError());
        REPROJ_TRY(cudaDeviceSynchronize());
    }
    REPROJ_TRY(cudaDeviceSynchronize());
    return ACHR_OK;
}

}  // namespace

achr_status ensure_reproj(achr_ctx *ctx) {
    if (ctx->reproj) return ACHR_OK;
    ReprojState *R = new (std::nothrow) ReprojState();
    if (!R) return set_err(ACHR_ERR_NOMEM, "allocation failed");
    const achr_status st = build_reproj(ctx, *R);
    if (st != ACHR_OK) {
        delete R;
        return st;
    }
    ctx->reproj = R;
    return ACHR_OK;
}

namespace {

achr_status ensure_chunk(ReprojState &R, int chunk) {
    if (chunk <= R.chunk_cap) return ACHR_OK;
    R.Rh.reset();
    R.Rl.reset();
    R.Z.reset();
    R.chunk_cap = 0;
    REPROJ_TRY(R.Rh.alloc((size_t)chunk * R.kpad));
    REPROJ_TRY(R.Rl.alloc((size_t)chunk * R.kpad));
    REPROJ_TRY(R.Z.alloc((size_t)R.m * chunk));
    R.chunk_cap = chunk;
    return ACHR_OK;
}

double bits_to_double(unsigned long long b) {
    double v;
    std::memcpy(&v, &b, sizeof v);
    return v;
}

dim3 residual_grid(int P, int kpad) {
    const int nchunks = kpad / kRowChunk;
    return dim3((unsigned)((P + 31) / 32), (unsigned)((nchunks + kResWarps - 1) / kResWarps));
}

}  // namespace

achr_status build_pinv32(achr_ctx *ctx) {
    if (ctx->pinv32.p) return ACHR_OK;
    if ((int)ctx->h_row_order.size() != ctx->m) return set_err(ACHR_ERR_INVALID, "row order missing");
    // Rebuild the operator with the FP32 copy requested (the first build frees B).
    ReprojState *R = new (std::nothrow) ReprojState();
    if (!R) return set_err(ACHR_ERR_NOMEM, "allocation failed");
    const achr_status st = build_reproj(ctx, *R, true);
    if (st != ACHR_OK) {
        delete R;
        return st;
    }
    reproj_free(ctx->reproj);
    ctx->reproj = R;
    return ACHR_OK;
}

}  // namespace achr

using achr::ReprojState;

extern "C" {

achr_status achr_gemm_bf16(int32_t M, int32_t N, int32_t K, int32_t nsplit, const void *A0, const void *A1,
                           int64_t lda, const void *B0, const void *B1, int64_t ldb, float *C, int64_t ldc,
                           void *stream) {
    achr::TcGemm g{M, N, K, nsplit, A0, A1, (long long)lda, B0, B1, (long long)ldb, C, (long long)ldc};
    if (const char *why = achr::tc_gemm_check(g)) return achr::set_err(ACHR_ERR_INVALID, why);
    achr::DevBuf<unsigned long long> err;
    REPROJ_TRY(err.alloc(1));
    REPROJ_TRY(cudaMemsetAsync(err.p, 0, sizeof(unsigned long long), (cudaStream_t)stream));
    REPROJ_TRY(achr::launch_tc_gemm(g, err.p, (cudaStream_t)stream));
    unsigned long long h = 0;
    REPROJ_TRY(cudaMemcpyAsync(&h, err.p, sizeof h, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
    REPROJ_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    if (h) return achr::set_err(ACHR_ERR_TIMEOUT, "a tensor-core pipeline wait expired");
    return ACHR_OK;
}

achr_status achr_reproject_batch(achr_ctx *ctx, int32_t n_points, double *d_points, double *d_centre_acc, int64_t ld,
                                 int32_t max_rounds, void *stream_v, achr_reproj_stats *stats) {
    using namespace achr;
    if (!ctx || !d_points || n_points < 0 || max_rounds < 1 || max_rounds > 16 || ld < n_points)
        return set_err(ACHR_ERR_INVALID, "bad reprojection arguments");
    if (stats) std::memset(stats, 0, sizeof *stats);
    if (n_points == 0 || ctx->m == 0) return ACHR_OK;
    achr_status st = ensure_reproj(ctx);
    if (st != ACHR_OK) return st;
    ReprojState &R = *ctx->reproj;
    const int chunk = std::min(n_points, kMaxChunk);
    st = ensure_chunk(R, chunk);
    if (st != ACHR_OK) return st;
    const int nchunks = (n_points + chunk - 1) / chunk;
    const size_t nflags = 8 + (size_t)max_rounds * nchunks;
    if (R.flags.count < nflags) REPROJ_TRY(R.flags.alloc(nflags));
    cudaStream_t s = (cudaStream_t)stream_v;
    REPROJ_TRY(cudaMemsetAsync(R.flags.p, 0, nflags * sizeof(unsigned long long), s));
    double tol = ctx->opt.residual_tol;
    unsigned long long tol_bits;
    std::memcpy(&tol_bits, &tol, sizeof tol_bits);

    std::vector<cudaEvent_t> ev;  // destroyed on every return below
    struct EvGuard {
        std::vector<cudaEvent_t> &v;
        ~EvGuard() {
            for (cudaEvent_t e : v) cudaEventDestroy(e);
        }
    } ev_guard{ev};
    auto new_event = [&](cudaEvent_t &e) -> bool {
        if (cudaEventCreate(&e) != cudaSuccess) return false;
        ev.push_back(e);
        return true;
    };
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    if (stats) {
        if (!new_event(t0) || !new_event(t1)) return set_err(ACHR_ERR_CUDA, "cudaEventCreate failed");
        REPROJ_TRY(cudaEventRecord(t0, s));
    }
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> gemm_ev;
    std::vector<double> chunk_flops((size_t)nchunks, 0.0);
    // Round r, chunk c: residual + split, then (gated on that chunk's residual
    // exceeding residual_tol) the tensor-core GEMM and the FP64 correction.
    for (int r = 0; r < max_rounds; ++r) {
        for (int c = 0; c < nchunks; ++c) {
            const int c0 = c * chunk;
            const int pc = std::min(chunk, n_points - c0);
            double *X = d_points + c0;
            unsigned long long *slot = R.flags.p + 8 + (size_t)r * nchunks + c;
            const unsigned long long *prev = r > 0 ? slot - nchunks : nullptr;
            residual_kernel<true><<<residual_grid(pc, R.kpad), kResWarps * 32, 0, s>>>(
                R.m, R.kpad, pc, X, ld, R.rp.p, R.ci.p, R.rv.p, R.Rh.p, R.Rl.p, slot, prev, tol_bits);
            REPROJ_TRY(cudaGetLastError());
            TcGemm g{R.m, pc, R.kpad, 3, R.Bh.p, R.Bl.p, (long long)R.kpad, R.Rh.p, R.Rl.p, (long long)R.kpad,
                     R.Z.p, (long long)pc};
            g.gate = slot;
            g.gate_max = tol_bits;
            if (const char *why = tc_gemm_check(g)) return set_err(ACHR_ERR_INVALID, why);
            cudaEvent_t g0 = nullptr, g1 = nullptr;
            if (stats) {
                if (!new_event(g0) || !new_event(g1)) return set_err(ACHR_ERR_CUDA, "cudaEventCreate failed");
                REPROJ_TRY(cudaEventRecord(g0, s));
            }
            REPROJ_TRY(launch_tc_gemm(g, R.flags.p + 2, s));
            if (stats) {
                REPROJ_TRY(cudaEventRecord(g1, s));
                gemm_ev.emplace_back(g0, g1);
            }
            chunk_flops[(size_t)c] = tc_gemm_flops(g);
            const int ny = std::max(1, std::min((R.n + kCorrWarps * 16 - 1) / (kCorrWarps * 16), 65535));
            correct_kernel<<<dim3((unsigned)((pc + 31) / 32), (unsigned)ny), kCorrWarps * 32, 0, s>>>(
                R.n, pc, X, ld, d_centre_acc ? d_centre_acc + c0 : nullptr, ld, R.cp.p, R.ri.p, R.cv.p, R.Z.p,
                (long long)pc, ctx->lbub.p, slot, tol_bits);
            REPROJ_TRY(cudaGetLastError());
        }
    }
    if (stats) {
        residual_kernel<false><<<residual_grid(n_points, R.kpad), kResWarps * 32, 0, s>>>(
            R.m, R.kpad, n_points, d_points, ld, R.rp.p, R.ci.p, R.rv.p, nullptr, nullptr, R.flags.p + 1, nullptr,
            0ull);
        REPROJ_TRY(cudaGetLastError());
        REPROJ_TRY(cudaEventRecord(t1, s));
    }
    std::vector<unsigned long long> h(nflags, 0);
    REPROJ_TRY(cudaMemcpyAsync(h.data(), R.flags.p, nflags * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    REPROJ_TRY(cudaStreamSynchronize(s));
    if (h[2]) return set_err(ACHR_ERR_TIMEOUT, "a tensor-core pipeline wait expired");
    if (stats) {
        float ms = 0.0f;
        double gms = 0.0, flops = 0.0;
        int rounds = 0;
        unsigned long long before = 0;
        for (int c = 0; c < nchunks; ++c) before = std::max(before, h[8 + (size_t)c]);
        for (int r = 0; r < max_rounds; ++r) {
            bool any = false;
            for (int c = 0; c < nchunks; ++c)
                if (h[8 + (size_t)r * nchunks + c] > tol_bits) {
                    any = true;
                    flops += chunk_flops[(size_t)c];
                    if (cudaEventElapsedTime(&ms, gemm_ev[(size_t)r * nchunks + c].first,
                                             gemm_ev[(size_t)r * nchunks + c].second) == cudaSuccess)
                        gms += ms;
                }
            rounds += any ? 1 : 0;
        }
        REPROJ_TRY(cudaEventElapsedTime(&ms, t0, t1));
        stats->residual_before = bits_to_double(before);
        stats->residual_after = bits_to_double(h[1]);
        stats->gemm_ms = gms;
        stats->total_ms = ms;
        stats->gemm_flops = flops;
        stats->rounds = rounds;
        stats->rank = R.rank;
        stats->lambda_min = R.lam_min;
        stats->lambda_max = R.lam_max;
    }
    return ACHR_OK;
}

achr_status achr_sample_periodic(achr_ctx *ctx, uint64_t seed, uint64_t chain_offset, int32_t n_points,
                                 int32_t n_steps, int32_t period, int32_t max_rounds, double *d_points,
                                 double *d_centre_acc, int64_t ld, void *stream, achr_stats *stats,
                                 achr_reproj_stats *rstats) {
    if (!ctx || !d_points || !d_centre_acc || n_points < 0 || n_steps < 0 || period <= 0 || max_rounds < 1 ||
        ld < n_points)
        return achr::set_err(ACHR_ERR_INVALID, "bad periodic-sampling arguments");
    if (stats) std::memset(stats, 0, sizeof *stats);
    if (rstats) std::memset(rstats, 0, sizeof *rstats);
    for (int t0 = 0; t0 < n_steps || (t0 == 0 && n_steps == 0); t0 += period) {
        const int seg = std::min(period, n_steps - t0);
        achr_stats s1;
        achr_status st = achr_sample_resume(ctx, seed, chain_offset, n_points, t0, seg, t0 > 0 ? 1 : 0, d_points,
                                            d_centre_acc, ld, stream, stats ? &s1 : nullptr);
        if (st != ACHR_OK) return st;
        if (stats) {
            stats->accepted += s1.accepted;
            stats->rejected += s1.rejected;
            stats->checks += s1.checks;
            stats->reprojections += s1.reprojections;
            stats->stuck_chains = std::max(stats->stuck_chains, s1.stuck_chains);
            stats->exact_evals += s1.exact_evals;
            stats->final_projections += s1.final_projections;
            stats->max_bound_violation = std::max(stats->max_bound_violation, s1.max_bound_violation);
            stats->max_residual = s1.max_residual;
            stats->kernel_ms += s1.kernel_ms;
        }
        if (n_steps == 0) break;
        achr_reproj_stats r1;
        st = achr_reproject_batch(ctx, n_points, d_points, d_centre_acc, ld, max_rounds, stream,
                                  rstats ? &r1 : nullptr);
        if (st != ACHR_OK) return st;
        if (rstats) {
            rstats->residual_before = std::max(rstats->residual_before, r1.residual_before);
            rstats->residual_after = std::max(rstats->residual_after, r1.residual_after);
            rstats->gemm_ms += r1.gemm_ms;
            rstats->total_ms += r1.total_ms;
            rstats->gemm_flops += r1.gemm_flops;
            rstats->rounds += r1.rounds;
            rstats->rank = r1.rank;
            rstats->lambda_min = r1.lambda_min;
            rstats->lambda_max = r1.lambda_max;
        }
        if (stats && rstats) stats->max_residual = r1.residual_after;  // the emitted points are the reprojected ones
    }
    return ACHR_OK;
}

}  // extern "C"
