// Learned direction preconditioner: a low-rank-plus-diagonal linear map in
// the coordinates of the directions the polytope spans (the null space of S
// with the reactions pinned in every warmup point held fixed), fitted on the GPU to samples of the plain sampler,
// and the pool of hit-and-run directions it generates.  No reference
// counterpart (the reference's only direction rule is ACHR's, ACHRcu/
// ACHRCuda.cu:260-264).
//
// Model.  Directions u = N L z, z ~ N(0, I), with L = [diag(exp(s)), U]
// (d x (d + r)), so the direction covariance in null-space coordinates is
//     C = L L^T = D + U U^T,   D = diag(exp(2 s)).
// It is fitted to samples y = N^T (x - mu) by the Gaussian KL loss
//     loss = 1/2 tr(C^-1 Sigma_b) + 1/2 log det C      (KL up to a constant),
// Sigma_b the covariance of a minibatch of B samples, using
//     A = D^-1, W = A U, M = I + U^T W (r x r),  C^-1 = A - W M^-1 W^T,
//     log det C = 2 sum s + log det M,
// and the gradients (V = C^-1 Y_b, K = C^-1 U = W M^-1)
//     dloss/dU = K - V (V^T U) / B,
//     dloss/ds_i = D_i (A_i - sum_j K_ij W_ij - sum_b V_ib^2 / B).
// Every step is a kernel of this file: FP32 tiled GEMMs, a single-CTA
// Cholesky factorisation and inverse of M, row reductions, Adam.
#include <cublas_v2.h>
#include <cusolverDn.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "achr_ctx.h"
#include "achr_rng.cuh"

extern "C" void achr_io_set_error(const char *msg);

namespace achr {
namespace {

achr_status pc_err(achr_status st, const std::string &msg) {
    achr_io_set_error(msg.c_str());
    return st;
}

#define PC_TRY(expr)                                                                              \
    do {                                                                                          \
        cudaError_t e_ = (expr);                                                                  \
        if (e_ != cudaSuccess) return pc_err(ACHR_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// ---------------------------------------------------------------------------
// FP32 GEMM with arbitrary strides:  C = alpha * op(A) op(B) + beta * C,
// op(A)(i, k) = A[i * sai + k * sak], op(B)(k, j) = B[k * sbk + j * sbj],
// C(i, j) = C[i * ldc + j].  64 x 64 tiles, 256 threads, 4 x 4 per thread.
constexpr int kT = 64, kTK = 16;

__global__ void __launch_bounds__(256)
    sgemm_kernel(int M, int N, int K, float alpha, const float *__restrict__ A, long long sai, long long sak,
                 const float *__restrict__ B, long long sbk, long long sbj, float beta, float *__restrict__ C,
                 long long ldc) {
    __shared__ float As[kTK][kT + 4];
    __shared__ float Bs[kTK][kT + 4];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int i0 = blockIdx.y * kT, j0 = blockIdx.x * kT;
    float acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += kTK) {
        // Each operand's tile is loaded with consecutive threads on its
        // contiguous index (k when the stride along k is 1, else the row index).
        for (int t = threadIdx.x; t < kT * kTK; t += 256) {
            const int ii = (sak == 1) ? t / kTK : t % kT, kk = (sak == 1) ? t % kTK : t / kT;
            const int i = i0 + ii, k = k0 + kk;
            As[kk][ii] = (i < M && k < K) ? A[(long long)i * sai + (long long)k * sak] : 0.0f;
        }
        for (int t = threadIdx.x; t < kT * kTK; t += 256) {
            const int jj = (sbk == 1) ? t / kTK : t % kT, kk = (sbk == 1) ? t % kTK : t / kT;
            const int j = j0 + jj, k = k0 + kk;
            Bs[kk][jj] = (j < N && k < K) ? B[(long long)k * sbk + (long long)j * sbj] : 0.0f;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kTK; ++kk) {
            float a[4], b[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                a[q] = As[kk][ty + 16 * q];
                b[q] = Bs[kk][tx + 16 * q];
            }
#pragma unroll
            for (int p = 0; p < 4; ++p)
#pragma unroll
                for (int q = 0; q < 4; ++q) acc[p][q] = fmaf(a[p], b[q], acc[p][q]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int p = 0; p < 4; ++p) {
        const int i = i0 + ty + 16 * p;
        if (i >= M) continue;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int j = j0 + tx + 16 * q;
            if (j >= N) continue;
            float *c = C + (long long)i * ldc + j;
            *c = alpha * acc[p][q] + (beta != 0.0f ? beta * *c : 0.0f);
        }
    }
}

cudaError_t sgemm(cudaStream_t s, int M, int N, int K, float alpha, const float *A, long long sai, long long sak,
                  const float *B, long long sbk, long long sbj, float beta, float *C, long long ldc) {
    if (M <= 0 || N <= 0) return cudaSuccess;
    dim3 grid((unsigned)((N + kT - 1) / kT), (unsigned)((M + kT - 1) / kT));
    sgemm_kernel<<<grid, 256, 0, s>>>(M, N, K, alpha, A, sai, sak, B, sbk, sbj, beta, C, ldc);
    return cudaGetLastError();
}

// a = exp(-2 s), W = a * U (row scale), and M = I (the GEMM adds U^T W).
__global__ void prep_kernel(int d, int r, const float *__restrict__ s, const float *__restrict__ U,
                            float *__restrict__ a, float *__restrict__ W, float *__restrict__ M) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < (long long)d * r) {
        const int i = (int)(t / r);
        W[t] = expf(-2.0f * s[i]) * U[t];
    }
    if (t < d) a[t] = expf(-2.0f * s[t]);
    if (t < (long long)r * r) M[t] = ((int)(t / r) == (int)(t % r)) ? 1.0f : 0.0f;
}

// Cholesky factorisation M = L L^T (r x r, in place in Lw), log det M, and
// Minv = L^-T L^-1.  One CTA; the factorisation is right-looking with a
// barrier per column.  A non-positive pivot sets *bad.
__global__ void __launch_bounds__(1024)
    chol_inv_kernel(int r, const float *__restrict__ M, float *__restrict__ Lw, float *__restrict__ Xw,
                    float *__restrict__ Minv, float *__restrict__ logdet, int *__restrict__ bad) {
    const int tid = threadIdx.x, nt = blockDim.x;
    __shared__ float piv;
    __shared__ float red[32];
    for (int t = tid; t < r * r; t += nt) Lw[t] = M[t];
    __syncthreads();
    for (int k = 0; k < r; ++k) {
        if (tid == 0) {
            float dkk = Lw[k * r + k];
            if (!(dkk > 0.0f)) {
                *bad = 1;
                dkk = 1.0f;
            }
            piv = sqrtf(dkk);
            Lw[k * r + k] = piv;
        }
        __syncthreads();
        const float lkk = piv;
        for (int i = k + 1 + tid; i < r; i += nt) Lw[i * r + k] /= lkk;
        __syncthreads();
        const int nt2 = r - k - 1;
        for (int t = tid; t < nt2 * nt2; t += nt) {
            const int i = k + 1 + t / nt2, j = k + 1 + t % nt2;
            if (j <= i) Lw[i * r + j] -= Lw[i * r + k] * Lw[j * r + k];
        }
        __syncthreads();
    }
    float ld = 0.0f;
    for (int k = tid; k < r; k += nt) ld += logf(Lw[k * r + k]);
    for (int o = 16; o; o >>= 1) ld += __shfl_xor_sync(0xffffffffu, ld, o);
    if ((tid & 31) == 0) red[tid >> 5] = ld;
    __syncthreads();
    if (tid == 0) {
        float t = 0.0f;
        for (int w = 0; w < (nt + 31) / 32; ++w) t += red[w];
        *logdet = 2.0f * t;
    }
    // X = L^-1 (lower): column c by forward substitution, one thread per column.
    for (int c = tid; c < r; c += nt) {
        for (int i = 0; i < c; ++i) Xw[i * r + c] = 0.0f;
        for (int i = c; i < r; ++i) {
            float acc = (i == c) ? 1.0f : 0.0f;
            for (int k = c; k < i; ++k) acc -= Lw[i * r + k] * Xw[k * r + c];
            Xw[i * r + c] = acc / Lw[i * r + i];
        }
    }
    __syncthreads();
    // Minv = X^T X
    for (int t = tid; t < r * r; t += nt) {
        const int a = t / r, b = t % r;
        float acc = 0.0f;
        for (int i = max(a, b); i < r; ++i) acc = fmaf(Xw[i * r + a], Xw[i * r + b], acc);
        Minv[t] = acc;
    }
}

// Per null-space coordinate i (one warp each): V_i. += a_i Y_i. (V holds
// -W Rq on entry), the loss terms sum_b Y_ib V_ib, and the gradient of s_i.
__global__ void rows_kernel(int d, int r, int B, const float *__restrict__ Y, long long ldy,
                            const float *__restrict__ a, const float *__restrict__ s, float *__restrict__ V,
                            const float *__restrict__ K, const float *__restrict__ W, float *__restrict__ gs,
                            float *__restrict__ yv) {
    const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (i >= d) return;
    const float ai = a[i];
    float syv = 0.0f, svv = 0.0f, skw = 0.0f;
    for (int b = lane; b < B; b += 32) {
        const float y = Y[(long long)i * ldy + b];
        const float v = fmaf(ai, y, V[(long long)i * B + b]);
        V[(long long)i * B + b] = v;
        syv = fmaf(y, v, syv);
        svv = fmaf(v, v, svv);
    }
    for (int j = lane; j < r; j += 32) skw = fmaf(K[(long long)i * r + j], W[(long long)i * r + j], skw);
    for (int o = 16; o; o >>= 1) {
        syv += __shfl_xor_sync(0xffffffffu, syv, o);
        svv += __shfl_xor_sync(0xffffffffu, svv, o);
        skw += __shfl_xor_sync(0xffffffffu, skw, o);
    }
    if (lane == 0) {
        const float Di = expf(2.0f * s[i]);
        gs[i] = Di * (ai - skw - svv / (float)B);
        yv[i] = syv;
    }
}

// loss = 1/2 (sum_i yv_i / B + 2 sum_i s_i + logdet M), fixed summation order.
__global__ void loss_kernel(int d, int B, const float *__restrict__ yv, const float *__restrict__ s,
                            const float *__restrict__ logdet, float *__restrict__ loss) {
    __shared__ double red[32];
    double acc = 0.0;
    for (int i = threadIdx.x; i < d; i += blockDim.x) acc += (double)yv[i] / (double)B + 2.0 * (double)s[i];
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        *loss = (float)(0.5 * (t + (double)*logdet));
    }
}

__global__ void adam_kernel(long long n, float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                            float *__restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const float gi = g[t];
    const float mi = b1 * m[t] + (1.0f - b1) * gi;
    const float vi = b2 * v[t] + (1.0f - b2) * gi * gi;
    m[t] = mi;
    v[t] = vi;
    p[t] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// Root mean square of every row of Y (d x ns, leading dimension ldy): the
// per-coordinate scale of centred samples.  One warp per row.
__global__ void row_rms_kernel(int d, int ns, const float *__restrict__ Y, long long ldy, float *__restrict__ sig) {
    const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (i >= d) return;
    double acc = 0.0;
    for (int b = lane; b < ns; b += 32) {
        const double y = Y[(long long)i * ldy + b];
        acc += y * y;
    }
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) sig[i] = (float)fmax(sqrt(acc / (double)ns), 1e-30);
}

// Ys = Y / sig (rows), into a dense d x ns buffer.
__global__ void scale_rows_kernel(int d, int ns, const float *__restrict__ Y, long long ldy,
                                  const float *__restrict__ sig, float *__restrict__ Ys) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)d * ns) return;
    const int i = (int)(t / ns), b = (int)(t % ns);
    Ys[t] = Y[(long long)i * ldy + b] / sig[i];
}

// Parameters between original and standardised coordinates (y = sig * ys):
// forward s -= log sig, U /= sig; backward s += log sig, U *= sig.
__global__ void rescale_params_kernel(int d, int r, const float *__restrict__ sig, float *__restrict__ s,
                                      float *__restrict__ U, int forward) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < (long long)d * r) {
        const int i = (int)(t / r);
        U[t] = forward ? U[t] / sig[i] : U[t] * sig[i];
    }
    if (t < d) s[t] += forward ? -logf(sig[t]) : logf(sig[t]);
}

__global__ void f32_to_f64_scaled_kernel(long long n, const float *__restrict__ in, double scale,
                                         double *__restrict__ out) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) out[t] = scale * (double)in[t];
}

// Probabilistic-PCA start (the maximum-likelihood C = sigma^2 I + U U^T):
// with eigenpairs (lam ascending, V column-major) of the sample covariance,
// U = V_top (lam_top - sigma^2)^1/2, sigma^2 = mean of the other eigenvalues.
__global__ void ppca_init_kernel(int d, int r, const double *__restrict__ V, const double *__restrict__ lam,
                                 double sigma2, float *__restrict__ s, float *__restrict__ U) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < (long long)d * r) {
        const int i = (int)(t / r), j = (int)(t % r);
        const int col = d - r + j;
        U[t] = (float)(V[(long long)col * d + i] * sqrt(fmax(lam[col] - sigma2, 0.0)));
    }
    if (t < d) s[t] = (float)(0.5 * log(sigma2));
}

// Square root of a covariance from its eigenpairs (lam ascending, V column-major):
// Y (d x d, row-major) = V diag(sqrt(max(lam, 0) * d)), so Y Y^T / d = V diag(lam) V^T.
__global__ void cov_sqrt_kernel(int d, const double *__restrict__ V, const double *__restrict__ lam,
                                float *__restrict__ Y) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)d * d) return;
    const int i = (int)(t / d), k = (int)(t % d);
    Y[t] = (float)(V[(long long)k * d + i] * sqrt(fmax(lam[k], 0.0) * (double)d));
}

// Standard normal (Box-Muller on two 32-bit Philox words) for entry (row, col).
__device__ __forceinline__ float philox_normal(unsigned long long seed, unsigned row, unsigned col, unsigned tag) {
    const Philox4 w = philox4x32_10(row, col, tag, 0x6e6f726du, (uint32_t)seed, (uint32_t)(seed >> 32));
    const float u1 = ((float)(w.v[0] >> 8) + 0.5f) * (1.0f / 16777216.0f);
    const float u2 = ((float)(w.v[1] >> 8) + 0.5f) * (1.0f / 16777216.0f);
    return sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
}

// Yp (d x K) = exp(s) * Z1; Z2 (r x K) for the low-rank part.
__global__ void pool_noise_kernel(int d, int r, int K, unsigned long long seed, const float *__restrict__ s,
                                  float *__restrict__ Yp, float *__restrict__ Z2) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < (long long)d * K) {
        const int i = (int)(t / K), c = (int)(t % K);
        Yp[t] = expf(s[i]) * philox_normal(seed, (unsigned)i, (unsigned)c, 1u);
    }
    if (t < (long long)r * K) {
        const int j = (int)(t / K), c = (int)(t % K);
        Z2[t] = philox_normal(seed, (unsigned)j, (unsigned)c, 2u);
    }
}

__global__ void f32_to_f64_kernel(long long n, const float *__restrict__ in, double *__restrict__ out) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) out[t] = (double)in[t];
}

// N (n x d, column-major FP64) -> BF16 hi/lo rows of N^T (d x kpad, K = reaction).
__global__ void split_nt_kernel(int n, int d, int kpad, const double *__restrict__ N, __nv_bfloat16 *__restrict__ Nh,
                                __nv_bfloat16 *__restrict__ Nl) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)d * kpad) return;
    const int j = (int)(t / kpad), i = (int)(t % kpad);
    const double v = i < n ? N[(long long)j * n + i] : 0.0;
    const __nv_bfloat16 hi = __double2bfloat16(v);
    Nh[t] = hi;
    Nl[t] = __double2bfloat16(v - (double)__bfloat162float(hi));
}

// (x - mu) for 32 chains x 64 reactions per warp, transposed through shared
// memory into chain-major BF16 hi/lo rows (K = reaction contiguous).
constexpr int kSplitWarps = 4, kSplitStride = 72;
__global__ void __launch_bounds__(kSplitWarps * 32)
    split_points_kernel(int n, int kpad, int P, const double *__restrict__ X, long long ldx,
                        const double *__restrict__ mu, __nv_bfloat16 *__restrict__ Xh, __nv_bfloat16 *__restrict__ Xl) {
    __shared__ __align__(16) __nv_bfloat16 stage[kSplitWarps][2][32 * kSplitStride];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int p0 = blockIdx.x * 32, p = p0 + lane;
    const bool live = p < P;
    const int nchunks = kpad / 64;
    for (int c = blockIdx.y * kSplitWarps + warp; c < nchunks; c += gridDim.y * kSplitWarps) {
        for (int r = 0; r < 64; ++r) {
            const int i = c * 64 + r;
            double v = 0.0;
            if (live && i < n) v = X[(long long)i * ldx + p] - (mu ? mu[i] : 0.0);
            const __nv_bfloat16 hi = __double2bfloat16(v);
            stage[warp][0][lane * kSplitStride + r] = hi;
            stage[warp][1][lane * kSplitStride + r] = __double2bfloat16(v - (double)__bfloat162float(hi));
        }
        __syncwarp();
        for (int t = lane; t < 32 * 8; t += 32) {
            const int row = t / 8, part = t % 8;
            if (p0 + row < P) {
                const size_t off = (size_t)(p0 + row) * (size_t)kpad + (size_t)c * 64 + (size_t)part * 8;
                *reinterpret_cast<uint4 *>(Xh + off) =
                    *reinterpret_cast<const uint4 *>(&stage[warp][0][row * kSplitStride + part * 8]);
                *reinterpret_cast<uint4 *>(Xl + off) =
                    *reinterpret_cast<const uint4 *>(&stage[warp][1][row * kSplitStride + part * 8]);
            }
        }
        __syncwarp();
    }
}

unsigned blocks_for(long long n, int t = 256) { return (unsigned)((n + t - 1) / t); }

// Reactions whose value is the same in every warmup point (to 1e-9 relative):
// implicit equalities of the polytope (blocked or pinned fluxes).  One thread
// per reaction, coalesced over reactions.
__global__ void frozen_kernel(int n, int W, int ldw, const double *__restrict__ warmup, int *__restrict__ frozen) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double lo = INFINITY, hi = -INFINITY;
    for (int j = 0; j < W; ++j) {
        const double v = warmup[(long long)j * ldw + i];
        lo = fmin(lo, v);
        hi = fmax(hi, v);
    }
    frozen[i] = (hi - lo) <= 1e-9 * fmax(1.0, fmax(fabs(lo), fabs(hi))) ? 1 : 0;
}

__global__ void add_diag_kernel(int n, const int *__restrict__ frozen, double *__restrict__ G) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && frozen[i]) G[(long long)i * n + i] += 1.0;
}

// The basis the preconditioner works in: null space of [S; E], E the unit rows
// of the frozen reactions, by the reference's eigenvalue rule on
// S^T S + E^T E (ACHRCuda.cu:436-502 applied to the stacked matrix).
achr_status ensure_active_basis(achr_ctx *ctx) {
    if (ctx->d_act >= 0) return ACHR_OK;
    const int n = ctx->n, m = ctx->m;
    DevBuf<int> frozen, info;
    PC_TRY(frozen.alloc(n));
    frozen_kernel<<<blocks_for(n), 256>>>(n, ctx->W, ctx->ldw, ctx->warmup.p, frozen.p);
    PC_TRY(cudaGetLastError());
    std::vector<int> hf((size_t)n);
    PC_TRY(cudaMemcpy(hf.data(), frozen.p, sizeof(int) * n, cudaMemcpyDeviceToHost));
    int nf = 0;
    for (int v : hf) nf += v;
    if (nf == 0) {  // nothing pinned: the null space itself
        PC_TRY(ctx->Nact.alloc((size_t)n * std::max(ctx->d, 1)));
        if (ctx->d > 0)
            PC_TRY(cudaMemcpy(ctx->Nact.p, ctx->N.p, sizeof(double) * (size_t)n * ctx->d, cudaMemcpyDeviceToDevice));
        ctx->d_act = ctx->d;
        ctx->n_frozen = 0;
        return ACHR_OK;
    }
    std::vector<double> dS((size_t)m * n, 0.0);
    for (int i = 0; i < m; ++i)
        for (int q = ctx->h_rowptr[(size_t)i]; q < ctx->h_rowptr[(size_t)i + 1]; ++q)
            dS[(size_t)ctx->h_colidx[(size_t)q] * m + i] = ctx->h_val[(size_t)q];
    DevBuf<double> S, G, lam, work;
    PC_TRY(S.upload(dS.data(), dS.size()));
    PC_TRY(G.alloc((size_t)n * n));
    PC_TRY(lam.alloc(n));
    PC_TRY(info.alloc(1));
    cublasHandle_t cb = nullptr;
    if (cublasCreate(&cb) != CUBLAS_STATUS_SUCCESS) return pc_err(ACHR_ERR_CUDA, "cublasCreate failed");
    const double one = 1.0, zero = 0.0;
    const cublasStatus_t bs =
        m > 0 ? cublasDgemm(cb, CUBLAS_OP_T, CUBLAS_OP_N, n, n, m, &one, S.p, m, S.p, m, &zero, G.p, n)
              : CUBLAS_STATUS_SUCCESS;
    cublasDestroy(cb);
    if (bs != CUBLAS_STATUS_SUCCESS) return pc_err(ACHR_ERR_CUDA, "cublasDgemm (S^T S) failed");
    if (m == 0) PC_TRY(cudaMemset(G.p, 0, sizeof(double) * (size_t)n * n));
    add_diag_kernel<<<blocks_for(n), 256>>>(n, frozen.p, G.p);
    PC_TRY(cudaGetLastError());
    cusolverDnHandle_t sh = nullptr;
    if (cusolverDnCreate(&sh) != CUSOLVER_STATUS_SUCCESS) return pc_err(ACHR_ERR_CUDA, "cusolverDnCreate failed");
    int lwork = 0;
    cusolverStatus_t ss =
        cusolverDnDsyevd_bufferSize(sh, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, G.p, n, lam.p, &lwork);
    if (ss == CUSOLVER_STATUS_SUCCESS) {
        if (cudaError_t e = work.alloc((size_t)std::max(lwork, 1))) {
            cusolverDnDestroy(sh);
            return pc_err(ACHR_ERR_CUDA, std::string("syevd workspace: ") + cudaGetErrorString(e));
        }
        ss = cusolverDnDsyevd(sh, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, G.p, n, lam.p, work.p, lwork,
                              info.p);
    }
    cusolverDnDestroy(sh);
    if (ss != CUSOLVER_STATUS_SUCCESS) return pc_err(ACHR_ERR_NUMERIC, "cusolverDnDsyevd (active basis) failed");
    int h_info = 0;
    PC_TRY(cudaMemcpy(&h_info, info.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (h_info != 0) return pc_err(ACHR_ERR_NUMERIC, "syevd (active basis) did not converge");
    std::vector<double> hl((size_t)n);
    PC_TRY(cudaMemcpy(hl.data(), lam.p, sizeof(double) * n, cudaMemcpyDeviceToHost));
    double smax = 0.0;
    for (double v : hl) smax = std::max(smax, std::fabs(v));
    const double tol = (double)n * smax * 2.2204e-16;
    int d = 0;  // eigenvalues ascend: the basis is the leading block of columns
    while (d < n && std::fabs(hl[(size_t)d]) < tol) ++d;
    PC_TRY(ctx->Nact.alloc((size_t)n * std::max(d, 1)));
    if (d > 0) PC_TRY(cudaMemcpy(ctx->Nact.p, G.p, sizeof(double) * (size_t)n * d, cudaMemcpyDeviceToDevice));
    ctx->d_act = d;
    ctx->n_frozen = nf;
    return ACHR_OK;
}

// Device workspace of one loss/gradient evaluation.
struct PcWork {
    DevBuf<float> a, W, M, Lw, Xw, Minv, Q, Rq, V, K, T, yv, scal;  // scal: [0] logdet, [1] loss
    DevBuf<int> bad;
    cudaError_t alloc(int d, int r, int B) {
        cudaError_t e;
        if ((e = a.alloc(d)) || (e = W.alloc((size_t)d * r)) || (e = M.alloc((size_t)r * r)) ||
            (e = Lw.alloc((size_t)r * r)) || (e = Xw.alloc((size_t)r * r)) || (e = Minv.alloc((size_t)r * r)) ||
            (e = Q.alloc((size_t)r * B)) || (e = Rq.alloc((size_t)r * B)) || (e = V.alloc((size_t)d * B)) ||
            (e = K.alloc((size_t)d * r)) || (e = T.alloc((size_t)B * r)) || (e = yv.alloc(d)) || (e = scal.alloc(2)) ||
            (e = bad.alloc(1)))
            return e;
        return cudaMemset(bad.p, 0, sizeof(int));
    }
};

// Loss and gradients for the minibatch Y (d x B, leading dimension ldy).
cudaError_t loss_grad(cudaStream_t st, int d, int r, int B, const float *s, const float *U, const float *Y,
                      long long ldy, PcWork &w, float *gs, float *gU) {
    cudaError_t e;
    const long long big = std::max<long long>((long long)d * r, std::max<long long>(d, (long long)r * r));
    prep_kernel<<<blocks_for(big), 256, 0, st>>>(d, r, s, U, w.a.p, w.W.p, w.M.p);
    if ((e = cudaGetLastError())) return e;
    // M = I + U^T W
    if ((e = sgemm(st, r, r, d, 1.0f, U, 1, r, w.W.p, r, 1, 1.0f, w.M.p, r))) return e;
    chol_inv_kernel<<<1, 1024, 0, st>>>(r, w.M.p, w.Lw.p, w.Xw.p, w.Minv.p, w.scal.p, w.bad.p);
    if ((e = cudaGetLastError())) return e;
    // Q = W^T Y (r x B); Rq = Minv Q; V = -W Rq (d x B)
    if ((e = sgemm(st, r, B, d, 1.0f, w.W.p, 1, r, Y, ldy, 1, 0.0f, w.Q.p, B))) return e;
    if ((e = sgemm(st, r, B, r, 1.0f, w.Minv.p, r, 1, w.Q.p, B, 1, 0.0f, w.Rq.p, B))) return e;
    if ((e = sgemm(st, d, B, r, -1.0f, w.W.p, r, 1, w.Rq.p, B, 1, 0.0f, w.V.p, B))) return e;
    // K = W Minv (d x r)
    if ((e = sgemm(st, d, r, r, 1.0f, w.W.p, r, 1, w.Minv.p, r, 1, 0.0f, w.K.p, r))) return e;
    // V += a Y; per-row loss terms and ds
    rows_kernel<<<blocks_for(d, 8), 256, 0, st>>>(d, r, B, Y, ldy, w.a.p, s, w.V.p, w.K.p, w.W.p, gs, w.yv.p);
    if ((e = cudaGetLastError())) return e;
    loss_kernel<<<1, 1024, 0, st>>>(d, B, w.yv.p, s, w.scal.p, w.scal.p + 1);
    if ((e = cudaGetLastError())) return e;
    // T = V^T U (B x r);  gU = K - V T / B
    if ((e = sgemm(st, B, r, d, 1.0f, w.V.p, 1, B, U, r, 1, 0.0f, w.T.p, r))) return e;
    if ((e = cudaMemcpyAsync(gU, w.K.p, sizeof(float) * (size_t)d * r, cudaMemcpyDeviceToDevice, st))) return e;
    return sgemm(st, d, r, B, -1.0f / (float)B, w.V.p, B, 1, w.T.p, r, 1, 1.0f, gU, r);
}

}  // namespace
}  // namespace achr

extern "C" {

void achr_precond_default_options(achr_precond_options *opt) {
    if (!opt) return;
    std::memset(opt, 0, sizeof *opt);
    opt->iterations = 2000;
    opt->batch = 4096;
    opt->learning_rate = 0.01f;
    opt->beta1 = 0.9f;
    opt->beta2 = 0.999f;
    opt->eps = 1e-8f;
    opt->seed = 1;
    opt->init = 1;
    opt->standardize = 1;
    opt->full_batch = 1;
}

achr_status achr_precond_loss_grad(int32_t d, int32_t r, int32_t B, const float *d_s, const float *d_U,
                                   const float *d_Y, int64_t ldy, float *loss_out, float *d_gs, float *d_gU,
                                   void *stream) {
    using namespace achr;
    if (d <= 0 || r <= 0 || r > 1024 || B <= 0 || !d_s || !d_U || !d_Y || ldy < B || !d_gs || !d_gU)
        return pc_err(ACHR_ERR_INVALID, "bad preconditioner arguments");
    cudaStream_t st = (cudaStream_t)stream;
    PcWork w;
    PC_TRY(w.alloc(d, r, B));
    PC_TRY(loss_grad(st, d, r, B, d_s, d_U, d_Y, ldy, w, d_gs, d_gU));
    float h[2];
    int bad = 0;
    PC_TRY(cudaMemcpyAsync(h, w.scal.p, sizeof h, cudaMemcpyDeviceToHost, st));
    PC_TRY(cudaMemcpyAsync(&bad, w.bad.p, sizeof bad, cudaMemcpyDeviceToHost, st));
    PC_TRY(cudaStreamSynchronize(st));
    if (bad) return pc_err(ACHR_ERR_NUMERIC, "I + U^T D^-1 U is not positive definite");
    if (loss_out) *loss_out = h[1];
    return ACHR_OK;
}

achr_status achr_precond_train(int32_t d, int32_t r, int32_t n_samples, const float *d_Y, int64_t ldy,
                               const achr_precond_options *opt, float *d_s, float *d_U, void *stream,
                               achr_precond_stats *stats) {
    using namespace achr;
    if (!opt || d <= 0 || r <= 0 || r > 1024 || !d_Y || !d_s || !d_U || n_samples <= 0 || ldy < n_samples ||
        (!opt->full_batch && (opt->batch <= 0 || opt->batch > n_samples)) || opt->iterations < 0 ||
        (opt->full_batch != 0 && opt->full_batch != 1))
        return pc_err(ACHR_ERR_INVALID, "bad preconditioner training arguments");
    if (opt->init && r >= d) return pc_err(ACHR_ERR_INVALID, "the PCA start needs rank < d");
    cudaStream_t st = (cudaStream_t)stream;
    const bool full = opt->full_batch != 0;
    const int B = full ? d : opt->batch;
    DevBuf<float> Yfull;  // full_batch: d columns with the samples' covariance
    // Standardised coordinates: every coordinate scaled to unit RMS, so one
    // learning rate suits coordinates whose spreads differ by orders of magnitude.
    DevBuf<float> sig, Ys;
    const float *Yt = d_Y;
    long long ldt = ldy;
    if (opt->standardize || opt->init) {
        PC_TRY(sig.alloc(d));
        row_rms_kernel<<<blocks_for(d, 8), 256, 0, st>>>(d, n_samples, d_Y, ldy, sig.p);
        PC_TRY(cudaGetLastError());
        if (opt->standardize) {
            PC_TRY(Ys.alloc((size_t)d * n_samples));
            scale_rows_kernel<<<blocks_for((long long)d * n_samples), 256, 0, st>>>(d, n_samples, d_Y, ldy, sig.p,
                                                                                  Ys.p);
            PC_TRY(cudaGetLastError());
            Yt = Ys.p;
            ldt = n_samples;
        }
    }
    if (opt->init || full) {
        // sample covariance of the (standardised) samples, its eigenpairs in FP64
        DevBuf<float> Sig;
        DevBuf<double> Sd, lam, work;
        DevBuf<int> info;
        PC_TRY(Sig.alloc((size_t)d * d));
        PC_TRY(sgemm(st, d, d, n_samples, 1.0f, Yt, ldt, 1, Yt, 1, ldt, 0.0f, Sig.p, d));
        PC_TRY(Sd.alloc((size_t)d * d));
        f32_to_f64_scaled_kernel<<<blocks_for((long long)d * d), 256, 0, st>>>((long long)d * d, Sig.p,
                                                                              1.0 / (double)n_samples, Sd.p);
        PC_TRY(cudaGetLastError());
        PC_TRY(lam.alloc(d));
        PC_TRY(info.alloc(1));
        cusolverDnHandle_t sh = nullptr;
        if (cusolverDnCreate(&sh) != CUSOLVER_STATUS_SUCCESS) return pc_err(ACHR_ERR_CUDA, "cusolverDnCreate failed");
        cusolverDnSetStream(sh, st);
        int lwork = 0;
        cusolverStatus_t ss =
            cusolverDnDsyevd_bufferSize(sh, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, d, Sd.p, d, lam.p, &lwork);
        if (ss == CUSOLVER_STATUS_SUCCESS) {
            if (cudaError_t e = work.alloc((size_t)std::max(lwork, 1))) {
                cusolverDnDestroy(sh);
                return pc_err(ACHR_ERR_CUDA, std::string("syevd workspace: ") + cudaGetErrorString(e));
            }
            ss = cusolverDnDsyevd(sh, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, d, Sd.p, d, lam.p, work.p,
                                  lwork, info.p);
        }
        cusolverDnDestroy(sh);
        if (ss != CUSOLVER_STATUS_SUCCESS) return pc_err(ACHR_ERR_NUMERIC, "syevd of the sample covariance failed");
        std::vector<double> hl((size_t)d);
        PC_TRY(cudaMemcpyAsync(hl.data(), lam.p, sizeof(double) * d, cudaMemcpyDeviceToHost, st));
        PC_TRY(cudaStreamSynchronize(st));
        if (full) {  // the training data from here on: the covariance's square root
            PC_TRY(Yfull.alloc((size_t)d * d));
            cov_sqrt_kernel<<<blocks_for((long long)d * d), 256, 0, st>>>(d, Sd.p, lam.p, Yfull.p);
            PC_TRY(cudaGetLastError());
        }
        if (opt->init) {
            double sigma2 = 0.0;
            for (int k = 0; k < d - r; ++k) sigma2 += std::max(hl[(size_t)k], 0.0);
            sigma2 = std::max(sigma2 / (double)(d - r), 1e-12 * std::max(hl.back(), 1e-300));
            ppca_init_kernel<<<blocks_for((long long)d * r), 256, 0, st>>>(d, r, Sd.p, lam.p, sigma2, d_s, d_U);
            PC_TRY(cudaGetLastError());
            if (!opt->standardize)  // the start is in standardised units: bring it back
                rescale_params_kernel<<<blocks_for((long long)d * r), 256, 0, st>>>(d, r, sig.p, d_s, d_U, 0);
        } else if (opt->standardize) {
            rescale_params_kernel<<<blocks_for((long long)d * r), 256, 0, st>>>(d, r, sig.p, d_s, d_U, 1);
        }
    } else if (opt->standardize) {
        rescale_params_kernel<<<blocks_for((long long)d * r), 256, 0, st>>>(d, r, sig.p, d_s, d_U, 1);
    }
    PC_TRY(cudaGetLastError());
    PcWork w;
    PC_TRY(w.alloc(d, r, B));
    DevBuf<float> gs, gU, ms, vs, mU, vU, losses;
    PC_TRY(gs.alloc(d));
    PC_TRY(gU.alloc((size_t)d * r));
    PC_TRY(ms.alloc(d));
    PC_TRY(vs.alloc(d));
    PC_TRY(mU.alloc((size_t)d * r));
    PC_TRY(vU.alloc((size_t)d * r));
    const int iters = opt->iterations;
    PC_TRY(losses.alloc((size_t)std::max(iters, 1)));
    PC_TRY(cudaMemsetAsync(ms.p, 0, sizeof(float) * d, st));
    PC_TRY(cudaMemsetAsync(vs.p, 0, sizeof(float) * d, st));
    PC_TRY(cudaMemsetAsync(mU.p, 0, sizeof(float) * (size_t)d * r, st));
    PC_TRY(cudaMemsetAsync(vU.p, 0, sizeof(float) * (size_t)d * r, st));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    PC_TRY(cudaEventCreate(&e0));
    PC_TRY(cudaEventCreate(&e1));
    struct EvG {
        cudaEvent_t a, b;
        ~EvG() {
            cudaEventDestroy(a);
            cudaEventDestroy(b);
        }
    } evg{e0, e1};
    PC_TRY(cudaEventRecord(e0, st));
    if (full) {
        Yt = Yfull.p;
        ldt = d;
    }
    const int nb = full ? 1 : n_samples / B;  // minibatches: consecutive blocks of B samples, in a seeded order
    std::vector<int> order((size_t)nb);
    for (int q = 0; q < nb; ++q) order[(size_t)q] = q;
    uint64_t rs = opt->seed * 6364136223846793005ull + 1442695040888963407ull;
    for (int it = 0; it < iters; ++it) {
        const int q = it % nb;
        if (q == 0) {  // reshuffle once per pass over the samples
            for (int k = nb - 1; k > 0; --k) {
                rs = rs * 6364136223846793005ull + 1442695040888963407ull;
                std::swap(order[(size_t)k], order[(size_t)((rs >> 33) % (uint64_t)(k + 1))]);
            }
        }
        const float *Yb = Yt + (size_t)order[(size_t)q] * B;
        PC_TRY(loss_grad(st, d, r, B, d_s, d_U, Yb, ldt, w, gs.p, gU.p));
        PC_TRY(cudaMemcpyAsync(losses.p + it, w.scal.p + 1, sizeof(float), cudaMemcpyDeviceToDevice, st));
        const float c1 = 1.0f - std::pow(opt->beta1, (float)(it + 1));
        const float c2 = 1.0f - std::pow(opt->beta2, (float)(it + 1));
        adam_kernel<<<blocks_for(d), 256, 0, st>>>(d, d_s, gs.p, ms.p, vs.p, opt->learning_rate, opt->beta1,
                                                  opt->beta2, opt->eps, c1, c2);
        adam_kernel<<<blocks_for((long long)d * r), 256, 0, st>>>((long long)d * r, d_U, gU.p, mU.p, vU.p,
                                                                  opt->learning_rate, opt->beta1, opt->beta2,
                                                                  opt->eps, c1, c2);
        PC_TRY(cudaGetLastError());
    }
    if (opt->standardize) {  // parameters back to the caller's coordinates
        rescale_params_kernel<<<blocks_for((long long)d * r), 256, 0, st>>>(d, r, sig.p, d_s, d_U, 0);
        PC_TRY(cudaGetLastError());
    }
    PC_TRY(cudaEventRecord(e1, st));
    int bad = 0;
    std::vector<float> hl((size_t)std::max(iters, 1), 0.0f);
    if (iters > 0)
        PC_TRY(cudaMemcpyAsync(hl.data(), losses.p, sizeof(float) * iters, cudaMemcpyDeviceToHost, st));
    PC_TRY(cudaMemcpyAsync(&bad, w.bad.p, sizeof bad, cudaMemcpyDeviceToHost, st));
    PC_TRY(cudaStreamSynchronize(st));
    if (bad) return pc_err(ACHR_ERR_NUMERIC, "I + U^T D^-1 U lost positive definiteness during training");
    if (stats) {
        std::memset(stats, 0, sizeof *stats);
        float ms_ = 0.0f;
        cudaEventElapsedTime(&ms_, e0, e1);
        stats->train_ms = ms_;
        stats->iterations = iters;
        if (iters > 0) {
            const int k = std::min(iters, 20);  // means over the first and last 20 minibatches
            double f = 0.0, l = 0.0;
            for (int i = 0; i < k; ++i) {
                f += hl[(size_t)i];
                l += hl[(size_t)(iters - 1 - i)];
            }
            stats->loss_first = f / k;
            stats->loss_last = l / k;
        }
    }
    return ACHR_OK;
}

achr_status achr_precond_dim(achr_ctx *ctx, int32_t *d_out, int32_t *n_frozen_out) {
    using namespace achr;
    if (!ctx) return pc_err(ACHR_ERR_INVALID, "ctx is NULL");
    achr_status st = ensure_active_basis(ctx);
    if (st != ACHR_OK) return st;
    if (d_out) *d_out = ctx->d_act;
    if (n_frozen_out) *n_frozen_out = ctx->n_frozen;
    return ACHR_OK;
}

achr_status achr_get_precond_basis(achr_ctx *ctx, double *basis_out) {
    using namespace achr;
    if (!ctx || !basis_out) return pc_err(ACHR_ERR_INVALID, "NULL argument");
    achr_status st = ensure_active_basis(ctx);
    if (st != ACHR_OK) return st;
    if (ctx->d_act > 0)
        PC_TRY(cudaMemcpy(basis_out, ctx->Nact.p, sizeof(double) * (size_t)ctx->n * ctx->d_act, cudaMemcpyDefault));
    return ACHR_OK;
}

achr_status achr_null_coords(achr_ctx *ctx, int32_t n_points, const double *d_points, int64_t ld, const double *d_mu,
                             float *d_Y, int64_t ldy, void *stream) {
    using namespace achr;
    if (!ctx || n_points < 0 || (n_points > 0 && (!d_points || !d_Y)) || ld < n_points || ldy < n_points)
        return pc_err(ACHR_ERR_INVALID, "bad null-coordinate arguments");
    achr_status bst = ensure_active_basis(ctx);
    if (bst != ACHR_OK) return bst;
    if (n_points == 0 || ctx->d_act == 0) return ACHR_OK;
    const int n = ctx->n, d = ctx->d_act, kpad = (n + 63) / 64 * 64;
    cudaStream_t st = (cudaStream_t)stream;
    DevBuf<__nv_bfloat16> Nh, Nl, Xh, Xl;
    DevBuf<unsigned long long> err;
    PC_TRY(Nh.alloc((size_t)d * kpad));
    PC_TRY(Nl.alloc((size_t)d * kpad));
    PC_TRY(err.alloc(1));
    PC_TRY(cudaMemsetAsync(err.p, 0, sizeof(unsigned long long), st));
    split_nt_kernel<<<blocks_for((long long)d * kpad), 256, 0, st>>>(n, d, kpad, ctx->Nact.p, Nh.p, Nl.p);
    PC_TRY(cudaGetLastError());
    const int chunk = std::min(n_points, 65536);
    PC_TRY(Xh.alloc((size_t)chunk * kpad));
    PC_TRY(Xl.alloc((size_t)chunk * kpad));
    for (int c0 = 0; c0 < n_points; c0 += chunk) {
        const int pc = std::min(chunk, n_points - c0);
        const int nchunks = kpad / 64;
        dim3 grid((unsigned)((pc + 31) / 32), (unsigned)((nchunks + kSplitWarps - 1) / kSplitWarps));
        split_points_kernel<<<grid, kSplitWarps * 32, 0, st>>>(n, kpad, pc, d_points + c0, ld, d_mu, Xh.p, Xl.p);
        PC_TRY(cudaGetLastError());
        TcGemm g{d, pc, kpad, 3, Nh.p, Nl.p, (long long)kpad, Xh.p, Xl.p, (long long)kpad, d_Y + c0, (long long)ldy};
        if (const char *why = tc_gemm_check(g)) return pc_err(ACHR_ERR_INVALID, why);
        PC_TRY(launch_tc_gemm(g, err.p, st));
    }
    unsigned long long h = 0;
    PC_TRY(cudaMemcpyAsync(&h, err.p, sizeof h, cudaMemcpyDeviceToHost, st));
    PC_TRY(cudaStreamSynchronize(st));
    if (h) return pc_err(ACHR_ERR_TIMEOUT, "a tensor-core pipeline wait expired");
    return ACHR_OK;
}

achr_status achr_precond_pool(achr_ctx *ctx, int32_t r, const float *d_s, const float *d_U, int32_t n_dirs,
                              uint64_t seed) {
    using namespace achr;
    if (!ctx || r < 0 || !d_s || (r > 0 && !d_U) || n_dirs <= 0) return pc_err(ACHR_ERR_INVALID, "bad pool arguments");
    achr_status bst = ensure_active_basis(ctx);
    if (bst != ACHR_OK) return bst;
    const int n = ctx->n, d = ctx->d_act, K = n_dirs;
    if (d == 0) return pc_err(ACHR_ERR_UNSUPPORTED, "the polytope spans no direction");
    DevBuf<float> Yp, Z2;
    DevBuf<double> Yd, G;
    PC_TRY(Yp.alloc((size_t)d * K));
    PC_TRY(Z2.alloc((size_t)std::max(r, 1) * K));
    const long long big = std::max<long long>((long long)d * K, (long long)r * K);
    pool_noise_kernel<<<blocks_for(big), 256>>>(d, r, K, seed, d_s, Yp.p, Z2.p);
    PC_TRY(cudaGetLastError());
    // Yp += U Z2  (d x K)
    if (r > 0) PC_TRY(sgemm(nullptr, d, K, r, 1.0f, d_U, r, 1, Z2.p, K, 1, 1.0f, Yp.p, K));
    PC_TRY(Yd.alloc((size_t)d * K));
    f32_to_f64_kernel<<<blocks_for((long long)d * K), 256>>>((long long)d * K, Yp.p, Yd.p);
    PC_TRY(cudaGetLastError());
    // G = N Yp in FP64 (n x K, column-major, ld = ldw): the directions lie in
    // the null space of S to FP64 rounding.  Yp is row-major d x K, i.e. the
    // column-major K x d matrix Yp^T, so G = N * (Yp^T)^T.
    PC_TRY(G.alloc((size_t)ctx->ldw * K));
    PC_TRY(cudaMemset(G.p, 0, sizeof(double) * (size_t)ctx->ldw * K));
    cublasHandle_t cb = nullptr;
    if (cublasCreate(&cb) != CUBLAS_STATUS_SUCCESS) return pc_err(ACHR_ERR_CUDA, "cublasCreate failed");
    const double one = 1.0, zero = 0.0;
    const cublasStatus_t bs =
        cublasDgemm(cb, CUBLAS_OP_N, CUBLAS_OP_T, n, K, d, &one, ctx->Nact.p, n, Yd.p, K, &zero, G.p, ctx->ldw);
    cublasDestroy(cb);
    if (bs != CUBLAS_STATUS_SUCCESS) return pc_err(ACHR_ERR_CUDA, "cublasDgemm (direction pool) failed");
    PC_TRY(cudaDeviceSynchronize());
    return achr_set_directions(ctx, G.p, ctx->ldw, K);
}

}  // extern "C"
