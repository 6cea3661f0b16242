// Convergence check of an installed hit-and-run direction pool, with the
// fallback to the reference's own direction rule.
//
// A learned (or any) direction pool changes only how directions are drawn;
// plain ACHR (a random warmup point minus the running centre, ACHRcu/
// ACHRCuda.cu:260-264) stays the method of record.  achr_check_directions
// runs a pilot of the pool from over-dispersed starts (random warmup points),
// computes the split-R-hat of every flux on the GPU, and removes the pool --
// the context goes back to plain ACHR -- when the largest R-hat is at or above
// the caller's limit (1.01 in the usual practice).
//
// Split-R-hat as in Gelman et al., Bayesian Data Analysis (3rd ed., 11.4):
// every chain's draws are cut into a first and a second half, and with n draws
// per half, W the mean of the halves' variances and B/n the variance of their
// means, R-hat = sqrt(((n - 1)/n W + B/n) / W).  Fluxes that do not move
// (W = 0: blocked or pinned reactions) are left out.
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

constexpr int kRhatThreads = 256;

achr_status rh_err(achr_status st, const std::string &msg) {
    achr_io_set_error(msg.c_str());
    return st;
}

#define RH_TRY(expr)                                                                              \
    do {                                                                                          \
        cudaError_t e_ = (expr);                                                                  \
        if (e_ != cudaSuccess) return rh_err(ACHR_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// x (n x M row-major) = warmup point idx_p for chain p, idx_p from Philox keyed by seed.
__global__ void dispersed_start_kernel(int n, int M, int W, int ldw, const double *__restrict__ warmup,
                                       unsigned long long seed, double *__restrict__ x) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n * M) return;
    const int i = (int)(t / M), p = (int)(t % M);
    const Philox4 w = philox4x32_10((uint32_t)p, 0x73746172u, 0u, 0u, (uint32_t)seed, (uint32_t)(seed >> 32));
    const int idx = (int)(((unsigned long long)w.v[0] * (unsigned long long)W) >> 32);
    x[t] = warmup[(size_t)idx * (size_t)ldw + (size_t)i];
}

// One block per flux i: trace is K slices of n x M (row-major), draws of chain p
// at trace[k * n * M + i * M + p].  Writes the split-R-hat (NaN when the flux
// does not move) to rhat[i].
__global__ void __launch_bounds__(kRhatThreads)
    split_rhat_kernel(int n, int M, int K, const double *__restrict__ trace, double *__restrict__ rhat) {
    __shared__ double red[3][kRhatThreads / 32];
    const int i = blockIdx.x;
    const int h = K / 2;  // draws per half (an odd middle draw is left out)
    double sw = 0.0, sm = 0.0, smm = 0.0;  // sums over halves of variance, mean, mean^2
    for (int p = threadIdx.x; p < M; p += blockDim.x) {
        for (int half = 0; half < 2; ++half) {
            const int k0 = half == 0 ? 0 : K - h;
            double mean = 0.0, m2 = 0.0;
            for (int k = 0; k < h; ++k) {  // Welford
                const double v = trace[((size_t)(k0 + k) * (size_t)n + (size_t)i) * (size_t)M + (size_t)p];
                const double dlt = v - mean;
                mean += dlt / (double)(k + 1);
                m2 += dlt * (v - mean);
            }
            sw += h > 1 ? m2 / (double)(h - 1) : 0.0;
            sm += mean;
            smm += mean * mean;
        }
    }
    for (int o = 16; o; o >>= 1) {
        sw += __shfl_xor_sync(0xffffffffu, sw, o);
        sm += __shfl_xor_sync(0xffffffffu, sm, o);
        smm += __shfl_xor_sync(0xffffffffu, smm, o);
    }
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = sw;
        red[1][threadIdx.x >> 5] = sm;
        red[2][threadIdx.x >> 5] = smm;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        sw = sm = smm = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            sw += red[0][w];
            sm += red[1][w];
            smm += red[2][w];
        }
        const double halves = 2.0 * (double)M;
        const double Wv = sw / halves;
        const double mbar = sm / halves;
        const double b_over_n = (smm - halves * mbar * mbar) / (halves - 1.0);
        const double nd = (double)h;
        const double scale = 1.0 + fabs(mbar);
        rhat[i] = (Wv > 1e-24 * scale * scale) ? sqrt(((nd - 1.0) / nd * Wv + fmax(b_over_n, 0.0)) / Wv) : nan("");
    }
}

}  // namespace
}  // namespace achr

extern "C" achr_status achr_check_directions(achr_ctx *ctx, int32_t chains, int32_t burnin, int32_t draws,
                                             int32_t gap, uint64_t seed, double rhat_limit,
                                             achr_direction_check *out) {
    using namespace achr;
    if (!ctx || chains < 2 || burnin < 0 || draws < 4 || gap < 1 || !(rhat_limit > 1.0))
        return rh_err(ACHR_ERR_INVALID, "bad direction-check arguments (chains >= 2, draws >= 4, gap >= 1, limit > 1)");
    if ((long long)burnin + (long long)draws * gap > 2147483647LL) return rh_err(ACHR_ERR_INVALID, "step count overflow");
    if (ctx->n_dirs == 0) return rh_err(ACHR_ERR_INVALID, "no direction pool is installed");
    const int n = ctx->n, M = chains;
    const size_t nm = (size_t)n * (size_t)M;
    DevBuf<double> x, A, trace, rh;
    RH_TRY(x.alloc(nm));
    RH_TRY(A.alloc(nm));
    RH_TRY(trace.alloc(nm * (size_t)draws));
    RH_TRY(rh.alloc((size_t)n));
    RH_TRY(cudaMemset(A.p, 0, sizeof(double) * nm));  // hit-and-run keeps no centre
    dispersed_start_kernel<<<(unsigned)((nm + 255) / 256), 256>>>(n, M, ctx->W, ctx->ldw, ctx->warmup.p, seed,
                                                                  x.p);
    RH_TRY(cudaGetLastError());
    achr_stats st;
    double ms = 0.0;
    achr_status s = achr_sample_resume(ctx, seed, 0, M, 0, burnin, 1, x.p, A.p, M, nullptr, &st);
    if (s != ACHR_OK) return s;
    ms += st.kernel_ms;
    for (int k = 0; k < draws; ++k) {
        s = achr_sample_resume(ctx, seed, 0, M, burnin + k * gap, gap, 1, x.p, A.p, M, nullptr, &st);
        if (s != ACHR_OK) return s;
        ms += st.kernel_ms;
        RH_TRY(cudaMemcpy(trace.p + (size_t)k * nm, x.p, sizeof(double) * nm, cudaMemcpyDeviceToDevice));
    }
    split_rhat_kernel<<<(unsigned)n, kRhatThreads>>>(n, M, draws, trace.p, rh.p);
    RH_TRY(cudaGetLastError());
    std::vector<double> h((size_t)n);
    RH_TRY(cudaMemcpy(h.data(), rh.p, sizeof(double) * n, cudaMemcpyDeviceToHost));
    double mx = 0.0;
    int moving = 0;
    for (double v : h)
        if (!std::isnan(v)) {
            ++moving;
            mx = std::max(mx, v);
        }
    const bool keep = moving > 0 && mx < rhat_limit;
    if (!keep) {
        s = achr_set_directions(ctx, nullptr, 0, 0);  // back to the reference's direction rule
        if (s != ACHR_OK) return s;
    }
    if (out) {
        std::memset(out, 0, sizeof *out);
        out->rhat_max = mx;
        out->fluxes = moving;
        out->kept = keep ? 1 : 0;
        out->sampling_ms = ms;
    }
    return ACHR_OK;
}
