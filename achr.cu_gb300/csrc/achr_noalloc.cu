// achr_sample_noalloc: the chain sampler for callers that cannot allocate GPU
// memory.
//
// Some callers may not call cudaMalloc at all: code running inside another
// framework's memory pool or a pre-sized arena, processes whose device memory
// is reserved up front, or callers that must not add allocations (and their
// latency and possible failure) to a path that runs repeatedly.  This entry
// point takes the model and warmup points already resident on the device, the
// output buffer, and a stream, and performs no allocation of its own.
//
// The working data the chain kernel needs beyond its inputs and outputs (the
// padded start point and centre accumulator, the FP64 and FP32 images of the
// bounds, the conversion-error bound and the statistics counters) lives in one
// file-scope __device__ array, g_noalloc_scratch, sized for models of up to
// ACHR_NOALLOC_MAX_RXNS reactions (about 321 KB).  Every GPU that loads this
// library holds that array until the process exits.
//
// Host code may not pass the array's name to a kernel: on the host the name is
// only a stand-in, not a device address.  The device address is obtained once
// per device with cudaGetSymbolAddress, with that device current, by the first
// call on that device; make that first call before any stream capture.
//
// Every call reuses the same array and leaves the last call's contents in it;
// each call rewrites or clears everything it reads.  Calls whose GPU work
// overlaps (different streams, or different host threads on one device) race
// on the array and must be serialised by the caller.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/achr.h"
#include "achr_internal.h"

extern "C" void achr_io_set_error(const char *msg);

namespace {

constexpr int kMaxRxns = ACHR_NOALLOC_MAX_RXNS;
constexpr int kMaxDevices = 64;
constexpr size_t kCounterBytes = 256;  // achr::CNT_SLOTS counters, rounded to the array alignment
constexpr size_t kScratchBytes = kCounterBytes + 256 /* bound error */ +
                                 (size_t)kMaxRxns * (sizeof(double) * 2 + sizeof(double2) + sizeof(float2));

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

struct ScratchView {
    unsigned long long *counters;
    unsigned int *bound_err_bits;
    double *c0, *A0;
    double2 *lbub;
    float2 *bnd;
};

ScratchView view_of(unsigned char *base) {
    ScratchView v;
    v.counters = reinterpret_cast<unsigned long long *>(base);
    v.bound_err_bits = reinterpret_cast<unsigned int *>(base + kCounterBytes);
    unsigned char *p = base + kCounterBytes + 256;
    v.c0 = reinterpret_cast<double *>(p);
    v.A0 = v.c0 + kMaxRxns;
    v.lbub = reinterpret_cast<double2 *>(v.A0 + kMaxRxns);
    v.bnd = reinterpret_cast<float2 *>(v.lbub + kMaxRxns);
    return v;
}

std::mutex g_addr_mutex;
unsigned char *g_addr[kMaxDevices] = {};

achr_status fail(achr_status st, const std::string &msg) {
    achr_io_set_error(msg.c_str());
    return st;
}

// Per-reaction derived arrays, padded to np: start point, centre accumulator,
// (lb, ub) in FP64 and FP32 (padding 0 / (-1, 1)), and the largest FP32
// conversion error of a finite bound (atomic max on the bits of a
// non-negative float).
__global__ void noalloc_prepare(int n, int np, int W, long long ldw, const double *__restrict__ warmup,
                                const double *__restrict__ lb, const double *__restrict__ ub, int centre_offset,
                                ScratchView sv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    if (i >= n) {
        sv.c0[i] = 0.0;
        sv.A0[i] = 0.0;
        sv.lbub[i] = make_double2(0.0, 0.0);
        sv.bnd[i] = make_float2(-1.0f, 1.0f);
        return;
    }
    double acc = 0.0;
    for (int j = 0; j < W; ++j) acc += warmup[(size_t)j * (size_t)ldw + i];
    const double c = (1.0 / (double)W) * acc;  // centre of the warmup points (ACHRCuda.cu:414-434)
    sv.c0[i] = c;
    sv.A0[i] = (double)(W + centre_offset) * c;
    const double l = lb[i], u = ub[i];
    sv.lbub[i] = make_double2(l, u);
    float lf, uf, err = 0.0f;
    if (isinf(l)) {
        lf = l > 0 ? 3.0e38f : -3.0e38f;
    } else {
        lf = __double2float_rn(l);
        err = fmaxf(err, __double2float_ru(fabs(l - (double)lf)));
    }
    if (isinf(u)) {
        uf = u > 0 ? 3.0e38f : -3.0e38f;
    } else {
        uf = __double2float_rn(u);
        err = fmaxf(err, __double2float_ru(fabs(u - (double)uf)));
    }
    sv.bnd[i] = make_float2(lf, uf);
    if (err > 0.0f) atomicMax(sv.bound_err_bits, __float_as_uint(err));
}

float f32_up(double v) {
    float f = (float)v;
    if ((double)f < v) f = std::nextafter(f, INFINITY);
    return f;
}

float f32_down(double v) {
    float f = (float)v;
    if ((double)f > v) f = std::nextafter(f, -INFINITY);
    return f;
}

#define NOALLOC_TRY(expr)                                                                  \
    do {                                                                                   \
        cudaError_t e_ = (expr);                                                           \
        if (e_ != cudaSuccess) return fail(ACHR_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

}  // namespace

extern "C" achr_status achr_sample_noalloc(const achr_device_model *m, const achr_options *opt_in, uint64_t seed,
                                           uint64_t chain_offset, int32_t n_points, int32_t n_steps,
                                           double *d_points_out, int64_t ld_out, void *stream, achr_stats *stats) {
    if (!m) return fail(ACHR_ERR_INVALID, "model is NULL");
    achr_options opt;
    if (opt_in) opt = *opt_in;
    else achr_default_options(&opt);
    const int n = m->n_rxns;
    if (n <= 0 || m->n_mets < 0 || m->n_warmup <= 0 || m->null_dim < 0 || m->null_dim > n)
        return fail(ACHR_ERR_INVALID, "bad model sizes");
    if (n > kMaxRxns)
        return fail(ACHR_ERR_UNSUPPORTED, "achr_sample_noalloc handles at most " + std::to_string(kMaxRxns) +
                                              " reactions (its scratch array is sized for that); got " +
                                              std::to_string(n));
    if (m->ld_warmup < n || (m->ld_warmup & 1) || !m->warmup || !m->lb || !m->ub || !m->row_ptr ||
        (m->null_dim > 0 && !m->N))
        return fail(ACHR_ERR_INVALID, "bad device model (ld_warmup must be even and >= n_rxns; pointers non-NULL)");
    if ((reinterpret_cast<uintptr_t>(m->warmup) & 15u) != 0)
        return fail(ACHR_ERR_INVALID, "warmup must start on a 16-byte boundary");
    if (n_points < 0 || n_steps < 0 || (n_points > 0 && (!d_points_out || ld_out < n_points)))
        return fail(ACHR_ERR_INVALID, "bad output arguments");
    if (opt.mode != ACHR_MODE_REFERENCE && opt.mode != ACHR_MODE_FEASIBLE) return fail(ACHR_ERR_INVALID, "unknown mode");
    if (opt.check_period < 0 || opt.max_attempts <= 0 || (opt.centre_offset != 0 && opt.centre_offset != 1))
        return fail(ACHR_ERR_INVALID, "bad options");
    const int np = achr::chain_padded_length(n, opt.threads_per_chain);
    if (np == 0 || np > kMaxRxns) return fail(ACHR_ERR_UNSUPPORTED, "no chain-kernel configuration for this size");

    int dev = 0;
    NOALLOC_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(ACHR_ERR_UNSUPPORTED, "device index out of range");
    unsigned char *base;
    {
        std::lock_guard<std::mutex> lock(g_addr_mutex);
        if (!g_addr[dev]) {
            void *ptr = nullptr;
            NOALLOC_TRY(cudaGetSymbolAddress(&ptr, g_noalloc_scratch));
            g_addr[dev] = static_cast<unsigned char *>(ptr);
        }
        base = g_addr[dev];
    }
    const ScratchView sv = view_of(base);
    cudaStream_t s = (cudaStream_t)stream;
    NOALLOC_TRY(cudaMemsetAsync(sv.counters, 0, kCounterBytes + 256, s));  // counters and the bound-error bits
    noalloc_prepare<<<(np + 127) / 128, 128, 0, s>>>(n, np, m->n_warmup, (long long)m->ld_warmup, m->warmup, m->lb,
                                                      m->ub, opt.centre_offset, sv);
    NOALLOC_TRY(cudaGetLastError());
    unsigned int err_bits = 0;
    NOALLOC_TRY(cudaMemcpyAsync(&err_bits, sv.bound_err_bits, sizeof err_bits, cudaMemcpyDeviceToHost, s));
    NOALLOC_TRY(cudaStreamSynchronize(s));
    float berr;
    std::memcpy(&berr, &err_bits, sizeof berr);

    achr::ChainArgs a{};
    a.n = n;
    a.m = m->n_mets;
    a.W = m->n_warmup;
    a.d = m->null_dim;
    a.np = np;
    a.ldw = (int)m->ld_warmup;
    a.P = n_points;
    a.T = n_steps;
    a.warmup = m->warmup;
    a.c0 = sv.c0;
    a.A0 = sv.A0;
    a.lbub = sv.lbub;
    a.bnd = sv.bnd;
    a.bound_err = berr;
    a.dtol_hi = f32_up(opt.d_tol) * (1.0f + 9.5367431640625e-07f);
    a.dtol_lo = f32_down(opt.d_tol) * (1.0f - 9.5367431640625e-07f);
    a.utol32 = (float)opt.u_tol;
    a.mmt32 = (float)opt.max_min_tol;
    a.row_ptr = m->row_ptr;
    a.col_idx = m->col_idx;
    a.val = m->val;
    a.N = m->N;
    a.out = d_points_out;
    a.ld_out = ld_out;
    a.seed = seed;
    a.chain_offset = chain_offset;
    a.check_period = opt.check_period > 0 ? opt.check_period : 0x7fffffff;
    a.max_attempts = opt.max_attempts;
    a.centre_offset = opt.centre_offset;
    a.exact_ratio = opt.exact_ratio;
    a.final_project = opt.mode == ACHR_MODE_FEASIBLE ? 1 : 0;
    a.residual_tol = opt.residual_tol;
    a.max_min_tol = opt.max_min_tol;
    a.u_tol = opt.u_tol;
    a.d_tol = opt.d_tol;
    a.feasibility_tol = opt.feasibility_tol;
    a.counters = sv.counters;
    a.step0 = 0;
    a.x_in = nullptr;
    a.A_in = nullptr;
    a.A_out = nullptr;
    a.ld_state = 0;
    cudaError_t e = achr::launch_chains(a, opt.threads_per_chain, s);
    if (e != cudaSuccess) return fail(ACHR_ERR_CUDA, std::string("chain kernel launch: ") + cudaGetErrorString(e));
    if (!stats) return ACHR_OK;
    unsigned long long c[achr::CNT_SLOTS];
    NOALLOC_TRY(cudaMemcpyAsync(c, sv.counters, sizeof c, cudaMemcpyDeviceToHost, s));
    NOALLOC_TRY(cudaStreamSynchronize(s));
    if (c[achr::CNT_ERROR] & achr::ERR_TMA_TIMEOUT)
        return fail(ACHR_ERR_TIMEOUT, "a warmup-column copy did not complete within its wait limit");
    std::memset(stats, 0, sizeof *stats);
    stats->accepted = (int64_t)c[achr::CNT_ACCEPTED];
    stats->rejected = (int64_t)c[achr::CNT_REJECTED];
    stats->checks = (int64_t)c[achr::CNT_CHECKS];
    stats->reprojections = (int64_t)c[achr::CNT_REPROJ];
    stats->stuck_chains = (int64_t)c[achr::CNT_STUCK];
    stats->exact_evals = (int64_t)c[achr::CNT_EXACT];
    stats->final_projections = (int64_t)c[achr::CNT_FINAL_PROJ];
    std::memcpy(&stats->max_residual, &c[achr::CNT_MAXRES_BITS], sizeof(double));
    std::memcpy(&stats->max_bound_violation, &c[achr::CNT_MAXVIOL_BITS], sizeof(double));
    stats->kernel_ms = 0.0;
    return ACHR_OK;
}
