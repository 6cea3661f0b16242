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
// bounds, the conversion-error bound, the input-check flags, the partial sums
// of the box norm and the statistics counters) lives in one file-scope
// __device__ array, g_noalloc_scratch, sized for models of up to
// ACHR_NOALLOC_MAX_RXNS reactions (about 322 KB).  Every GPU that loads this
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
//
// The caller's model is checked on the device before the chain kernel runs
// (the allocating path checks the same things on the host while it builds its
// own copy): a CSR of S whose offsets are not monotone, do not start at 0 or
// do not end at nnz, a column index outside [0, n), a non-finite coefficient,
// lb > ub or a NaN bound, or a non-finite warmup value make the call return
// ACHR_ERR_INVALID without sampling.
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
constexpr int kPrepThreads = 128;
constexpr int kMaxPrepBlocks = (kMaxRxns + kPrepThreads - 1) / kPrepThreads;  // 64
constexpr size_t kCounterBytes = 256;  // achr::CNT_SLOTS counters, rounded to the array alignment
// Header: bound-error bits (4 B), input-check flags (4 B), then one partial sum
// of max(lb^2, ub^2) per set-up block.
constexpr size_t kHeaderBytes = 1024;
static_assert(8 + sizeof(double) * kMaxPrepBlocks <= kHeaderBytes, "header too small");
constexpr size_t kScratchBytes =
    kCounterBytes + kHeaderBytes + (size_t)kMaxRxns * (sizeof(double) * 2 + sizeof(double2) + sizeof(float2));

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Input-check flags.
enum : unsigned {
    BAD_CSR = 1u,      // offsets not monotone / not from 0 to nnz, or a column index outside [0, n)
    BAD_COEF = 2u,     // a non-finite coefficient
    BAD_BOUND = 4u,    // lb > ub or a NaN bound
    BAD_WARMUP = 8u,   // a non-finite warmup value
};

struct ScratchView {
    unsigned long long *counters;
    unsigned int *bound_err_bits;
    unsigned int *check_bits;
    double *box_partial;
    double *c0, *A0;
    double2 *lbub;
    float2 *bnd;
};

ScratchView view_of(unsigned char *base) {
    ScratchView v;
    v.counters = reinterpret_cast<unsigned long long *>(base);
    v.bound_err_bits = reinterpret_cast<unsigned int *>(base + kCounterBytes);
    v.check_bits = v.bound_err_bits + 1;
    v.box_partial = reinterpret_cast<double *>(base + kCounterBytes + 8);
    unsigned char *p = base + kCounterBytes + kHeaderBytes;
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

// Device-side check of the caller's model (grid-stride over every array; reads
// only within the extents the caller declared).
__global__ void noalloc_validate(int n, int m, long long nnz, int W, long long ldw, const double *__restrict__ warmup,
                                 const double *__restrict__ lb, const double *__restrict__ ub,
                                 const int *__restrict__ row_ptr, const int *__restrict__ col_idx,
                                 const double *__restrict__ val, unsigned *bits) {
    const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    unsigned f = 0;
    if (t0 == 0 && m > 0 && (row_ptr[0] != 0 || (long long)row_ptr[m] != nnz)) f |= BAD_CSR;
    for (long long i = t0; i < m; i += stride)
        if (row_ptr[i] > row_ptr[i + 1]) f |= BAD_CSR;
    for (long long q = t0; q < nnz; q += stride) {
        const int c = col_idx[q];
        if (c < 0 || c >= n) f |= BAD_CSR;
        if (!isfinite(val[q])) f |= BAD_COEF;
    }
    for (long long i = t0; i < n; i += stride) {
        const double l = lb[i], u = ub[i];
        if (!(l <= u)) f |= BAD_BOUND;
    }
    const long long nw = (long long)n * W;
    for (long long k = t0; k < nw; k += stride) {
        const long long j = k / n, i = k - j * n;
        if (!isfinite(warmup[j * ldw + i])) f |= BAD_WARMUP;
    }
    if (f) atomicOr(bits, f);
}

// Per-reaction derived arrays, padded to np: start point, centre accumulator,
// (lb, ub) in FP64 and FP32 (padding 0 / (-1, 1)), the largest FP32
// conversion error of a finite bound (atomic max on the bits of a
// non-negative float), and per block the sum of max(lb^2, ub^2) over its
// reactions, reduced in a fixed order so that the host's total (and with it
// the bracket bound derived from the box) is the same on every call.
__global__ void __launch_bounds__(kPrepThreads)
    noalloc_prepare(int n, int np, int W, long long ldw, const double *__restrict__ warmup,
                    const double *__restrict__ lb, const double *__restrict__ ub, int centre_offset, ScratchView sv) {
    __shared__ double part[kPrepThreads / 32];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double box = 0.0;
    if (i < np) {
        if (i >= n) {
            sv.c0[i] = 0.0;
            sv.A0[i] = 0.0;
            sv.lbub[i] = make_double2(0.0, 0.0);
            sv.bnd[i] = make_float2(-1.0f, 1.0f);
        } else {
            double acc = 0.0;
            for (int j = 0; j < W; ++j) acc += warmup[(size_t)j * (size_t)ldw + i];
            const double c = (1.0 / (double)W) * acc;  // centre of the warmup points (ACHRCuda.cu:414-434)
            sv.c0[i] = c;
            sv.A0[i] = (double)(W + centre_offset) * c;
            const double l = lb[i], u = ub[i];
            sv.lbub[i] = make_double2(l, u);
            box = fmax(l * l, u * u);
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
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) box += __shfl_xor_sync(0xffffffffu, box, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = box;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < kPrepThreads / 32; ++w) s += part[w];
        sv.box_partial[blockIdx.x] = s;
    }
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
    if (n <= 0 || m->n_mets < 0 || m->n_warmup <= 0 || m->null_dim < 0 || m->null_dim > n || m->nnz < 0)
        return fail(ACHR_ERR_INVALID, "bad model sizes");
    if (n > kMaxRxns)
        return fail(ACHR_ERR_UNSUPPORTED, "achr_sample_noalloc handles at most " + std::to_string(kMaxRxns) +
                                              " reactions (its scratch array is sized for that); got " +
                                              std::to_string(n));
    if (m->ld_warmup < n || (m->ld_warmup & 1) || !m->warmup || !m->lb || !m->ub || !m->row_ptr ||
        (m->nnz > 0 && (!m->col_idx || !m->val)) || (m->null_dim > 0 && !m->N))
        return fail(ACHR_ERR_INVALID,
                    "bad device model (ld_warmup must be even and >= n_rxns; warmup, bounds, row_ptr, and with "
                    "nnz > 0 col_idx and val, and with null_dim > 0 N must be non-NULL)");
    if (m->n_mets == 0 && m->nnz != 0) return fail(ACHR_ERR_INVALID, "nnz must be 0 when n_mets is 0");
    if ((reinterpret_cast<uintptr_t>(m->warmup) & 15u) != 0)
        return fail(ACHR_ERR_INVALID, "warmup must start on a 16-byte boundary");
    if (n_points < 0 || n_steps < 0 || (n_points > 0 && (!d_points_out || ld_out < n_points)))
        return fail(ACHR_ERR_INVALID, "bad output arguments");
    if (chain_offset + (uint64_t)n_points < chain_offset) return fail(ACHR_ERR_INVALID, "chain ids overflow");
    if (opt.mode != ACHR_MODE_REFERENCE && opt.mode != ACHR_MODE_FEASIBLE) return fail(ACHR_ERR_INVALID, "unknown mode");
    if (opt.check_period < 0 || opt.max_attempts <= 0 || (opt.centre_offset != 0 && opt.centre_offset != 1) ||
        (opt.bracket_pass != 0 && opt.bracket_pass != 1) || opt.reproject_form < 0 || opt.reproject_form > 3)
        return fail(ACHR_ERR_INVALID, "bad options");
    if (!(opt.residual_tol >= 0) || !(opt.max_min_tol >= 0) || !(opt.u_tol >= 0) || !(opt.d_tol >= 0) ||
        !(opt.feasibility_tol >= 0))
        return fail(ACHR_ERR_INVALID, "tolerances must be non-negative");
    if (opt.reproject_form == 2 || opt.reproject_form == 3)
        return fail(ACHR_ERR_UNSUPPORTED,
                    "achr_sample_noalloc reprojects as N (N^T x) in FP64; the residual and deferred forms "
                    "(reproject_form 2 and 3) need a pseudo-inverse of S S^T and buffers that only a context builds");
    const int np = achr::chain_padded_length(n, opt.threads_per_chain);
    if (np == 0 || np > kMaxRxns) return fail(ACHR_ERR_UNSUPPORTED, "no chain-kernel configuration for this size");
    const int prep_blocks = (np + kPrepThreads - 1) / kPrepThreads;

    int dev = 0, sms = 0;
    NOALLOC_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(ACHR_ERR_UNSUPPORTED, "device index out of range");
    NOALLOC_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
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
    // counters, bound-error bits and check flags start at zero
    NOALLOC_TRY(cudaMemsetAsync(sv.counters, 0, kCounterBytes + 8, s));
    noalloc_validate<<<(unsigned)(sms > 0 ? 4 * sms : 64), 256, 0, s>>>(
        n, m->n_mets, (long long)m->nnz, m->n_warmup, (long long)m->ld_warmup, m->warmup, m->lb, m->ub, m->row_ptr,
        m->col_idx, m->val, sv.check_bits);
    NOALLOC_TRY(cudaGetLastError());
    noalloc_prepare<<<(unsigned)prep_blocks, kPrepThreads, 0, s>>>(n, np, m->n_warmup, (long long)m->ld_warmup,
                                                                   m->warmup, m->lb, m->ub, opt.centre_offset, sv);
    NOALLOC_TRY(cudaGetLastError());
    unsigned char head[8 + sizeof(double) * kMaxPrepBlocks];
    NOALLOC_TRY(cudaMemcpyAsync(head, sv.bound_err_bits, 8 + sizeof(double) * (size_t)prep_blocks,
                                cudaMemcpyDeviceToHost, s));
    NOALLOC_TRY(cudaStreamSynchronize(s));
    unsigned check = 0;
    float berr;
    std::memcpy(&berr, head, sizeof berr);
    std::memcpy(&check, head + 4, sizeof check);
    if (check) {
        std::string why;
        if (check & BAD_CSR) why += " CSR offsets or column indices out of range;";
        if (check & BAD_COEF) why += " non-finite coefficient;";
        if (check & BAD_BOUND) why += " lb > ub or NaN bound;";
        if (check & BAD_WARMUP) why += " non-finite warmup value;";
        return fail(ACHR_ERR_INVALID, "device model rejected:" + why);
    }
    double box_sq = 0.0;
    for (int b = 0; b < prep_blocks; ++b) {
        double v;
        std::memcpy(&v, head + 8 + sizeof(double) * b, sizeof v);
        box_sq += v;
    }

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
    a.dtol_hi = achr::f32_up(opt.d_tol) * (1.0f + 9.5367431640625e-07f);
    a.dtol_lo = achr::f32_down(opt.d_tol) * (1.0f - 9.5367431640625e-07f);
    a.utol32 = (float)opt.u_tol;
    a.mmt32 = (float)opt.max_min_tol;
    // Brackets formed with the direction when the box bounds ||d|| (every point
    // and centre lies in it: ||w - c|| <= 2 sqrt(sum max(lb^2, ub^2))), as the
    // allocating path does; infinite bounds or bracket_pass = 1 keep a separate pass.
    achr::set_merged_bound(a, opt.u_tol, opt.bracket_pass == 1 ? INFINITY : 2.0 * std::sqrt(box_sq));
    // The residual check reads the caller's CSR rows directly (the allocating
    // path reads a sliced-ELL copy it builds; the sums are the same).
    a.row_ptr = m->row_ptr;
    a.col_idx = m->col_idx;
    a.val = m->val;
    a.sell_off = nullptr;
    a.pinv32 = nullptr;  // reprojection as N (N^T x) in FP64
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
    const long long wl = opt.wait_limit_ns;
    a.wait_ns = wl != 0 ? (unsigned long long)(wl < 0 ? -wl : wl) : 0ull;
    a.wait_never = wl < 0 ? 1 : 0;
    cudaError_t e = achr::launch_chains(a, opt.threads_per_chain, s);
    if (e != cudaSuccess) return fail(ACHR_ERR_CUDA, std::string("chain kernel launch: ") + cudaGetErrorString(e));
    unsigned long long c[achr::CNT_SLOTS];
    NOALLOC_TRY(cudaMemcpyAsync(c, sv.counters, sizeof c, cudaMemcpyDeviceToHost, s));
    NOALLOC_TRY(cudaStreamSynchronize(s));
    if (c[achr::CNT_ERROR] & achr::ERR_TMA_TIMEOUT)
        return fail(ACHR_ERR_TIMEOUT, "a warmup-column copy did not complete within its wait limit");
    if (!stats) return ACHR_OK;
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
