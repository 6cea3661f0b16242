// Persistent chain kernel: the ACHR sampling hot loop on sm_103a.
//
// Replaces the reference's chain driver and step loop (ACHRcu/ACHRCuda.cu:
// stepPointProgress :361-385, createPoint :297-359, fillrandPoint :251-289,
// advNextStep :242-249, findMaxAbs :232-240, reprojectPoint(2) :208-230,
// correctBounds :193-206), which run one chain per GPU thread and launch child
// grids from the device for every step.
//
// Design (one CTA per chain, persistent over chains):
//   * The chain's point x and centre accumulator A = (W + t) c live in shared
//     memory for all T steps; only the warmup column w_r is read from HBM/L2
//     each step, staged into shared memory by a 1-D TMA bulk copy
//     (cp.async.bulk + mbarrier) that is issued one step ahead.
//   * GB300's FP64 pipe issues about 1.6 DFMA per clock per SM, 72x less than
//     FP32.  Per element and accepted step the kernel therefore spends three
//     FP64 pipe operations on the update (d = w - A/(W+t), x += s d, A += x),
//     one for the norm, and none for the ratio test: the bound distances and
//     ratios are bracketed in FP32 with rigorous error bounds, and only the
//     candidates whose bracket can hold the minimum are evaluated in FP64.
//   * The ratio test uses the unnormalised direction d (t/||d|| is what the
//     update needs), so no per-element FP64 division remains.
//   * Reductions are warp shuffles plus one shared-memory exchange; summation
//     order is fixed, so a launch is bitwise repeatable.
#include <cfloat>
#include <cmath>

#include "achr_internal.h"
#include "achr_rng.cuh"

namespace achr {
namespace {

constexpr float kErrK = 2.384185791015625e-07f;        // 2^-22: bound on truncation + FP32 rounding
constexpr float kTiny = 2.350988701644575e-38f;        // 2^-125: absolute error of flushed tiny values
constexpr float kUp = 1.0f + 9.5367431640625e-07f;     // 1 + 2^-20
constexpr float kDn = 1.0f - 9.5367431640625e-07f;     // 1 - 2^-20
constexpr float kAdUp = 1.0f + 4.76837158203125e-07f;  // 1 + 2^-21
constexpr unsigned long long kWaitNs = 2000000000ull;  // bounded mbarrier wait: 2 s

// FP64 -> FP32 rounding toward zero with integer operations only (no FP64
// pipe).  |v - f| <= 2^-23 |f| + 2^-126; tiny values flush to signed zero,
// overflow and inf map to inf.
__device__ __forceinline__ float f64_to_f32_rz(double v) {
    const unsigned hi = (unsigned)__double2hiint(v);
    const unsigned lo = (unsigned)__double2loint(v);
    const unsigned sign = hi & 0x80000000u;
    const int fe = (int)((hi >> 20) & 0x7FFu) - 896;  // re-bias 1023 -> 127
    unsigned mag = ((unsigned)fe << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29);
    mag = (fe <= 0) ? 0u : mag;
    mag = (fe >= 255) ? 0x7F800000u : mag;
    return __uint_as_float(sign | mag);
}

__device__ __forceinline__ unsigned smem_addr(const void *p) {
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// 1-D bulk copy global -> shared, completion counted on `bar`.  Both addresses
// are 16-byte aligned and bytes is a multiple of 16 (the warmup leading
// dimension is even and the shared buffer starts on a 128-byte boundary).
__device__ __forceinline__ void tma_load_1d(void *dst, const void *src, unsigned bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Wait for the phase with the given parity to complete, giving up after kWaitNs.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, unsigned parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    for (;;) {
        if (mbar_try_wait(bar, parity)) return true;
        if (global_ns() - t0 > kWaitNs) return false;
    }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ double warp_min(double v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ float warp_minf(float v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ int warp_or(int v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v |= __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Shared-memory exchange slots of the block reductions.  Each reduction in a
// step uses its own slots; a __syncthreads() separates two uses of one slot.
struct RedSlots {
    double sum[32];
    float2 fmin2[32];
    int flag2[32];
    double2 dmin2[32];
    int flag3[32];
    double mx[32];
    double viol[32];
};

__device__ __forceinline__ double block_sum(double v, double *slot, int lane, int warp, int nwarps) {
    v = warp_sum(v);
    if (lane == 0) slot[warp] = v;
    __syncthreads();
    double r = 0.0;
    for (int w = 0; w < nwarps; ++w) r += slot[w];
    return r;
}

__device__ __forceinline__ double block_max(double v, double *slot, int lane, int warp, int nwarps) {
    v = warp_max(v);
    if (lane == 0) slot[warp] = v;
    __syncthreads();
    double r = slot[0];
    for (int w = 1; w < nwarps; ++w) r = fmax(r, slot[w]);
    return r;
}

// FP32 bracket of one coordinate's ratio-test contribution.
enum { ST_INVALID = 0, ST_VALID = 1, ST_AMBIG = 2 };
struct Bracket {
    int st;
    float qh_dn, qh_up;  // bracket of (d > 0 ? ub - x : x - lb) / |d|   (upper step)
    float ql_dn, ql_up;  // bracket of (d > 0 ? x - lb : ub - x) / |d|   (lower step magnitude)
};

// Decide, from FP32 approximations with error bounds, whether coordinate i is
// certainly a ratio-test candidate (reference ACHRCuda.cu:270-279: distUb > dTol,
// distLb > dTol and |u_i| > uTol), certainly not, or undecided; for certain
// candidates bracket the two step ratios.
__device__ __forceinline__ Bracket bracket(double x, double dk, float4 b, float dtol_hi, float dtol_lo,
                                           float uthr_hi, float uthr_lo) {
    Bracket c;
    const float x32 = f64_to_f32_rz(x);
    const float d32 = f64_to_f32_rz(dk);
    const float ad = fabsf(d32);
    const float Dp = b.y - x32;  // ub - x
    const float Dm = x32 - b.x;  // x - lb
    const float ex = fmaf(fabsf(x32), kErrK, kTiny);
    const float Ep = isinf(Dp) ? 0.0f : (b.w + ex) + fabsf(Dp) * kErrK;
    const float Em = isinf(Dm) ? 0.0f : (b.z + ex) + fabsf(Dm) * kErrK;
    const bool p_ok = (Dp - Ep) > dtol_hi, p_bad = (Dp + Ep) <= dtol_lo;
    const bool m_ok = (Dm - Em) > dtol_hi, m_bad = (Dm + Em) <= dtol_lo;
    const bool u_ok = ad > uthr_hi, u_bad = ad * kAdUp < uthr_lo;
    c.st = (p_bad || m_bad || u_bad) ? ST_INVALID : ((p_ok && m_ok && u_ok) ? ST_VALID : ST_AMBIG);
    const float r = __frcp_rn(ad);
    const bool pos = d32 > 0.0f;
    const float nh = pos ? Dp : Dm, eh = pos ? Ep : Em;
    const float nl = pos ? Dm : Dp, el = pos ? Em : Ep;
    c.qh_up = ((nh + eh) * r) * kUp;
    c.qh_dn = ((nh - eh) * r) * kDn;
    c.ql_up = ((nl + el) * r) * kUp;
    c.ql_dn = ((nl - el) * r) * kDn;
    return c;
}

// Exact FP64 candidate test and step ratios of one coordinate.
__device__ __forceinline__ bool exact_candidate(double x, double dk, double lbv, double ubv, double dtol, double thr,
                                            double &qh, double &ql) {
    const double Dp = ubv - x, Dm = x - lbv;
    if (!(Dp > dtol && Dm > dtol && fabs(dk) > thr)) return false;
    const double ad = fabs(dk);
    qh = (dk > 0.0 ? Dp : Dm) / ad;
    ql = (dk > 0.0 ? Dm : Dp) / ad;
    return true;
}

// Residual max|S x| with x in shared memory (reference findMaxAbs + the
// serial max, ACHRCuda.cu:232-240, 326-337; here CSR rows, no atomics).
__device__ __forceinline__ double residual_max(const ChainArgs &a, const double *xs, double *slot, int tid, int BD,
                                               int lane, int warp, int nwarps) {
    double mx = 0.0;
    for (int row = tid; row < a.m; row += BD) {
        double acc = 0.0;
        const int q1 = __ldg(a.row_ptr + row + 1);
        for (int q = __ldg(a.row_ptr + row); q < q1; ++q) acc = fma(__ldg(a.val + q), xs[__ldg(a.col_idx + q)], acc);
        mx = fmax(mx, fabs(acc));
    }
    return block_max(mx, slot, lane, warp, nwarps);
}

// x <- N (N^T x) in FP64 (reference reprojectPoint / reprojectPoint2,
// ACHRCuda.cu:208-230).  ys holds d doubles of shared scratch.
__device__ __forceinline__ void reproject(const ChainArgs &a, double *xs, double *ys, int tid, int BD, int lane,
                                          int warp, int nwarps) {
    const int n = a.n;
    for (int j = warp; j < a.d; j += nwarps) {
        const double *Nj = a.N + (size_t)j * (size_t)n;
        double acc = 0.0;
        for (int i = lane; i < n; i += 32) acc = fma(__ldg(Nj + i), xs[i], acc);
        acc = warp_sum(acc);
        if (lane == 0) ys[j] = acc;
    }
    __syncthreads();
    for (int i = tid; i < n; i += BD) {
        double acc = 0.0;
        for (int j = 0; j < a.d; ++j) acc = fma(__ldg(a.N + (size_t)j * (size_t)n + i), ys[j], acc);
        xs[i] = acc;
    }
    __syncthreads();
}

__device__ __forceinline__ void atomic_max_nonneg(unsigned long long *slot, double v) {
    if (v > 0.0) atomicMax(slot, (unsigned long long)__double_as_longlong(v));
}

}  // namespace

size_t chain_smem_bytes(int n, int d, int ldw, int block) {
    (void)block;
    const size_t npad = ((size_t)n + 15) & ~(size_t)15;
    const size_t wpad = ((size_t)ldw + 15) & ~(size_t)15;
    const size_t dpad = ((size_t)(d > 0 ? d : 1) + 15) & ~(size_t)15;
    return sizeof(double) * (2 * npad + wpad + dpad) + sizeof(RedSlots) + 64;
}

template <int EPT>
__global__ void __launch_bounds__(512, 1) achr_chain_kernel(const ChainArgs a) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int n = a.n;
    const int BD = blockDim.x, tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5, nwarps = BD >> 5;
    const size_t npad = ((size_t)n + 15) & ~(size_t)15;
    const size_t wpad = ((size_t)a.ldw + 15) & ~(size_t)15;
    const size_t dpad = ((size_t)(a.d > 0 ? a.d : 1) + 15) & ~(size_t)15;
    double *xs = reinterpret_cast<double *>(smem_raw);
    double *As = xs + npad;
    double *ws = As + npad;
    double *ys = ws + wpad;
    RedSlots *rs = reinterpret_cast<RedSlots *>(ys + dpad);
    uint64_t *bar = reinterpret_cast<uint64_t *>(rs + 1);
    int *exact_count = reinterpret_cast<int *>(bar + 1);

    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
        *exact_count = 0;
    }
    __syncthreads();

    const unsigned col_bytes = (unsigned)(sizeof(double) * (size_t)a.ldw);
    const float dtol32 = (float)a.d_tol;
    const float dtol_hi = dtol32 * kUp, dtol_lo = dtol32 * kDn;
    unsigned phase = 0;
    bool failed = false;
    long long n_acc = 0, n_rej = 0, n_chk = 0, n_rep = 0, n_stuck = 0, n_fin = 0;
    double worst_res = 0.0, worst_viol = 0.0;

    for (long long p = blockIdx.x; p < a.P && !failed; p += gridDim.x) {
        const unsigned long long chain = a.chain_offset + (unsigned long long)p;
        for (int i = tid; i < n; i += BD) {
            xs[i] = a.c0[i];
            As[i] = a.A0[i];
        }
        long long buf_col = -1;
        bool inflight = false, any_accepted = false, stuck = false;
        __syncthreads();

        for (int s = 0; s < a.T && !stuck && !failed; ++s) {
            const double inv = 1.0 / (double)(a.W + s + a.centre_offset);
            const Philox4 pd0 = step_draw(a.seed, chain, (uint32_t)s, 0u);
            const double U = step_uniform(pd0);
            for (int att = 0;; ++att) {
                if (att >= a.max_attempts) {
                    stuck = true;
                    break;
                }
                const Philox4 pd = (att == 0) ? pd0 : step_draw(a.seed, chain, (uint32_t)s, (uint32_t)att);
                const long long r = (long long)warmup_index(pd, (uint32_t)a.W);
                __syncthreads();  // previous readers of ws and of the reduction slots are done
                if (buf_col != r) {
                    if (inflight) {
                        if (!mbar_wait_bounded(bar, phase)) failed = true;
                        phase ^= 1u;
                        inflight = false;
                        __syncthreads();
                    }
                    if (tid == 0) {
                        fence_proxy_async_smem();
                        mbar_arrive_expect_tx(bar, col_bytes);
                        tma_load_1d(ws, a.warmup + (size_t)r * (size_t)a.ldw, col_bytes, bar);
                    }
                    inflight = true;
                    buf_col = r;
                }
                if (inflight) {
                    if (!mbar_wait_bounded(bar, phase)) failed = true;
                    phase ^= 1u;
                    inflight = false;
                }
                if (__syncthreads_or(failed ? 1 : 0)) {
                    failed = true;
                    break;
                }

                // Phase A: d = w_r - A / (W + t)  (reference ACHRCuda.cu:260-264)
                double dreg[EPT];
                double ss = 0.0;
#pragma unroll
                for (int k = 0; k < EPT; ++k) {
                    const int i = tid + k * BD;
                    double dk = 0.0;
                    if (i < n) dk = fma(-As[i], inv, ws[i]);
                    dreg[k] = dk;
                    ss = fma(dk, dk, ss);
                }
                ss = block_sum(ss, rs->sum, lane, warp, nwarps);
                const double norm = sqrt(ss);

                // Prefetch the next step's warmup column while this one is tested.
                if (s + 1 < a.T) {
                    const long long rn =
                        (long long)warmup_index(step_draw(a.seed, chain, (uint32_t)(s + 1), 0u), (uint32_t)a.W);
                    if (rn != buf_col) {
                        if (tid == 0) {
                            fence_proxy_async_smem();
                            mbar_arrive_expect_tx(bar, col_bytes);
                            tma_load_1d(ws, a.warmup + (size_t)rn * (size_t)a.ldw, col_bytes, bar);
                        }
                        inflight = true;
                        buf_col = rn;
                    }
                }
                if (!(norm > 0.0) || !isfinite(norm)) {
                    ++n_rej;
                    continue;
                }

                // Phase B1: FP32 brackets (reference ratio test ACHRCuda.cu:266-281)
                const double thr = a.u_tol * norm;
                const float uthr = (float)thr;
                const float uthr_hi = uthr * kUp, uthr_lo = uthr * kDn;
                float uh = INFINITY, ul = INFINITY;
                int fl = a.exact_ratio ? 2 : 0;
                if (!a.exact_ratio) {
#pragma unroll
                    for (int k = 0; k < EPT; ++k) {
                        const int i = tid + k * BD;
                        if (i < n) {
                            const Bracket c = bracket(xs[i], dreg[k], __ldg(a.bnd32 + i), dtol_hi, dtol_lo, uthr_hi,
                                                      uthr_lo);
                            if (c.st == ST_VALID) {
                                uh = fminf(uh, c.qh_up);
                                ul = fminf(ul, c.ql_up);
                                fl |= 1;
                            } else if (c.st == ST_AMBIG) {
                                fl |= 2;
                            }
                        }
                    }
                }
                uh = warp_minf(uh);
                ul = warp_minf(ul);
                fl = warp_or(fl);
                if (lane == 0) {
                    rs->fmin2[warp] = make_float2(uh, ul);
                    rs->flag2[warp] = fl;
                }
                __syncthreads();
                uh = INFINITY;
                ul = INFINITY;
                fl = 0;
                for (int w = 0; w < nwarps; ++w) {
                    const float2 v = rs->fmin2[w];
                    uh = fminf(uh, v.x);
                    ul = fminf(ul, v.y);
                    fl |= rs->flag2[w];
                }

                // Phase B2: FP64 evaluation of every coordinate whose bracket can
                // hold a minimum, or whose candidacy the brackets left open.
                double qh = INFINITY, ql = INFINITY;
                int anyv = 0, nex = 0;
#pragma unroll
                for (int k = 0; k < EPT; ++k) {
                    const int i = tid + k * BD;
                    if (i < n) {
                        const double xi = xs[i];
                        bool contender = a.exact_ratio != 0;
                        if (!contender) {
                            const Bracket c =
                                bracket(xi, dreg[k], __ldg(a.bnd32 + i), dtol_hi, dtol_lo, uthr_hi, uthr_lo);
                            contender = (c.st == ST_AMBIG) ||
                                        (c.st == ST_VALID && (c.qh_dn <= uh || c.ql_dn <= ul));
                        }
                        if (contender) {
                            ++nex;
                            double eh, el;
                            if (exact_candidate(xi, dreg[k], __ldg(a.lb + i), __ldg(a.ub + i), a.d_tol, thr, eh, el)) {
                                qh = fmin(qh, eh);
                                ql = fmin(ql, el);
                                anyv = 1;
                            }
                        }
                    }
                }
                if (nex) atomicAdd(exact_count, nex);
                qh = warp_min(qh);
                ql = warp_min(ql);
                anyv = warp_or(anyv);
                if (lane == 0) {
                    rs->dmin2[warp] = make_double2(qh, ql);
                    rs->flag3[warp] = anyv;
                }
                __syncthreads();
                qh = INFINITY;
                ql = INFINITY;
                anyv = 0;
                for (int w = 0; w < nwarps; ++w) {
                    const double2 v = rs->dmin2[w];
                    qh = fmin(qh, v.x);
                    ql = fmin(ql, v.y);
                    anyv |= rs->flag3[w];
                }

                // Rejection test (reference ACHRCuda.cu:316-319; no candidate = rejection)
                const double maxStep = qh * norm, minStep = -(ql * norm);
                if (!anyv || (fabs(minStep) < a.max_min_tol && fabs(maxStep) < a.max_min_tol) ||
                    minStep > maxStep) {
                    ++n_rej;
                    continue;
                }
                // t / ||d|| with t = U (max - min) + min (reference ACHRCuda.cu:314)
                const double sstep = fma(U, qh + ql, -ql);

                // Phase C: x = prev + t u (ACHRCuda.cu:242-249), residual check every
                // check_period steps (:325-344), clip + centre (:193-206, :347-350).
                const bool check = (s % a.check_period) == 0;
                if (!check) {
#pragma unroll
                    for (int k = 0; k < EPT; ++k) {
                        const int i = tid + k * BD;
                        if (i < n) {
                            const double xn = fma(sstep, dreg[k], xs[i]);
                            const double xc = fmin(fmax(xn, __ldg(a.lb + i)), __ldg(a.ub + i));
                            xs[i] = xc;
                            As[i] += xc;
                        }
                    }
                } else {
#pragma unroll
                    for (int k = 0; k < EPT; ++k) {
                        const int i = tid + k * BD;
                        if (i < n) xs[i] = fma(sstep, dreg[k], xs[i]);
                    }
                    __syncthreads();
                    ++n_chk;
                    const double mx = residual_max(a, xs, rs->mx, tid, BD, lane, warp, nwarps);
                    if (mx > a.residual_tol) {
                        ++n_rep;
                        reproject(a, xs, ys, tid, BD, lane, warp, nwarps);
                    }
#pragma unroll
                    for (int k = 0; k < EPT; ++k) {
                        const int i = tid + k * BD;
                        if (i < n) {
                            const double xc = fmin(fmax(xs[i], __ldg(a.lb + i)), __ldg(a.ub + i));
                            xs[i] = xc;
                            As[i] += xc;
                        }
                    }
                }
                ++n_acc;
                any_accepted = true;
                break;
            }
        }
        if (inflight) {
            if (!mbar_wait_bounded(bar, phase)) failed = true;
            phase ^= 1u;
            inflight = false;
        }
        if (stuck) ++n_stuck;
        __syncthreads();
        if (__syncthreads_or(failed ? 1 : 0)) {
            failed = true;
            break;
        }

        // Emitted point: residual / bound diagnostics and, on request, the final
        // feasibility projection (project, clip, re-check).
        if (any_accepted) {
            double res = residual_max(a, xs, rs->mx, tid, BD, lane, warp, nwarps);
            if (a.final_project && res > a.feasibility_tol) {
                ++n_fin;
                __syncthreads();
                reproject(a, xs, ys, tid, BD, lane, warp, nwarps);
                for (int i = tid; i < n; i += BD) xs[i] = fmin(fmax(xs[i], __ldg(a.lb + i)), __ldg(a.ub + i));
                __syncthreads();
                res = residual_max(a, xs, rs->viol, tid, BD, lane, warp, nwarps);
            }
            double viol = 0.0;
            for (int i = tid; i < n; i += BD) {
                const double xi = xs[i];
                viol = fmax(viol, fmax(__ldg(a.lb + i) - xi, xi - __ldg(a.ub + i)));
            }
            __syncthreads();
            viol = block_max(viol, rs->viol, lane, warp, nwarps);
            worst_res = fmax(worst_res, res);
            worst_viol = fmax(worst_viol, viol);
        }
        for (int i = tid; i < n; i += BD) a.out[(size_t)i * (size_t)a.ld_out + (size_t)p] = any_accepted ? xs[i] : 0.0;
        __syncthreads();
    }

    __syncthreads();
    if (tid == 0) {
        unsigned long long *c = a.counters;
        if (n_acc) atomicAdd(c + CNT_ACCEPTED, (unsigned long long)n_acc);
        if (n_rej) atomicAdd(c + CNT_REJECTED, (unsigned long long)n_rej);
        if (n_chk) atomicAdd(c + CNT_CHECKS, (unsigned long long)n_chk);
        if (n_rep) atomicAdd(c + CNT_REPROJ, (unsigned long long)n_rep);
        if (n_stuck) atomicAdd(c + CNT_STUCK, (unsigned long long)n_stuck);
        if (n_fin) atomicAdd(c + CNT_FINAL_PROJ, (unsigned long long)n_fin);
        if (*exact_count) atomicAdd(c + CNT_EXACT, (unsigned long long)*exact_count);
        atomic_max_nonneg(c + CNT_MAXRES_BITS, worst_res);
        atomic_max_nonneg(c + CNT_MAXVIOL_BITS, worst_viol);
        if (failed) atomicOr(c + CNT_ERROR, ERR_TMA_TIMEOUT);
    }
}

int chain_block_size(int n, int threads_per_chain) {
    if (threads_per_chain > 0) return threads_per_chain;
    int bd = 32 * ((n + 32 * 16 - 1) / (32 * 16));
    if (bd < 32) bd = 32;
    if (bd > 512) bd = 512;
    return bd;
}

static int pick_ept(int n, int bd) {
    const int need = (n + bd - 1) / bd;
    if (need <= 1) return 1;
    if (need <= 2) return 2;
    if (need <= 4) return 4;
    if (need <= 8) return 8;
    if (need <= 16) return 16;
    if (need <= 32) return 32;
    return 0;
}

template <int EPT>
static cudaError_t launch_ept(const ChainArgs &a, int bd, size_t smem, cudaStream_t stream) {
    cudaError_t e = cudaFuncSetAttribute(achr_chain_kernel<EPT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, achr_chain_kernel<EPT>, bd, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long long grid = (long long)sms * per_sm;
    if (grid > a.P) grid = a.P;
    if (grid < 1) return cudaSuccess;
    achr_chain_kernel<EPT><<<(unsigned)grid, bd, smem, stream>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_chains(const ChainArgs &a, int threads_per_chain, cudaStream_t stream) {
    if (a.P <= 0) return cudaSuccess;
    const int bd = chain_block_size(a.n, threads_per_chain);
    if (bd % 32 != 0 || bd < 32 || bd > 512) return cudaErrorInvalidValue;
    const int ept = pick_ept(a.n, bd);
    const size_t smem = chain_smem_bytes(a.n, a.d, a.ldw, bd);
    switch (ept) {
        case 1: return launch_ept<1>(a, bd, smem, stream);
        case 2: return launch_ept<2>(a, bd, smem, stream);
        case 4: return launch_ept<4>(a, bd, smem, stream);
        case 8: return launch_ept<8>(a, bd, smem, stream);
        case 16: return launch_ept<16>(a, bd, smem, stream);
        case 32: return launch_ept<32>(a, bd, smem, stream);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace achr
