#pragma once
// Persistent chain kernel: the ACHR sampling hot loop on sm_103a.
// (Template; instantiated for each block-size / elements-per-thread pair in
// achr_chain_cfg_*.cu, dispatched by achr_chain_launch.cu.)
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
//     (cp.async.bulk + mbarrier) issued one step ahead.
//   * GB300's FP64 pipe issues about 1.6 DFMA per clock per SM, 72x less than
//     FP32, and FP64 compares cost as much as FMAs.  Per element and accepted
//     step the kernel spends exactly three FP64 pipe instructions
//     (d = w - A/(W+t), x += s d, A += x).  The norm is summed in FP32 (it only
//     feeds tolerance tests, which carry margins and fall back to FP64 when a
//     margin is not enough); the ratio test brackets every bound distance and
//     ratio in FP32 with rigorous error bounds and evaluates in FP64 only the
//     coordinates whose bracket can hold the minimum; clipping and the min/max
//     reductions compare FP64 values as integers (order-preserving keys).
//   * The brackets are formed in the same pass as d, before the block knows
//     ||d||, so one block reduction serves the norm and the bracket minima
//     (two barriers per accepted step: that one and the exact minima's).
//   * Per-step scalars (warmup index, step uniform, 1/(W+t)) come from a
//     shared-memory table that the CTA refills once every BD steps.
//   * The element loops are unrolled over compile-time BD x EPT with arrays
//     padded to that length, so no loop carries a bounds test.
//   * Reductions are warp shuffles plus one shared-memory exchange in a fixed
//     order, so a launch is bitwise repeatable.
#include <algorithm>
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
constexpr float kNormUp = 1.0f + 1e-5f;                // FP32 norm relative error margin
constexpr float kNormDn = 1.0f - 1e-5f;
// Lower bound of u_tol ||d|| from u_tol max|d_i|: the FP32 norm of a vector is
// at least its largest element within (1 - 1e-6), and the threshold carries
// the kNormDn margin; 0.999 leaves room for both and the products' rounding.
constexpr float kProvDn = 0.999f;
constexpr unsigned long long kWaitNs = 2000000000ull;  // bounded mbarrier wait: 2 s
constexpr unsigned long long kInfBits = 0x7FF0000000000000ull;

// FP64 -> FP32 rounding toward zero with integer operations only.
// |v - f| <= 2^-23 |f| + 2^-126; tiny values flush to signed zero, overflow
// and inf map to inf.
__device__ __forceinline__ float f64_to_f32_rz(double v) {
    const unsigned hi = (unsigned)__double2hiint(v);
    const unsigned lo = (unsigned)__double2loint(v);
    const int fe = (int)((hi >> 20) & 0x7FFu) - 896;  // re-bias 1023 -> 127
    unsigned mag = ((unsigned)fe << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29);
    mag = (fe <= 0) ? 0u : mag;
    mag = (fe >= 255) ? 0x7F800000u : mag;
    return __uint_as_float((hi & 0x80000000u) | mag);
}

// Order-preserving integer key of a double (sign-magnitude -> two's
// complement; -0 and +0 share key 0).  a < b  <=>  key(a) < key(b) for non-NaN.
__device__ __forceinline__ long long order_key(double v) {
    const long long b = __double_as_longlong(v);
    const long long mag = b & 0x7FFFFFFFFFFFFFFFll;
    return b < 0 ? -mag : mag;
}

// Exact clip of x to [lb, ub] (reference correctBounds, ACHRCuda.cu:198-202):
// x itself when inside, else the bound, compared through integer keys.
__device__ __forceinline__ double clip_exact(double x, double2 lu) {
    const long long kx = order_key(x);
    double r = x;
    if (kx < order_key(lu.x)) r = lu.x;
    if (kx > order_key(lu.y)) r = lu.y;
    return r;
}

// (lb, ub) of one reaction.  A volatile load, so that the compiler keeps it
// (and the FP64 work that depends on it) inside the rarely taken branches.
// |v| and its bit pattern through integer operations (fabs on a double can be
// issued to the FP64 pipe).
__device__ __forceinline__ unsigned long long abs_bits(double v) {
    return (unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull;
}
__device__ __forceinline__ double abs_int(double v) { return __longlong_as_double((long long)abs_bits(v)); }
__device__ __forceinline__ bool positive_int(double v) {  // v > 0 for non-NaN v
    const long long b = __double_as_longlong(v);
    return b > 0;
}

// r[k] for a run-time k without indexing the register array dynamically.
template <int EPT>
__device__ __forceinline__ double pick(const double (&r)[EPT], int k) {
    double v = r[0];
#pragma unroll
    for (int j = 1; j < EPT; ++j) v = (j == k) ? r[j] : v;
    return v;
}

__device__ __forceinline__ double2 ld_lbub(const double2 *p) {
    double2 v;
    asm volatile("ld.global.nc.v2.f64 {%0, %1}, [%2];" : "=d"(v.x), "=d"(v.y) : "l"(p));
    return v;
}

// FP32 test that x (as its truncation x32) lies strictly inside (lb, ub):
// true only when the bracket arithmetic proves it; false means "test exactly".
__device__ __forceinline__ bool surely_inside(float x32, float2 b, float berr) {
    const float ex = fmaf(fabsf(x32), kErrK, kTiny + berr);
    return (x32 - b.x) > ex && (b.y - x32) > ex;
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

// Wait for the phase with the given parity to complete, giving up after limit_ns.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, unsigned parity,
                                                  unsigned long long limit_ns = kWaitNs) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    for (;;) {
        if (mbar_try_wait(bar, parity)) return true;
        if (global_ns() - t0 > limit_ns) return false;
    }
}

__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

template <class T>
__device__ __forceinline__ T umin(T a, T b) {
    return a < b ? a : b;
}
template <class T>
__device__ __forceinline__ T umax(T a, T b) {
    return a > b ? a : b;
}

// Warp minima with the single-instruction integer reductions (redux.sync)
// instead of five shuffle rounds: floats through an order-preserving key,
// 64-bit keys as (high word, then low word among the lanes holding the high
// minimum).
__device__ __forceinline__ unsigned f32_key(float f) {
    const unsigned b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float key_f32(unsigned k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}
__device__ __forceinline__ float warp_min_f32(float v) {
    return key_f32(__reduce_min_sync(0xffffffffu, f32_key(v)));
}
__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
    const unsigned hi = (unsigned)(v >> 32);
    const unsigned mhi = __reduce_max_sync(0xffffffffu, hi);
    const unsigned mlo = __reduce_max_sync(0xffffffffu, hi == mhi ? (unsigned)v : 0u);
    return ((unsigned long long)mhi << 32) | mlo;
}
__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v) {
    const unsigned hi = (unsigned)(v >> 32);
    const unsigned mhi = __reduce_min_sync(0xffffffffu, hi);
    const unsigned mlo = __reduce_min_sync(0xffffffffu, hi == mhi ? (unsigned)v : 0xffffffffu);
    return ((unsigned long long)mhi << 32) | mlo;
}

// Shared-memory exchange slots, two sets selected by attempt parity so that
// consecutive attempts never overwrite slots another warp may still read.
struct RedSlots {
    float sum1[32];
    int flag1[32];
    float2 min2[32];
    int flag2[32];
    ulonglong2 min3[32];
    int flag3[32];
    unsigned long long max4[32];
    double sum5[32];
};

struct StepEntry {
    double U;      // step uniform of attempt 0
    double inv;    // 1 / (W + t + centre_offset)
    unsigned idx;  // warmup index of attempt 0
    unsigned pad;
};

// FP32 bracket of one coordinate's ratio-test contribution (reference
// fillrandPoint, ACHRCuda.cu:266-281: a coordinate is a candidate when
// distUb > dTol, distLb > dTol and |u_i| > uTol).  Writes the lower ends of
// the two ratio brackets: NaN = certainly not a candidate, -inf = undecided
// (evaluate in FP64), else the bracket's lower end; and folds the upper ends
// of certain candidates into the running minima.
__device__ __forceinline__ void bracket(double x, double dk, float2 b, float berr, float dtol_hi, float dtol_lo,
                                        float uthr_hi, float uthr_lo, float &lo_h, float &lo_l, float &uh, float &ul,
                                        int &fl) {
    const float x32 = f64_to_f32_rz(x);
    const float d32 = f64_to_f32_rz(dk);
    const float ad = fabsf(d32);
    const float Dp = b.y - x32;  // ub - x
    const float Dm = x32 - b.x;  // x - lb
    const float ex = fmaf(fabsf(x32), kErrK, kTiny + berr);
    const float Ep = fmaf(fabsf(Dp), kErrK, ex);
    const float Em = fmaf(fabsf(Dm), kErrK, ex);
    const bool p_ok = (Dp - Ep) > dtol_hi, p_bad = (Dp + Ep) <= dtol_lo;
    const bool m_ok = (Dm - Em) > dtol_hi, m_bad = (Dm + Em) <= dtol_lo;
    const bool u_ok = ad > uthr_hi, u_bad = ad * kAdUp < uthr_lo;
    const bool bad = p_bad || m_bad || u_bad;
    const bool ok = p_ok && m_ok && u_ok;
    const float r = rcp_approx(ad);
    const bool pos = d32 > 0.0f;
    const float nh = pos ? Dp : Dm, eh = pos ? Ep : Em;
    const float nl = pos ? Dm : Dp, el = pos ? Em : Ep;
    const float rup = r * kUp, rdn = r * kDn;
    const float qh_up = (nh + eh) * rup, qh_dn = (nh - eh) * rdn;
    const float ql_up = (nl + el) * rup, ql_dn = (nl - el) * rdn;
    if (ok) {
        uh = fminf(uh, qh_up);
        ul = fminf(ul, ql_up);
    }
    lo_h = ok ? qh_dn : (bad ? __int_as_float(0x7fc00000) : -INFINITY);
    lo_l = ok ? ql_dn : (bad ? __int_as_float(0x7fc00000) : -INFINITY);
    fl |= ok ? 1 : 0;
    fl |= (!ok && !bad) ? 2 : 0;
    fl |= (!ok && !bad && !u_ok && !u_bad) ? 4 : 0;  // needs the FP64 norm
}

// Largest |(S x)_i| over this thread's rows, as the bits of a non-negative
// double (reference findMaxAbs, ACHRCuda.cu:232-240, on the rows thread tid
// owns: tid, tid + BD, ...; a warp's 32 lanes own 32 consecutive rows).  With
// the sliced-ELL copy of S each warp's loads of one nonzero slot are one
// coalesced segment; without it (caller-owned models) the CSR rows are read
// directly.  Both visit a row's nonzeros in the same order, so the sums are
// bitwise equal (the ELL padding adds 0 * x_0).
template <int BD>
__device__ __forceinline__ unsigned long long residual_max_bits(const ChainArgs &a, const double *xs, int tid) {
    unsigned long long mx = 0;
    if (a.sell_off) {
        const int lane = tid & 31;
        for (int g = tid >> 5; g < a.sell_groups; g += BD / 32) {
            const int base = __ldg(a.sell_off + g);
            const int len = (__ldg(a.sell_off + g + 1) - base) >> 5;
            double acc = 0.0;
#pragma unroll 4
            for (int t = 0; t < len; ++t) {  // unrolled so the loads of 4 slots are in flight together
                const int q = base + (t << 5) + lane;
                acc = fma(__ldg(a.sell_val + q), xs[__ldg(a.sell_col + q)], acc);
            }
            mx = umax(mx, abs_bits(acc));
        }
    } else {
        for (int row = tid; row < a.m; row += BD) {
            double acc = 0.0;
            const int q1 = __ldg(a.row_ptr + row + 1);
            for (int q = __ldg(a.row_ptr + row); q < q1; ++q) acc = fma(__ldg(a.val + q), xs[__ldg(a.col_idx + q)], acc);
            mx = umax(mx, abs_bits(acc));
        }
    }
    return mx;
}

// The same row sums as residual_max_bits (same rows, same order of terms, so
// the same maximum), each stored to rr[row] (device row order) for the
// batched reprojection of segmented sampling.
template <int BD>
__device__ __forceinline__ unsigned long long residual_rows(const ChainArgs &a, const double *xs, double *rr, int tid) {
    unsigned long long mx = 0;
    if (a.sell_off) {
        const int lane = tid & 31;
        for (int g = tid >> 5; g < a.sell_groups; g += BD / 32) {
            const int base = __ldg(a.sell_off + g);
            const int len = (__ldg(a.sell_off + g + 1) - base) >> 5;
            double acc = 0.0;
#pragma unroll 4
            for (int t = 0; t < len; ++t) {
                const int q = base + (t << 5) + lane;
                acc = fma(__ldg(a.sell_val + q), xs[__ldg(a.sell_col + q)], acc);
            }
            mx = umax(mx, abs_bits(acc));
            const int row = (g << 5) + lane;
            if (row < a.m) rr[row] = acc;
        }
    } else {
        for (int row = tid; row < a.m; row += BD) {
            double acc = 0.0;
            const int q1 = __ldg(a.row_ptr + row + 1);
            for (int q = __ldg(a.row_ptr + row); q < q1; ++q) acc = fma(__ldg(a.val + q), xs[__ldg(a.col_idx + q)], acc);
            mx = umax(mx, abs_bits(acc));
            rr[row] = acc;
        }
    }
    return mx;
}

// 0.0 from a volatile asm statement.  A computation that starts from it stays
// inside the branch that guards it: without it the compiler may compute the
// FP64 norm of d (one DFMA per element, which almost no step needs) ahead of
// its branch on every step, as it did in the segmented instantiation (a third
// more FP64 work per step on the pipe that bounds this kernel).
__device__ __forceinline__ double fp64_zero_here() {
    double z;
    asm volatile("mov.b64 %0, 0;" : "=d"(z));
    return z;
}

// FP32 -> FP64 with integer operations only (exact for normal values; zero and
// subnormal values give a signed zero).
__device__ __forceinline__ double f32_to_f64_exact(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xFFu;
    const unsigned long long s = (unsigned long long)(u & 0x80000000u) << 32;
    if (e == 0) return __longlong_as_double((long long)s);
    return __longlong_as_double(
        (long long)(s | ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)(u & 0x7FFFFFu) << 29)));
}

// BF16 bits of f rounded to nearest even (hi) and of the remainder f - hi (lo),
// for finite f; FP32 and integer operations only.
__device__ __forceinline__ void split_bf16_bits(float f, unsigned short &hi, unsigned short &lo) {
    const unsigned u = __float_as_uint(f);
    const unsigned hu = (u + 0x7FFFu + ((u >> 16) & 1u)) & 0xFFFF0000u;
    hi = (unsigned short)(hu >> 16);
    const unsigned r = __float_as_uint(f - __uint_as_float(hu));
    const unsigned ru = (r + 0x7FFFu + ((r >> 16) & 1u)) & 0xFFFF0000u;
    lo = (unsigned short)(ru >> 16);
}

// x <- x - S^T z, z = (S S^T)^+ S x: the reference's N (N^T x) written through
// the residual (equal in exact arithmetic).  S x is summed in FP64 over the
// same rows as the check and kept as FP32 hi + lo pairs in rr (m entries of
// the staging buffer); z = (S S^T)^+ r runs in FP32 (a warp per row of the
// pseudo-inverse, coalesced), whose relative error (~1e-7 times the condition
// number) applies to the correction, not to x, which is at most of the size of
// the residual's preimage; the update x_j -= sum_i S_ij z_i is FP64 (CSC).
template <int BD>
__device__ __forceinline__ void residual_form_reproject(const ChainArgs &a, double *xs, float2 *rr, float *zs,
                                                        int tid) {
    constexpr int NW = BD / 32;
    const int lane = tid & 31, warp = tid >> 5;
    const int m = a.m;
    if (a.sell_off) {
        for (int g = warp; g < a.sell_groups; g += NW) {
            const int base = __ldg(a.sell_off + g);
            const int len = (__ldg(a.sell_off + g + 1) - base) >> 5;
            double acc = 0.0;
#pragma unroll 4
            for (int t = 0; t < len; ++t) {
                const int q = base + (t << 5) + lane;
                acc = fma(__ldg(a.sell_val + q), xs[__ldg(a.sell_col + q)], acc);
            }
            const int row = (g << 5) + lane;
            if (row < m) {
                const float hi = __double2float_rn(acc);
                rr[row] = make_float2(hi, __double2float_rn(acc - (double)hi));
            }
        }
    } else {
        for (int row = tid; row < m; row += BD) {
            double acc = 0.0;
            const int q1 = __ldg(a.row_ptr + row + 1);
            for (int q = __ldg(a.row_ptr + row); q < q1; ++q) acc = fma(__ldg(a.val + q), xs[__ldg(a.col_idx + q)], acc);
            const float hi = __double2float_rn(acc);
            rr[row] = make_float2(hi, __double2float_rn(acc - (double)hi));
        }
    }
    __syncthreads();
    for (int i = warp; i < m; i += NW) {
        const float *Bi = a.pinv32 + (size_t)i * (size_t)m;
        float acc = 0.0f;
        for (int k = lane; k < m; k += 32) {
            const float b = __ldg(Bi + k);
            const float2 r = rr[k];
            acc = fmaf(b, r.x, fmaf(b, r.y, acc));
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) zs[i] = acc;
    }
    __syncthreads();
    for (int j = tid; j < a.n; j += BD) {
        double dl = 0.0;
        const int q1 = __ldg(a.csc_ptr + j + 1);
        for (int q = __ldg(a.csc_ptr + j); q < q1; ++q) dl = fma(__ldg(a.csc_val + q), (double)zs[__ldg(a.csc_row + q)], dl);
        xs[j] -= dl;
    }
}

// Bytes of one staged warmup column (the leading dimension is even, so a
// multiple of 16).
__device__ __forceinline__ unsigned column_bytes(const ChainArgs &a) {
    return (unsigned)(sizeof(double) * (size_t)a.ldw);
}

}  // namespace

constexpr int kTbl = 64;  // steps per refill of the step table

// Shared memory of one CTA: xs, As, ws (NP doubles each; ws doubles as the
// reprojection scratch), the step table and the reduction slots.
__host__ __device__ inline size_t chain_smem_bytes_cfg(int np, int d, int bd) {
    (void)d;
    (void)bd;
    return sizeof(double) * 3 * (size_t)np + sizeof(StepEntry) * kTbl + 2 * sizeof(RedSlots) + 128;
}

// Shared-memory header of a CTA: x, A and the staging buffer (3 NP doubles),
// the step table, two reduction slots, then the column barrier, eight
// statistics counters, the exact-evaluation count (two ints), the `never`
// barrier and the two worst-case words.
template <int NP>
__device__ __forceinline__ void chain_barriers(unsigned char *smem_raw, uint64_t *&bar, uint64_t *&never) {
    RedSlots *rsb = reinterpret_cast<RedSlots *>(reinterpret_cast<StepEntry *>(reinterpret_cast<double *>(smem_raw) +
                                                                               3 * (size_t)NP) +
                                                 kTbl);
    bar = reinterpret_cast<uint64_t *>(rsb + 2);
    never = reinterpret_cast<uint64_t *>(reinterpret_cast<int *>(bar + 1 + 8) + 2);
}

// Entries e = tid, tid + BD, ... < kTbl of the step table for steps s + e below
// `end`: the step's Philox draw (uniform and warmup index) and 1 / (W + t).
template <int BD>
__device__ __forceinline__ void fill_step_table(const ChainArgs &a, StepEntry *tbl, unsigned long long chain, int s,
                                                int end, int tid) {
    for (int e = tid; e < kTbl; e += BD) {
        const int st = s + e;
        if (st < end) {
            const Philox4 pd = step_draw(a.seed, chain, (uint32_t)st, 0u);
            StepEntry en;
            en.U = step_uniform(pd);
            en.inv = 1.0 / (double)(a.W + st + a.centre_offset);
            en.idx = warmup_index(pd, (uint32_t)a.W);
            en.pad = 0;
            tbl[e] = en;
        }
    }
}

// One CTA's share of a launch: chains p_begin, p_begin + p_step, ... below
// p_end of the model `a` describes, then the CTA's statistics into
// a.counters.  The staging barriers live in the shared-memory header; the
// caller initialises them once per CTA and `phase` carries their parity from
// one call to the next.  Returns true when a bounded wait ran out.
// SEG: segmented launches of the deferred reprojection (a separate
// instantiation, so the plain kernel carries none of its code or registers).
template <int BD, int EPT, bool SEG>
__device__ __forceinline__ bool chain_run(const ChainArgs &a, int p_begin, int p_step, int p_end,
                                          unsigned char *smem_raw, unsigned &phase) {
    constexpr int NP = BD * EPT;
    constexpr int NW = BD / 32;
    const int tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    double *xs = reinterpret_cast<double *>(smem_raw);
    double *As = xs + NP;
    double *ws = As + NP;
    double *ys = ws;  // reprojection scratch (d <= n entries, below the zero padding of ws)
    StepEntry *tbl = reinterpret_cast<StepEntry *>(ws + NP);
    RedSlots *rsb = reinterpret_cast<RedSlots *>(tbl + kTbl);
    uint64_t *bar, *never;  // the staged column's barrier; a barrier nothing arrives on
    chain_barriers<NP>(smem_raw, bar, never);
    unsigned long long *cnt = reinterpret_cast<unsigned long long *>(bar + 1);  // CTA statistics, CNT_* slots
    int *exact_count = reinterpret_cast<int *>(cnt + 8);
    // largest residual and bound violation of the CTA's emitted points (bits of non-negative doubles)
    unsigned long long *worst = reinterpret_cast<unsigned long long *>(never + 1);
    // (S S^T)^+ r of the residual-form reprojection (m floats), when enabled
    float *zs = reinterpret_cast<float *>(smem_raw + chain_smem_bytes_cfg(NP, a.d, BD));

    if (tid == 0) {
        *exact_count = 0;
        for (int c = 0; c < 8; ++c) cnt[c] = 0;
        worst[0] = worst[1] = 0;
    }
    // The TMA copy fills ws[0, ldw); the padding beyond stays zero.
#pragma unroll
    for (int k = 0; k < EPT; ++k) ws[tid + k * BD] = 0.0;
    __syncthreads();

    const bool hr = a.hit_and_run != 0;  // directions are the staged columns themselves (no centre)
    const bool merged = a.merged_ab != 0 && !a.exact_ratio;  // ratio-test brackets formed in phase A
    const float uthr_max = a.uthr_max;
    // A warp whose 32 elements of the last slot (k = EPT - 1) all lie in the
    // padding (i >= n) skips that slot: its coordinates stay 0 and its d is 0,
    // so the FP64 operations on it would change nothing.
    const bool tail_live = warp * 32 + (EPT - 1) * BD < a.n;
// (Not for 32 elements per thread, where the branches cost more registers than they save.)
#define ACHR_PAD_SLOT(k) (EPT < 32 && (k) == EPT - 1 && !tail_live)
    unsigned it = 0;
    bool failed = false;

    // (Scalars that stay constant over a launch are read from the kernel
    // parameters where they are used rather than held in registers.)
    for (int p = p_begin; p < p_end && !failed; p = (int)min((long long)p + p_step, (long long)p_end)) {
#define ACHR_CHAIN_ID (a.chain_offset + (unsigned long long)p)
        // Segmented sampling: the chain's state bits from the earlier launches.
        const unsigned sflags = SEG ? a.seg_flags[p] : 0u;
        if (sflags & SEG_STARTED) {
#pragma unroll
            for (int k = 0; k < EPT; ++k) {
                const int i = tid + k * BD;
                const bool real = i < a.n;
                xs[i] = real ? a.seg_x[(size_t)p * (size_t)a.ld_seg + (size_t)i] : 0.0;
                As[i] = real ? a.seg_A[(size_t)p * (size_t)a.ld_seg + (size_t)i] : 0.0;
            }
        } else if (a.x_in) {  // resume: the chain's point and centre accumulator after step0 steps
#pragma unroll
            for (int k = 0; k < EPT; ++k) {
                const int i = tid + k * BD;
                const bool real = i < a.n;
                xs[i] = real ? a.x_in[(size_t)i * (size_t)a.ld_state + (size_t)p] : 0.0;
                As[i] = real ? a.A_in[(size_t)i * (size_t)a.ld_state + (size_t)p] : 0.0;
            }
        } else {
#pragma unroll
            for (int k = 0; k < EPT; ++k) {
                const int i = tid + k * BD;
                xs[i] = a.c0[i];
                As[i] = a.A0[i];
            }
        }
        int buf_col = -1;
        bool inflight = false, any_accepted = a.x_in != nullptr || (sflags & SEG_ACCEPTED), stuck = false;
        bool seg_pending = false;  // this launch ended the chain after a check step's update
        const bool was_stuck = (sflags & SEG_STUCK) != 0;
        if (was_stuck) stuck = true;  // stopped in an earlier launch: no more steps
        if (sflags & SEG_CORR) {
            // The batched passes' correction of this chain, x <- x - S^T z summed over
            // the passes, held as a double-float pair: two FP64 subtractions per
            // reaction (the FP32 -> FP64 conversions are integer operations).
#pragma unroll
            for (int k = 0; k < EPT; ++k) {
                const int i = tid + k * BD;
                if (i < a.n) {
                    const size_t o = (size_t)p * (size_t)a.ld_seg + (size_t)i;
                    xs[i] = (xs[i] - f32_to_f64_exact(a.seg_dxh[o])) - f32_to_f64_exact(a.seg_dxl[o]);
                }
            }
        }
        if (sflags & SEG_PENDING) {
            // Finish the check step the previous launch ended on (the batched
            // pass has reprojected the point if its residual was above the
            // tolerance): clip, then add the point to the centre accumulator.
            unsigned edge = 0;
#pragma unroll
            for (int k = 0; k < EPT; ++k) {
                const int i = tid + k * BD;
                if (ACHR_PAD_SLOT(k)) continue;
                const double xv = xs[i];
                if (surely_inside(f64_to_f32_rz(xv), __ldg(a.bnd + i), a.bound_err)) {
                    if (!hr) As[i] += xv;
                } else {
                    edge |= 1u << k;
                }
            }
            for (; edge; edge &= edge - 1) {
                const int i = tid + (__ffs(edge) - 1) * BD;
                const double xc = clip_exact(xs[i], ld_lbub(a.lbub + i));
                xs[i] = xc;
                if (!hr) As[i] += xc;
            }
        }
        // The reference checks when the step count is a multiple of the period
        // (ACHRCuda.cu:325); a period of INT_MAX stands for "never".
        int chk = a.check_period == 0x7fffffff ? 1 : a.step0 % a.check_period;
        int tbase = a.step0 - kTbl;

        for (int s = a.step0; s < (a.step0 + a.T) && !stuck && !failed && !seg_pending; ++s) {
            if (s - tbase >= kTbl) {
                // refill the step table: entry e holds step tbase + e
                tbase = s;
                __syncthreads();
                fill_step_table<BD>(a, tbl, ACHR_CHAIN_ID, s, a.step0 + a.T, tid);
                __syncthreads();
            }
            // this step's table entry (its fields are read where they are used)
            const StepEntry *te = tbl + (s - tbase);
            for (int att = 0;; ++att, ++it) {
                if (att >= a.max_attempts) {
                    stuck = true;
                    break;
                }
                RedSlots *rs = rsb + (it & 1u);
                const int r = att == 0
                                  ? (int)te->idx
                                  : (int)warmup_index(step_draw(a.seed, ACHR_CHAIN_ID, (uint32_t)s, (uint32_t)att),
                                                                  (uint32_t)a.W);
                if (buf_col != r) {
                    if (inflight) {
                        if (!mbar_wait_bounded(bar, phase)) failed = true;
                        phase ^= 1u;
                        inflight = false;
                    }
                    __syncthreads();  // every thread has seen the previous phase complete
                    if (r < 0 || r >= a.W) {  // never copy from outside the warmup matrix
                        failed = true;
                        break;
                    }
                    if (tid == 0) {
                        fence_proxy_async_smem();
                        mbar_arrive_expect_tx(bar, column_bytes(a));
                        tma_load_1d(ws, a.warmup + (size_t)r * (size_t)a.ldw, column_bytes(a), bar);
                    }
                    inflight = true;
                    buf_col = r;
                }
                if (inflight) {
                    // a.wait_never (failure-detection test): the wait is on a barrier
                    // that nothing completes, so it always runs out.
                    if (!mbar_wait_bounded(a.wait_never ? never : bar, phase, a.wait_ns ? a.wait_ns : kWaitNs)) {
                        // The column did not arrive within the caller's limit: record it,
                        // then let the copy land (default limit) before the buffer is left.
                        failed = true;
                        mbar_wait_bounded(bar, phase);
                    }
                    phase ^= 1u;
                    inflight = false;
                }

                // Phase A: d = w_r - A / (W + t)  (reference ACHRCuda.cu:260-264);
                // in hit-and-run mode the staged column is the direction itself.
                double dreg[EPT];
                float ss = 0.0f, admax = 0.0f;
                if (hr) {
#pragma unroll
                    for (int k = 0; k < EPT; ++k) {
                        const int i = tid + k * BD;
                        if (ACHR_PAD_SLOT(k)) {
                            dreg[k] = 0.0;
                            continue;
                        }
                        const double dk = ws[i];
                        dreg[k] = dk;
                        const float d32 = f64_to_f32_rz(dk);
                        ss = fmaf(d32, d32, ss);
                        admax = fmaxf(admax, fabsf(d32));
                    }
                } else {
                    const double ninv = -te->inv;
#pragma unroll
                    for (int k = 0; k < EPT; ++k) {
                        const int i = tid + k * BD;
                        if (ACHR_PAD_SLOT(k)) {
                            dreg[k] = 0.0;
                            continue;
                        }
                        const double dk = fma(As[i], ninv, ws[i]);
                        dreg[k] = dk;
                        const float d32 = f64_to_f32_rz(dk);
                        ss = fmaf(d32, d32, ss);
                        admax = fmaxf(admax, fabsf(d32));
                    }
                }
                // Phase B1 folded into phase A (merged): the brackets need ||d||
                // only for the candidacy test |d_i| > u_tol ||d||, so they are
                // formed now with a threshold interval that holds for any norm
                // the block sum can give: above by uthr_max (checked after the
                // reduction), below by u_tol times this thread's largest |d_i|.
                // A coordinate certain under both is classified; any other
                // gets a -inf lower end and is settled exactly in phase B2.
                float uh = INFINITY, ul = INFINITY;
                float my_lh = INFINITY, my_ll = INFINITY;  // this thread's smallest bracket lower ends
                int fl = 0;
                if (merged) {
                    const float uthr_lo_p = a.utol32 * admax * kProvDn;
#pragma unroll
                    for (int k = 0; k < EPT; ++k) {
                        const int i = tid + k * BD;
                        if (ACHR_PAD_SLOT(k)) continue;  // padding: never a candidate
                        float lo_h, lo_l;
                        bracket(xs[i], dreg[k], __ldg(a.bnd + i), a.bound_err, a.dtol_hi, a.dtol_lo, uthr_max,
                                uthr_lo_p, lo_h, lo_l, uh, ul, fl);
                        my_lh = fminf(my_lh, lo_h);
                        my_ll = fminf(my_ll, lo_l);
                    }
                    uh = warp_min_f32(uh);
                    ul = warp_min_f32(ul);
                }
#pragma unroll
                for (int o = 16; o; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
                // Each thread timed its own wait: OR every lane's outcome so that
                // the whole block leaves (or stays) together.
                const bool warp_failed = __any_sync(0xffffffffu, failed);
                if (lane == 0) {
                    rs->sum1[warp] = ss;
                    rs->flag1[warp] = warp_failed ? 1 : 0;
                    if (merged) rs->min2[warp] = make_float2(uh, ul);
                }
                __syncthreads();
                ss = 0.0f;
                int f1 = 0;
#pragma unroll
                for (int w = 0; w < NW; ++w) {
                    ss += rs->sum1[w];
                    f1 |= rs->flag1[w];
                }
                if (merged) {
                    uh = INFINITY;
                    ul = INFINITY;
#pragma unroll
                    for (int w = 0; w < NW; ++w) {
                        const float2 v = rs->min2[w];
                        uh = fminf(uh, v.x);
                        ul = fminf(ul, v.y);
                    }
                }
                if (f1) {
                    failed = true;
                    break;
                }
                const float norm32 = sqrtf(ss);

                // Prefetch the next step's warmup column while this one is tested.
                if (s + 1 < (a.step0 + a.T)) {
                    const int rn =
                        (s + 1 - tbase < kTbl)
                            ? (int)tbl[s + 1 - tbase].idx
                            : (int)warmup_index(step_draw(a.seed, ACHR_CHAIN_ID, (uint32_t)(s + 1), 0u), (uint32_t)a.W);
                    if (rn != buf_col && rn >= 0 && rn < a.W) {
                        if (tid == 0) {
                            fence_proxy_async_smem();
                            mbar_arrive_expect_tx(bar, column_bytes(a));
                            tma_load_1d(ws, a.warmup + (size_t)rn * (size_t)a.ldw, column_bytes(a), bar);
                        }
                        inflight = true;
                        buf_col = rn;
                    }
                }
                if (!(norm32 > 0.0f) || !(norm32 < INFINITY)) {
                    if (tid == 0) ++cnt[CNT_REJECTED];
                    continue;
                }

                // Phase B1: FP32 brackets (reference ratio test ACHRCuda.cu:266-281)
                const float uthr = a.utol32 * norm32;
                const float uthr_hi = uthr * kNormUp, uthr_lo = uthr * kNormDn;
                if (merged && uthr_hi <= uthr_max) {
                    fl = 0;  // the merged brackets stand; their flags are not used
                } else {
                    // separate pass (merged: ||d|| exceeded the bound the merged brackets assumed)
                    if (merged) __syncthreads();  // min2 of this attempt may still be read
                    uh = INFINITY;
                    ul = INFINITY;
                    my_lh = INFINITY;
                    my_ll = INFINITY;
                    fl = 0;
                    if (!a.exact_ratio) {
#pragma unroll
                        for (int k = 0; k < EPT; ++k) {
                            const int i = tid + k * BD;
                            if (ACHR_PAD_SLOT(k)) continue;
                            float lo_h, lo_l;
                            bracket(xs[i], dreg[k], __ldg(a.bnd + i), a.bound_err, a.dtol_hi, a.dtol_lo, uthr_hi,
                                    uthr_lo, lo_h, lo_l, uh, ul, fl);
                            my_lh = fminf(my_lh, lo_h);  // NaN (not a candidate) is ignored, -inf (undecided) wins
                            my_ll = fminf(my_ll, lo_l);
                        }
                    } else {
                        fl = 2 | 4;
                        my_lh = my_ll = -INFINITY;
                    }
                    uh = warp_min_f32(uh);
                    ul = warp_min_f32(ul);
                    fl = (int)__reduce_or_sync(0xffffffffu, (unsigned)fl);
                    if (lane == 0) {
                        rs->min2[warp] = make_float2(uh, ul);
                        rs->flag2[warp] = fl;
                    }
                    __syncthreads();
                    uh = INFINITY;
                    ul = INFINITY;
                    fl = 0;
#pragma unroll
                    for (int w = 0; w < NW; ++w) {
                        const float2 v = rs->min2[w];
                        uh = fminf(uh, v.x);
                        ul = fminf(ul, v.y);
                        fl |= rs->flag2[w];
                    }
                }

                // FP64 norm, only when some candidacy test sits inside the FP32
                // norm's margin (or every candidate is evaluated in FP64).  With
                // merged brackets that is known only in phase B2, which then
                // asks for it and runs once more.
                double thr64 = 0.0;
                bool have_norm64 = false;
                double norm64 = 0.0;
                unsigned long long kh, kl;
                int anyv;
                for (int b2 = 0;; ++b2) {
                    if ((fl & 4) && !have_norm64) {
                        double s64 = fp64_zero_here();
#pragma unroll
                        for (int k = 0; k < EPT; ++k) s64 = fma(dreg[k], dreg[k], s64);
#pragma unroll
                        for (int o = 16; o; o >>= 1) s64 += __shfl_xor_sync(0xffffffffu, s64, o);
                        if (lane == 0) rs->sum5[warp] = s64;
                        __syncthreads();
                        s64 = 0.0;
#pragma unroll
                        for (int w = 0; w < NW; ++w) s64 += rs->sum5[w];
                        norm64 = sqrt(s64);
                        have_norm64 = true;
                        thr64 = a.u_tol * norm64;
                    }

                    // Phase B2: FP64 evaluation of every coordinate whose bracket can
                    // hold a minimum, or whose candidacy the brackets left open.
                    kh = kInfBits;
                    kl = kInfBits;
                    anyv = 0;
                    int nex = 0, need64 = 0;
                    unsigned mh = 0, ml = 0, mam = 0;  // bit k: contender for max / min step, undecided
                    // Only a thread whose own bracket lower ends reach the block minima
                    // can hold a contender; the others skip the second pass.
                    const bool mine = my_lh <= uh || my_ll <= ul;
                    if (!a.exact_ratio && mine) {
#pragma unroll
                        for (int k = 0; k < EPT; ++k) {
                            const int i = tid + k * BD;
                            if (ACHR_PAD_SLOT(k)) continue;
                            float lo_h, lo_l, uh2 = INFINITY, ul2 = INFINITY;  // minima already known
                            int fl2 = 0;
                            bracket(xs[i], dreg[k], __ldg(a.bnd + i), a.bound_err, a.dtol_hi, a.dtol_lo, uthr_hi,
                                    uthr_lo, lo_h, lo_l, uh2, ul2, fl2);
                            mh |= (lo_h <= uh ? 1u : 0u) << k;
                            ml |= (lo_l <= ul ? 1u : 0u) << k;
                            mam |= (lo_h == -INFINITY ? 1u : 0u) << k;
                        }
                    } else if (a.exact_ratio) {
                        mh = ml = mam = (EPT >= 32) ? 0xFFFFFFFFu : ((1u << EPT) - 1u);
                    }
                    for (unsigned m = mh | ml; m; m &= m - 1) {
                        const int k = __ffs(m) - 1;
                        const unsigned bit = 1u << k;
                        const int i = tid + k * BD;
                        ++nex;
                        const double xi = xs[i], dk = pick(dreg, k);
                        const double2 lu = ld_lbub(a.lbub + i);
                        const double Dp = lu.y - xi, Dm = xi - lu.x;
                        bool valid = true;
                        if (mam & bit) {  // undecided: full FP64 candidacy test
                            bool u_pass;
                            if (have_norm64) {
                                u_pass = abs_bits(dk) > (unsigned long long)__double_as_longlong(thr64);
                            } else {
                                const float ad32 = fabsf(f64_to_f32_rz(dk));
                                // inside the FP32 norm's margin: settled with the FP64 norm
                                if (!(ad32 > uthr_hi) && !(ad32 * kAdUp < uthr_lo)) need64 = 1;
                                u_pass = ad32 > uthr_hi;
                            }
                            valid = Dp > a.d_tol && Dm > a.d_tol && u_pass;
                        }
                        if (valid) {
                            const double ad = abs_int(dk);
                            const bool pos = positive_int(dk);
                            if (mh & bit) kh = umin(kh, (unsigned long long)__double_as_longlong((pos ? Dp : Dm) / ad));
                            if (ml & bit) kl = umin(kl, (unsigned long long)__double_as_longlong((pos ? Dm : Dp) / ad));
                            anyv = 1;
                        }
                    }
                    if (nex) atomicAdd(exact_count, nex);
                    kh = warp_min_u64(kh);
                    kl = warp_min_u64(kl);
                    anyv = (int)__reduce_or_sync(0xffffffffu, (unsigned)(anyv | (need64 << 1)));
                    if (lane == 0) {
                        rs->min3[warp] = make_ulonglong2(kh, kl);
                        rs->flag3[warp] = anyv;
                    }
                    __syncthreads();
                    kh = kInfBits;
                    kl = kInfBits;
                    anyv = 0;
#pragma unroll
                    for (int w = 0; w < NW; ++w) {
                        const ulonglong2 v = rs->min3[w];
                        kh = umin(kh, v.x);
                        kl = umin(kl, v.y);
                        anyv |= rs->flag3[w];
                    }
                    if (!(anyv & 2) || have_norm64) break;
                    fl |= 4;  // a contender's candidacy needs the FP64 norm: evaluate again with it
                }
                anyv &= 1;
                if (!anyv) {  // no candidate: rejection (see ACHRCuda.cu:283-288)
                    if (tid == 0) ++cnt[CNT_REJECTED];
                    continue;
                }
                const double qh = __longlong_as_double((long long)kh);
                const double ql = __longlong_as_double((long long)kl);

                // Rejection test |min| < tol && |max| < tol (ACHRCuda.cu:316-319),
                // min = -ql ||d||, max = qh ||d||; FP32 unless inside the margin.
                bool reject;
                {
                    const float qh32 = f64_to_f32_rz(qh), ql32 = f64_to_f32_rz(ql);
                    const float th_lo = qh32 * norm32 * kNormDn, th_hi = qh32 * kAdUp * norm32 * kNormUp;
                    const float tl_lo = ql32 * norm32 * kNormDn, tl_hi = ql32 * kAdUp * norm32 * kNormUp;
                    const float tol_lo = a.mmt32 * kDn, tol_hi = a.mmt32 * kUp;
                    const bool big = th_lo >= tol_hi || tl_lo >= tol_hi;
                    const bool small = th_hi < tol_lo && tl_hi < tol_lo;
                    if (big) {
                        reject = false;
                    } else if (small) {
                        reject = true;
                    } else {
                        double s64 = fp64_zero_here();
#pragma unroll
                        for (int k = 0; k < EPT; ++k) s64 = fma(dreg[k], dreg[k], s64);
#pragma unroll
                        for (int o = 16; o; o >>= 1) s64 += __shfl_xor_sync(0xffffffffu, s64, o);
                        __syncthreads();  // slot sum5 may hold this attempt's earlier norm
                        if (lane == 0) rs->sum5[warp] = s64;
                        __syncthreads();
                        s64 = 0.0;
#pragma unroll
                        for (int w = 0; w < NW; ++w) s64 += rs->sum5[w];
                        const double nrm = sqrt(s64);
                        reject = fabs(ql * nrm) < a.max_min_tol && fabs(qh * nrm) < a.max_min_tol;
                    }
                }
                if (reject) {
                    if (tid == 0) ++cnt[CNT_REJECTED];
                    continue;
                }
                // t / ||d|| with t = U (max - min) + min (reference ACHRCuda.cu:314)
                const double sstep = fma(te->U, qh + ql, -ql);

                // Phase C: x = prev + t u (ACHRCuda.cu:242-249), residual check every
                // check_period steps (:325-344), clip + centre (:193-206, :347-350).
                const bool check = chk == 0;
                chk = (chk + 1 == a.check_period) ? 0 : chk + 1;
                if (!check && hr) {  // hit-and-run: no centre to update
                    unsigned edge = 0;
#pragma unroll
                    for (int k = 0; k < EPT; ++k) {
                        const int i = tid + k * BD;
                        if (ACHR_PAD_SLOT(k)) continue;
                        const double xn = fma(sstep, dreg[k], xs[i]);
                        xs[i] = xn;
                        if (!surely_inside(f64_to_f32_rz(xn), __ldg(a.bnd + i), a.bound_err)) edge |= 1u << k;
                    }
                    for (; edge; edge &= edge - 1) {
                        const int i = tid + (__ffs(edge) - 1) * BD;
                        xs[i] = clip_exact(xs[i], ld_lbub(a.lbub + i));
                    }
                } else if (!check) {
                    unsigned edge = 0;  // bit k: not provably inside the box, clip exactly below
#pragma unroll
                    for (int k = 0; k < EPT; ++k) {
                        const int i = tid + k * BD;
                        if (ACHR_PAD_SLOT(k)) continue;
                        const double xn = fma(sstep, dreg[k], xs[i]);
                        xs[i] = xn;
                        if (surely_inside(f64_to_f32_rz(xn), __ldg(a.bnd + i), a.bound_err)) As[i] += xn;
                        else edge |= 1u << k;
                    }
                    for (; edge; edge &= edge - 1) {
                        const int i = tid + (__ffs(edge) - 1) * BD;
                        const double xc = clip_exact(xs[i], ld_lbub(a.lbub + i));
                        xs[i] = xc;
                        As[i] += xc;
                    }
                } else if (SEG) {
                    // Segmented sampling: the check ends this launch for the chain.
#pragma unroll
                    for (int k = 0; k < EPT; ++k) {
                        const int i = tid + k * BD;
                        if (ACHR_PAD_SLOT(k)) continue;
                        xs[i] = fma(sstep, dreg[k], xs[i]);
                    }
                    if (inflight) {  // (the launch ends here, so nothing was prefetched; kept for safety)
                        if (!mbar_wait_bounded(bar, phase)) failed = true;
                        phase ^= 1u;
                        inflight = false;
                    }
                    __syncthreads();  // every x update visible; the staging buffer is free
                    if (tid == 0) ++cnt[CNT_CHECKS];
                    double *rr = ws;  // S x, m doubles (m <= BD * EPT for segmented launches)
                    unsigned long long mx = residual_rows<BD>(a, xs, rr, tid);
                    mx = warp_max_u64(mx);
                    if (lane == 0) rs->max4[warp] = mx;
                    __syncthreads();
                    mx = 0;
#pragma unroll
                    for (int w = 0; w < NW; ++w) mx = umax(mx, rs->max4[w]);
                    const bool reproject = mx > (unsigned long long)__double_as_longlong(a.residual_tol);
                    if (reproject) {
                        if (tid == 0) {
                            ++cnt[CNT_REPROJ];
                            if (*a.seg_any == 0ull) atomicOr(a.seg_any, 1ull);
                        }
                        unsigned short *rh = a.seg_Rh + (size_t)p * (size_t)a.kpad;
                        unsigned short *rl = a.seg_Rl + (size_t)p * (size_t)a.kpad;
                        double *rd = a.seg_rd + (size_t)p * (size_t)a.ld_r;
                        for (int q = tid; q < a.m; q += BD) {
                            // (no FP64 operation: the FP32 image for the split is a truncation by
                            // integer operations, and the FP64 value is stored as it is)
                            unsigned short h, l;
                            split_bf16_bits(f64_to_f32_rz(rr[q]), h, l);
                            rh[q] = h;  // device row order, as the batched passes read them
                            rl[q] = l;
                            rd[q] = rr[q];
                        }
                    }
#pragma unroll
                    for (int k = 0; k < EPT; ++k) {
                        const int i = tid + k * BD;
                        if (i < a.n) {
                            a.seg_x[(size_t)p * (size_t)a.ld_seg + (size_t)i] = xs[i];
                            a.seg_A[(size_t)p * (size_t)a.ld_seg + (size_t)i] = As[i];
                        }
                    }
                    if (tid == 0) {
                        a.seg_flags[p] =
                            SEG_STARTED | SEG_ACCEPTED | SEG_PENDING | (reproject ? SEG_REPROJ : 0u);
                        ++cnt[CNT_ACCEPTED];
                    }
                    __syncthreads();  // the residual rows in ws are read before the next chain's column lands
                    any_accepted = true;
                    seg_pending = true;
                    break;
                } else {
#pragma unroll
                    for (int k = 0; k < EPT; ++k) {
                        const int i = tid + k * BD;
                        if (ACHR_PAD_SLOT(k)) continue;
                        xs[i] = fma(sstep, dreg[k], xs[i]);
                    }
                    __syncthreads();
                    if (tid == 0) ++cnt[CNT_CHECKS];
                    unsigned long long mx = residual_max_bits<BD>(a, xs, tid);
                    mx = warp_max_u64(mx);
                    if (lane == 0) rs->max4[warp] = mx;
                    __syncthreads();
                    mx = 0;
#pragma unroll
                    for (int w = 0; w < NW; ++w) mx = umax(mx, rs->max4[w]);
                    if (mx > (unsigned long long)__double_as_longlong(a.residual_tol)) {
                        // x <- N (N^T x) in FP64 (reference reprojectPoint(2), ACHRCuda.cu:208-230).
                        // The scratch is ws: let the prefetched column land, use the
                        // buffer, then fetch the column again.
                        if (tid == 0) ++cnt[CNT_REPROJ];
                        if (inflight) {
                            if (!mbar_wait_bounded(bar, phase)) failed = true;
                            phase ^= 1u;
                            inflight = false;
                        }
                        if (__syncthreads_or(failed ? 1 : 0)) failed = true;  // block-uniform from here
                        if (a.pinv32) {
                            residual_form_reproject<BD>(a, xs, reinterpret_cast<float2 *>(ws), zs, tid);
                        } else {
                            const int n = a.n;
                            for (int j = warp; j < a.d; j += NW) {
                                const double *Nj = a.N + (size_t)j * (size_t)n;
                                double acc = 0.0;
                                for (int i = lane; i < n; i += 32) acc = fma(__ldg(Nj + i), xs[i], acc);
#pragma unroll
                                for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
                                if (lane == 0) ys[j] = acc;
                            }
                            __syncthreads();
                            for (int i = tid; i < n; i += BD) {
                                double acc = 0.0;
                                for (int j = 0; j < a.d; ++j)
                                    acc = fma(__ldg(a.N + (size_t)j * (size_t)n + i), ys[j], acc);
                                xs[i] = acc;
                            }
                        }
                        __syncthreads();
                        if (buf_col >= 0) {
                            if (tid == 0) {
                                fence_proxy_async_smem();
                                mbar_arrive_expect_tx(bar, column_bytes(a));
                                tma_load_1d(ws, a.warmup + (size_t)buf_col * (size_t)a.ldw, column_bytes(a), bar);
                            }
                            inflight = true;
                        }
                    }
                    unsigned edge = 0;
#pragma unroll
                    for (int k = 0; k < EPT; ++k) {
                        const int i = tid + k * BD;
                        if (ACHR_PAD_SLOT(k)) continue;
                        const double xv = xs[i];
                        if (surely_inside(f64_to_f32_rz(xv), __ldg(a.bnd + i), a.bound_err)) {
                            if (!hr) As[i] += xv;
                        } else {
                            edge |= 1u << k;
                        }
                    }
                    for (; edge; edge &= edge - 1) {
                        const int i = tid + (__ffs(edge) - 1) * BD;
                        const double xc = clip_exact(xs[i], ld_lbub(a.lbub + i));
                        xs[i] = xc;
                        if (!hr) As[i] += xc;
                    }
                }
                if (tid == 0) ++cnt[CNT_ACCEPTED];
                any_accepted = true;
                break;
            }
        }
        if (inflight) {
            if (!mbar_wait_bounded(bar, phase)) failed = true;
            phase ^= 1u;
            inflight = false;
        }
        if (stuck && !was_stuck && tid == 0) ++cnt[CNT_STUCK];
        if (__syncthreads_or(failed ? 1 : 0)) {
            failed = true;
            break;
        }
        if (SEG && !seg_pending && !a.seg_final) {
            // A segmented launch that is not the run's last: keep the state for the next one.
#pragma unroll
            for (int k = 0; k < EPT; ++k) {
                const int i = tid + k * BD;
                if (i < a.n) {
                    a.seg_x[(size_t)p * (size_t)a.ld_seg + (size_t)i] = xs[i];
                    a.seg_A[(size_t)p * (size_t)a.ld_seg + (size_t)i] = As[i];
                }
            }
            if (tid == 0)
                a.seg_flags[p] = SEG_STARTED | (any_accepted ? SEG_ACCEPTED : 0u) | (stuck ? SEG_STUCK : 0u);
        }
        if (SEG && (seg_pending || !a.seg_final)) {
            __syncthreads();
            continue;  // the point is emitted by the run's last launch
        }

        // Emitted point: residual / bound diagnostics and, on request, the final
        // feasibility projection (project, clip, re-check).
        if (any_accepted) {
            RedSlots *rs = rsb;
            const int n = a.n;
            unsigned long long res = 0;
            for (int pass = 0; pass < 2; ++pass) {
                unsigned long long mx = residual_max_bits<BD>(a, xs, tid);
                mx = warp_max_u64(mx);
                __syncthreads();
                if (lane == 0) rs->max4[warp] = mx;
                __syncthreads();
                res = 0;
#pragma unroll
                for (int w = 0; w < NW; ++w) res = umax(res, rs->max4[w]);
                if (pass == 1 || !a.final_project || __longlong_as_double((long long)res) <= a.feasibility_tol) break;
                if (tid == 0) ++cnt[CNT_FINAL_PROJ];
                for (int j = warp; j < a.d; j += NW) {
                    const double *Nj = a.N + (size_t)j * (size_t)n;
                    double acc = 0.0;
                    for (int i = lane; i < n; i += 32) acc = fma(__ldg(Nj + i), xs[i], acc);
#pragma unroll
                    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
                    if (lane == 0) ys[j] = acc;
                }
                __syncthreads();
                for (int i = tid; i < n; i += BD) {
                    double acc = 0.0;
                    for (int j = 0; j < a.d; ++j) acc = fma(__ldg(a.N + (size_t)j * (size_t)n + i), ys[j], acc);
                    xs[i] = clip_exact(acc, ld_lbub(a.lbub + i));
                }
                __syncthreads();
            }
            double viol = 0.0;
            for (int i = tid; i < n; i += BD) {
                const double xi = xs[i];
                const double2 lu = ld_lbub(a.lbub + i);
                viol = fmax(viol, fmax(lu.x - xi, xi - lu.y));
            }
            unsigned long long vb = (unsigned long long)__double_as_longlong(viol);
            vb = warp_max_u64(vb);
            __syncthreads();
            if (lane == 0) rs->max4[warp] = vb;
            __syncthreads();
            vb = 0;
#pragma unroll
            for (int w = 0; w < NW; ++w) vb = umax(vb, rs->max4[w]);
            if (tid == 0) {
                worst[0] = umax(worst[0], res);
                worst[1] = umax(worst[1], vb);
            }
        }
        for (int i = tid; i < a.n; i += BD) a.out[(size_t)i * (size_t)a.ld_out + (size_t)p] = any_accepted ? xs[i] : 0.0;
        if (a.A_out)
            for (int i = tid; i < a.n; i += BD) a.A_out[(size_t)i * (size_t)a.ld_state + (size_t)p] = As[i];
        __syncthreads();
    }
#undef ACHR_CHAIN_ID
#undef ACHR_PAD_SLOT

    __syncthreads();
    if (tid == 0) {
        unsigned long long *c = a.counters;
        const int slots[6] = {CNT_ACCEPTED, CNT_REJECTED, CNT_CHECKS, CNT_REPROJ, CNT_STUCK, CNT_FINAL_PROJ};
        for (int q = 0; q < 6; ++q)
            if (cnt[slots[q]]) atomicAdd(c + slots[q], cnt[slots[q]]);
        if (*exact_count) atomicAdd(c + CNT_EXACT, (unsigned long long)*exact_count);
        if (worst[0]) atomicMax(c + CNT_MAXRES_BITS, worst[0]);
        if (worst[1]) atomicMax(c + CNT_MAXVIOL_BITS, worst[1]);
        if (failed) atomicOr(c + CNT_ERROR, ERR_TMA_TIMEOUT);
    }
    return failed;
}

// The staging barriers of a CTA (header of the dynamic shared memory).
template <int NP>
__device__ __forceinline__ void chain_init_barriers(unsigned char *smem_raw) {
    uint64_t *bar, *never;
    chain_barriers<NP>(smem_raw, bar, never);
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        mbar_init(never, 1);
        fence_mbar_init();
    }
    __syncthreads();
}

// One model: CTA b takes chains b, b + grid, ...
template <int BD, int EPT, bool SEG>
__global__ void __launch_bounds__(BD, (BD <= 384 ? 2 : 1)) achr_chain_kernel(const ChainArgs a) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    chain_init_barriers<BD * EPT>(smem_raw);
    unsigned phase = 0;
    chain_run<BD, EPT, SEG>(a, blockIdx.x, gridDim.x, a.P, smem_raw, phase);
}

// Many models of one configuration in one persistent launch: each CTA takes
// the next (model, first chain, end chain) item of a device work queue until
// the queue is empty.  The host orders the items longest model first, with
// tiles that shrink towards the end of the queue, and sets the residual-form
// reprojection off (its shared memory is not part of this launch).  When a
// model's last chain is done, its finish time (globaltimer, ns) goes to
// done_ns[model].
template <int BD, int EPT>
__global__ void __launch_bounds__(BD, (BD <= 384 ? 2 : 1)) achr_chain_queue_kernel(const ChainQueue q) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ ChainArgs sa;
    __shared__ int4 cur;
    static_assert(sizeof(ChainArgs) % sizeof(int) == 0, "ChainArgs is copied as 32-bit words");
    chain_init_barriers<BD * EPT>(smem_raw);
    unsigned phase = 0;
    int model = -1;
    for (;;) {
        if (threadIdx.x == 0) {
            const int k = atomicAdd(q.next, 1);
            cur = k < q.n_items ? q.items[k] : make_int4(-1, 0, 0, 0);
        }
        __syncthreads();
        const int4 item = cur;
        if (item.x < 0) break;
        if (item.x != model) {
            const int *src = reinterpret_cast<const int *>(q.args + item.x);
            int *dst = reinterpret_cast<int *>(&sa);
            for (int w = threadIdx.x; w < (int)(sizeof(ChainArgs) / sizeof(int)); w += BD) dst[w] = src[w];
            model = item.x;
        }
        __syncthreads();
        const bool failed = chain_run<BD, EPT, false>(sa, item.y, 1, item.z, smem_raw, phase);
        if (threadIdx.x == 0) {
            const int n = item.z - item.y;
            if (atomicAdd(q.chains_done + item.x, n) + n == sa.P) q.done_ns[item.x] = global_ns();
        }
        if (failed) break;  // recorded in the model's counters; the CTA stops taking work
        __syncthreads();    // `cur` and `sa` are rewritten only after every thread is done with them
    }
    if (threadIdx.x == 0 && q.cta_ns) q.cta_ns[blockIdx.x] = global_ns();
}

// Occupancy-sized persistent launch of one configuration.  max_ctas > 0 caps
// the grid.
template <int BD, int EPT, bool SEG>
cudaError_t launch_cfg_kernel(const ChainArgs &a_in, cudaStream_t stream, int max_ctas, int *per_sm_out) {
    auto *const KFN = achr_chain_kernel<BD, EPT, SEG>;
    ChainArgs a = a_in;
    const size_t base = chain_smem_bytes_cfg(BD * EPT, a.d, BD);
    // The residual-form reprojection keeps z (m floats) in shared memory and
    // the residual in the staging buffer; it is used only when both fit
    // without costing a resident CTA per SM.
    const size_t zbytes = ((size_t)a.m * sizeof(float) + 15) & ~(size_t)15;
    // (its residual occupies the column buffer below the buffer's zero padding: m <= ldw)
    if (a.pinv32 && a.m > a.ldw) a.pinv32 = nullptr;
    size_t smem = base + (a.pinv32 ? zbytes : 0);
    cudaError_t e = cudaFuncSetAttribute(KFN, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)std::max(smem, base));
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, KFN, BD, base);
    if (e != cudaSuccess) return e;
    if (a.pinv32) {
        int per_sm_z = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_z, KFN, BD, smem);
        if (e != cudaSuccess) return e;
        if (per_sm_z < per_sm) {
            a.pinv32 = nullptr;
            smem = base;
        }
    }
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    if (per_sm_out) *per_sm_out = per_sm;
    if (a.P <= 0) return cudaSuccess;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long long grid = (long long)sms * per_sm;
    if (max_ctas > 0 && grid > max_ctas) grid = max_ctas;
    if (grid > a.P) grid = a.P;
    if (grid < 1) return cudaSuccess;
    KFN<<<(unsigned)grid, BD, smem, stream>>>(a);
    return cudaGetLastError();
}

// Persistent work-queue launch of one configuration: `grid` CTAs (0: every
// resident slot of the GPU), with q.extra_smem bytes of shared memory beyond
// the header for the residual-form reprojection.  per_sm_out (if non-NULL)
// receives the CTAs that fit on one SM; with q.n_items = 0 nothing is launched.
template <int BD, int EPT>
cudaError_t launch_queue_cfg(const ChainQueue &q, cudaStream_t stream, int grid, int *per_sm_out) {
    auto *const KFN = achr_chain_queue_kernel<BD, EPT>;
    const size_t smem = chain_smem_bytes_cfg(BD * EPT, 0, BD) + q.extra_smem;
    cudaError_t e = cudaFuncSetAttribute(KFN, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, KFN, BD, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    if (per_sm_out) *per_sm_out = per_sm;
    if (q.n_items <= 0) return cudaSuccess;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long long g = grid > 0 ? grid : (long long)sms * per_sm;
    if (g > q.n_items) g = q.n_items;
    KFN<<<(unsigned)g, BD, smem, stream>>>(q);
    return cudaGetLastError();
}

// Occupancy-sized persistent launch of one configuration (segmented launches
// take the kernel's segmented instantiation).
template <int BD, int EPT>
cudaError_t launch_cfg(const ChainArgs &a, cudaStream_t stream, int max_ctas, int *per_sm_out) {
    return a.seg ? launch_cfg_kernel<BD, EPT, true>(a, stream, max_ctas, per_sm_out)
                 : launch_cfg_kernel<BD, EPT, false>(a, stream, max_ctas, per_sm_out);
}

}  // namespace achr
