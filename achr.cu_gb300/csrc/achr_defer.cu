// Segmented sampling: the reference's per-chain reprojection deferred to one
// batched pass over all chains on the tensor cores.
//
// The reference checks every 10th step whether max|S x| exceeds 1e-9 and, if
// so, reprojects that chain, x <- N (N^T x), with two FP64 GEMVs before it
// clips the point and updates the centre (ACHRcu/ACHRCuda.cu:325-350,
// reprojectPoint(2) :208-230).  With warmup points read from the %f CSV the
// reference's warmup generator writes (VFWarmup/createWarmupPtsGLPK.c:292),
// |S w| is about 1e-6 and nearly every check reprojects; per chain that is
// 4 n d FP64 operations, about a hundred times the FP64 work of the step
// itself at 2766 x 3742 on GB300's FP64 pipe.
//
// Here every chain runs to its next check step in one launch of the chain
// kernel (segmented mode, achr_chain_kernel.cuh), which ends each chain right
// after the check step's x <- x + t u and leaves, for every chain whose FP64
// residual exceeds the tolerance, r = S x (FP64) and its BF16 hi + lo split
// (chain-major block R).  The batched passes then apply the same orthogonal
// projector to all of those chains at once,
//
//     x <- x - S^T z,   z = B r,   B = (S S^T)^+,
//
// z for every chain as one tensor-core GEMM Z = R B^T (three BF16 split
// products, FP32 accumulation, achr_tc_gemm.cu).  The first pass removes all
// but ~1e-4 of the residual, so two things in it must be exact to FP64 level:
// the update d = S^T z (any rounding outside the row space of S would move the
// point off the reference's projection for good) and the new residual
// r <- r - S d (later passes can only remove what they measure).  GB300's
// FP64 pipe is the chain kernel's bottleneck, so both run in double-float
// arithmetic on the FP32 pipes (values as unevaluated sums hi + lo of two
// floats, error-free products and sums, about 48 significant bits).  Later
// passes only move the point by what is left: they form d = S^T z in FP32,
// add it into the double-float correction and track r in FP32.  The next
// launch of the chain kernel subtracts the correction (two FP64 additions per
// reaction), clips the point and adds it to its centre accumulator before the
// chain's next step, the order the reference uses.  A chain takes passes
// until max|r| falls to residual_tol / 1000, which leaves the point within
// that, over the smallest singular value of S, of the FP64 projection (about
// the projection's own FP64 rounding); models whose S S^T has a condition
// number above 2e4 reproject in the chain kernel instead.  The decisions
// (which chains reproject) are the chain kernel's own FP64 residual, identical
// to the check it makes when it reprojects in place.  S and S^T are read as
// sliced-ELL blocks (32 lines per group, slot-major, lines sorted by length)
// so a warp's loads of one slot are one coalesced segment.  Every per-row
// quantity (S x, R, Z = R B^T, r) is kept in the chain kernel's device row
// order (rows longest first), with B permuted to match, so the chain kernel
// and the passes read and write them as contiguous runs; the per-reaction
// update leaves the passes through shared memory in reaction order.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "achr_ctx.h"

extern "C" void achr_io_set_error(const char *msg);

namespace achr {

// Sparse lines (rows of S, or rows of S^T = columns of S) as a sliced-ELL
// block: groups of 32 lines sorted by length, slot t of lane l of group g at
// off[g] + 32 t + l, zero padding; values split into FP32 hi + lo.
struct SlicedEll {
    int groups = 0;
    DevBuf<int> off;      // groups + 1
    DevBuf<int> line;     // 32 * groups: the line lane l of group g holds (-1: none)
    DevBuf<unsigned short> idx;  // the other index of each entry (n and m are below 65536)
    DevBuf<float> vh, vl;
};

struct DeferState {
    int cap = 0;             // chains the buffers hold
    long long ld = 0;        // leading dimension of the chain-major state (n rounded up to even)
    int ldz = 0;             // leading dimension of Z and r (m rounded up to a multiple of 4)
    int kpad = 0;            // K of the GEMM: m rounded up to a multiple of 64
    bool exact32 = false;    // every coefficient of S is exact in FP32 (all lo parts zero)
    DevBuf<double> x, A;     // cap x ld: points and centre accumulators between launches
    DevBuf<unsigned> flags;  // cap: SEG_* bits
    DevBuf<unsigned short> Rh, Rl;  // cap x kpad BF16 bits: S x of the chains that reproject
    DevBuf<double> rd;       // cap x ldz: S x at the check, FP64
    DevBuf<float> Z;         // cap x ldz: B r
    DevBuf<float> r;         // cap x ldz: r after each pass, FP32
    DevBuf<float> dxh, dxl;  // cap x ld: the passes' summed correction S^T z, double-float
    DevBuf<float> r0;        // cap: max|S x| of the chain when its check fired
    SlicedEll cols, rows;    // S^T and S; rows of S (and the row indices of S^T) in the device row order
    DevBuf<__nv_bfloat16> Bh, Bl;  // m x kpad: (S S^T)^+ split into hi + lo, rows and columns in the device row order
    DevBuf<unsigned long long> any;  // one word per launch and pass: some chain needs that pass
    int any_cap = 0;
    // Timing of the last run (only when requested): an event before and after every
    // chain-kernel launch, and one at the end.
    std::vector<cudaEvent_t> ev;
    int ev_used = 0;
    double chains_per_sweep = 0.0;
    ~DeferState() {
        for (cudaEvent_t e : ev) cudaEventDestroy(e);
    }
};

void defer_free(DeferState *d) { delete d; }

namespace {

constexpr int kDeferChunk = 131072;        // chains per sweep through the segments (bounds the buffers)
constexpr double kDeferMaxKappa = 2.0e4;   // largest condition number of S S^T the passes are used for
constexpr int kPassThreads = 512;
constexpr int kPassWarps = kPassThreads / 32;
constexpr int kMaxPasses = 8;              // passes of one deferred reprojection at most
// A chain's passes end once max|S x| <= residual_tol / 1000 (1e-12 by default, about the FP64
// rounding floor of S x for fluxes of size 1000): the point is then within that, over the
// smallest singular value of S, of the FP64 projection.  (The bound is absolute: a check can
// find a residual of 0.1 after 25 steps on %f warmups, and 1e-9 of that would still be 1e-10.)
constexpr float kRelTol = 0.0f;
constexpr size_t kPassSmemMax = 220 * 1024;  // dynamic shared memory a pass CTA may use

achr_status set_err(achr_status st, const std::string &msg) {
    achr_io_set_error(msg.c_str());
    return st;
}

#define DEFER_TRY(expr)                                                                                        \
    do {                                                                                                       \
        cudaError_t e_ = (expr);                                                                               \
        if (e_ != cudaSuccess) return set_err(ACHR_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// Error-free transformations on FP32 (IEEE round-to-nearest; nvcc neither
// reassociates these nor contracts them beyond the explicit fmaf).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void fast_two_sum(float a, float b, float &s, float &e) {  // |a| >= |b| or a = 0
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}
__device__ __forceinline__ void two_prod(float a, float b, float &p, float &e) {
    p = __fmul_rn(a, b);
    e = fmaf(a, b, -p);
}

// FP64 -> (hi, lo) FP32 with integer operations only: hi is v truncated to 24
// significant bits, lo the rest (up to 29 bits, rounded to 24); |v - hi - lo|
// <= 2^-48 |v|.  Values below 2^-126 become 0.
__device__ __forceinline__ void split_f64(double v, float &hi, float &lo) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
    const int e = (int)((b >> 52) & 0x7FF);
    const int fe = e - 896;  // FP32 biased exponent
    if (fe <= 0 || fe >= 255) {
        hi = (fe >= 255) ? __uint_as_float(sign | 0x7F800000u) : __uint_as_float(sign);
        lo = 0.0f;
        return;
    }
    const unsigned long long mant = b & 0xFFFFFFFFFFFFFull;
    hi = __uint_as_float(sign | ((unsigned)fe << 23) | (unsigned)(mant >> 29));
    const unsigned rest = (unsigned)(mant & 0x1FFFFFFFull);  // the low 29 bits: rest * 2^(e - 1075)
    const float r = __uint2float_rn(rest);
    const float l = ldexpf(r, e - 1075);
    lo = sign ? -l : l;
}

__device__ __forceinline__ void split_store(float r, __nv_bfloat16 *rh, __nv_bfloat16 *rl, int i) {
    const __nv_bfloat16 h = __float2bfloat16_rn(r);
    rh[i] = h;
    rl[i] = __float2bfloat16_rn(__fsub_rn(r, __bfloat162float(h)));
}

struct EllView {
    int groups;
    const int *off, *line;
    const unsigned short *idx;
    const float *vh, *vl;
};

struct PassArgs {
    int n, m, kpad, P, pass, last;
    long long ld, ldz;
    unsigned *flags;
    const float *Z;
    const double *rd;
    float *r, *dxh, *dxl, *r0;
    __nv_bfloat16 *Rh, *Rl;
    EllView cols, rows;  // S^T (lines = columns of S) and S (lines = rows of S)
    float fine_tol, rel_tol, residual_tol;
    const unsigned long long *this_gate;
    unsigned long long *next_any, *counters;
};

// End of a chain's pass (thread 0): convergence, next-pass gate, divergence.
__device__ __forceinline__ void pass_verdict(const PassArgs &a, int p, float mx, float r0max) {
    atomicAdd(a.counters + CNT_PASSES, 1ull);
    if (mx <= fmaxf(a.fine_tol, a.rel_tol * r0max)) {
        a.flags[p] &= ~SEG_REPROJ;  // converged
    } else if (!a.last) {
        if (*a.next_any == 0ull) atomicOr(a.next_any, 1ull);
    } else if (mx > a.residual_tol) {
        atomicOr(a.counters + CNT_ERROR, (unsigned long long)ERR_DEFER_DIVERGED);
    }
}

// Per-warp maxima of NV values into red[i][warp] (lane 0 writes); the caller
// synchronises once and one thread reduces over the warps, so a CTA reduces
// every chain's values behind a single barrier.
template <int NV>
__device__ __forceinline__ void warp_max_to(float (&v)[NV], float (*red)[kPassWarps]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        float x = v[i];
#pragma unroll
        for (int o = 16; o; o >>= 1) x = fmaxf(x, __shfl_xor_sync(0xffffffffu, x, o));
        if (lane == 0) red[i][warp] = x;
    }
}

__device__ __forceinline__ float over_warps(const float *r) {
    float m = r[0];
#pragma unroll
    for (int w = 1; w < kPassWarps; ++w) m = fmaxf(m, r[w]);
    return m;
}


// Shared-memory floats per chain of the pass kernels (multiples of 4, so every
// chain's block starts on a 16-byte boundary): z (ldz floats) and d, as a
// double-float pair in the first pass, in FP32 in the later ones.
__host__ __device__ inline size_t pass1_floats(long long ldz, long long ld) {
    return ((size_t)ldz + 2 * (size_t)ld + 3) & ~(size_t)3;
}
__host__ __device__ inline size_t pass_floats(long long ldz, long long ld) {
    return ((size_t)ldz + (size_t)ld + 3) & ~(size_t)3;
}

// The kernels below are bound by latency, not by bandwidth or arithmetic: each
// sparse slot is a global load of its index and value followed by a shared-
// memory gather, and each per-chain vector moves between global and shared
// memory.  So every loop issues a batch of independent loads before it uses
// any of them: kSlots slots of a sparse line, and two elements per thread of
// every resident chain's vectors.
constexpr int kSlots = 8;

// z rows of the CTA's live chains into shared memory (float4 copies).
template <int CPB>
__device__ __forceinline__ void stage_z(const PassArgs &a, int p0, const int *live, float *sm, size_t per) {
    const int q4 = (int)(a.ldz >> 2);
    for (int i0 = 0; i0 < q4; i0 += 2 * kPassThreads) {
        float4 v[CPB][2];
#pragma unroll
        for (int c = 0; c < CPB; ++c)
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int i = i0 + u * kPassThreads + (int)threadIdx.x;
                v[c][u] = (live[c] && i < q4)
                              ? __ldg(reinterpret_cast<const float4 *>(a.Z + (size_t)(p0 + c) * (size_t)a.ldz) + i)
                              : make_float4(0.f, 0.f, 0.f, 0.f);
            }
#pragma unroll
        for (int c = 0; c < CPB; ++c)
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int i = i0 + u * kPassThreads + (int)threadIdx.x;
                if (live[c] && i < q4) reinterpret_cast<float4 *>(sm + c * per)[i] = v[c][u];
            }
    }
}

// Slots [t0, min(t0 + kSlots, len)) of the line lane `lane` of a group holds:
// indices and values, all loads issued before any is used.
template <bool LO>
__device__ __forceinline__ void load_slots(const EllView &E, int base, int len, int t0, int lane, int *ii, float *hh,
                                           float *ll) {
#pragma unroll
    for (int u = 0; u < kSlots; ++u) {
        const int t = t0 + u;
        if (t >= len) break;  // the warp's line length: a uniform branch
        const int q = base + (t << 5) + lane;
        ii[u] = __ldg(E.idx + q);
        hh[u] = __ldg(E.vh + q);
        if (LO) ll[u] = __ldg(E.vl + q);
    }
}

// The first pass, in double-float, for CPB chains at a time per CTA (the
// sparse structure each warp loads serves all of them): for every chain
// flagged SEG_REPROJ, d = S^T z (z the chain's GEMM row), dx = d, and
// r = r0 - S d from the chain kernel's FP64 r0; r goes on in FP32 (r) and as
// the next GEMM's BF16 split.
template <int CPB, bool EXACT32, int MINB>
__global__ void __launch_bounds__(kPassThreads, MINB) defer_pass1_kernel(const PassArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ float redm[2 * CPB][kPassWarps];
    __shared__ int live[CPB];
    const size_t per = pass1_floats(a.ldz, a.ld);
    float *const sm = reinterpret_cast<float *>(smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (*a.this_gate == 0ull) return;  // no chain's check fired (the GEMM did not run either)
    if (blockIdx.x == 0 && tid == 0) atomicAdd(a.counters + CNT_GEMMS, 1ull);
    for (int p0 = blockIdx.x * CPB; p0 < a.P; p0 += gridDim.x * CPB) {
        if (tid < CPB) live[tid] = (p0 + tid < a.P && (a.flags[p0 + tid] & SEG_REPROJ)) ? 1 : 0;
        __syncthreads();
        int any = 0;
#pragma unroll
        for (int c = 0; c < CPB; ++c) any |= live[c];
        if (!any) {
            __syncthreads();
            continue;
        }
        stage_z<CPB>(a, p0, live, sm, per);
        __syncthreads();
        // d = S^T z, one line (column of S) per lane
        for (int g = warp; g < a.cols.groups; g += kPassWarps) {
            const int base = __ldg(a.cols.off + g);
            const int len = (__ldg(a.cols.off + g + 1) - base) >> 5;
            const int j = __ldg(a.cols.line + (g << 5) + lane);
            float ah[CPB], al[CPB];
#pragma unroll
            for (int c = 0; c < CPB; ++c) ah[c] = al[c] = 0.0f;
            for (int t0 = 0; t0 < len; t0 += kSlots) {
                int ii[kSlots];
                float hh[kSlots], ll[kSlots];
                load_slots<!EXACT32>(a.cols, base, len, t0, lane, ii, hh, ll);
#pragma unroll
                for (int u = 0; u < kSlots; ++u) {
                    if (t0 + u >= len) break;  // (len is the warp's: a uniform branch)
#pragma unroll
                    for (int c = 0; c < CPB; ++c) {
                        const float z = sm[c * per + ii[u]];
                        float ph, pe, s, e;
                        two_prod(hh[u], z, ph, pe);
                        if (!EXACT32) pe = fmaf(ll[u], z, pe);
                        two_sum(ah[c], ph, s, e);
                        ah[c] = s;
                        al[c] = __fadd_rn(al[c], __fadd_rn(e, pe));
                    }
                }
            }
            if (j >= 0) {
#pragma unroll
                for (int c = 0; c < CPB; ++c) {
                    float h, l;
                    fast_two_sum(ah[c], al[c], h, l);
                    float *dh = sm + c * per + a.ldz;
                    dh[j] = h;
                    dh[a.ld + j] = l;
                }
            }
        }
        __syncthreads();
        // d leaves shared memory in reaction order (the lines above run in column-length order)
#pragma unroll
        for (int c = 0; c < CPB; ++c) {
            if (!live[c]) continue;
            const float *dh = sm + c * per + a.ldz;
            float *gh = a.dxh + (size_t)(p0 + c) * (size_t)a.ld, *gl = a.dxl + (size_t)(p0 + c) * (size_t)a.ld;
            for (int j = tid; j < a.n; j += kPassThreads) {
                gh[j] = dh[j];
                gl[j] = dh[a.ld + j];
            }
        }
        // r = r0 - S d, one line (row of S, device order: line q is row q) per lane
        float mx[CPB], m0[CPB];
#pragma unroll
        for (int c = 0; c < CPB; ++c) mx[c] = m0[c] = 0.0f;
        for (int g = warp; g < a.rows.groups; g += kPassWarps) {
            const int i = __ldg(a.rows.line + (g << 5) + lane);
            double r0d[CPB];
#pragma unroll
            for (int c = 0; c < CPB; ++c)
                r0d[c] = (i >= 0 && live[c]) ? a.rd[(size_t)(p0 + c) * (size_t)a.ldz + (size_t)i] : 0.0;
            const int base = __ldg(a.rows.off + g);
            const int len = (__ldg(a.rows.off + g + 1) - base) >> 5;
            float ah[CPB], al[CPB];
            bool init = false;
            for (int t0 = 0; t0 < len || !init; t0 += kSlots) {
                int ii[kSlots];
                float hh[kSlots], ll[kSlots];
                if (t0 < len) load_slots<!EXACT32>(a.rows, base, len, t0, lane, ii, hh, ll);
                if (!init) {  // the FP64 residual, split once its load has had the slot loads to hide behind
#pragma unroll
                    for (int c = 0; c < CPB; ++c) {
                        split_f64(r0d[c], ah[c], al[c]);
                        m0[c] = fmaxf(m0[c], fabsf(ah[c]));
                    }
                    init = true;
                }
                if (t0 >= len) break;
#pragma unroll
                for (int u = 0; u < kSlots; ++u) {
                    if (t0 + u >= len) break;
#pragma unroll
                    for (int c = 0; c < CPB; ++c) {
                        const float *dh = sm + c * per + a.ldz;
                        const float xh = dh[ii[u]], xl = dh[a.ld + ii[u]];
                        float ph, pe, s, e;
                        two_prod(hh[u], xh, ph, pe);
                        pe = fmaf(hh[u], xl, pe);
                        if (!EXACT32) pe = fmaf(ll[u], xh, pe);
                        two_sum(ah[c], -ph, s, e);
                        ah[c] = s;
                        al[c] = __fadd_rn(al[c], __fsub_rn(e, pe));
                    }
                }
            }
            if (i >= 0) {
#pragma unroll
                for (int c = 0; c < CPB; ++c) {
                    if (!live[c]) continue;
                    const float rn = __fadd_rn(ah[c], al[c]);
                    const size_t o = (size_t)(p0 + c) * (size_t)a.ldz + (size_t)i;
                    a.r[o] = rn;
                    mx[c] = fmaxf(mx[c], fabsf(rn));
                    if (!a.last)
                        split_store(rn, a.Rh + (size_t)(p0 + c) * (size_t)a.kpad,
                                    a.Rl + (size_t)(p0 + c) * (size_t)a.kpad, i);
                }
            }
        }
        {
            float v[2 * CPB];
#pragma unroll
            for (int c = 0; c < CPB; ++c) {
                v[c] = mx[c];
                v[CPB + c] = m0[c];
            }
            warp_max_to<2 * CPB>(v, redm);
        }
        __syncthreads();
        if (tid == 0) {
#pragma unroll
            for (int c = 0; c < CPB; ++c) {
                if (!live[c]) continue;
                const float vmx = over_warps(redm[c]), vm0 = over_warps(redm[CPB + c]);
                const int p = p0 + c;
                a.flags[p] |= SEG_CORR;  // dx holds a correction for the next launch
                a.r0[p] = vm0;
                pass_verdict(a, p, vmx, vm0);
            }
        }
        __syncthreads();
    }
}

// A later pass (pass >= 1), in FP32, for CPB chains at a time per CTA: for
// every chain still flagged SEG_REPROJ, d = S^T z, dx += d (double-float),
// r <- r - S d.
template <int CPB>
__global__ void __launch_bounds__(kPassThreads, 2) defer_pass_kernel(const PassArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ float redm[CPB][kPassWarps];
    __shared__ int live[CPB];
    const size_t per = pass_floats(a.ldz, a.ld);
    float *const sm = reinterpret_cast<float *>(smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (*a.this_gate == 0ull) return;  // no chain needed this pass (its GEMM did not run either)
    if (blockIdx.x == 0 && tid == 0) atomicAdd(a.counters + CNT_GEMMS, 1ull);
    for (int p0 = blockIdx.x * CPB; p0 < a.P; p0 += gridDim.x * CPB) {
        if (tid < CPB) live[tid] = (p0 + tid < a.P && (a.flags[p0 + tid] & SEG_REPROJ)) ? 1 : 0;
        __syncthreads();
        int any = 0;
#pragma unroll
        for (int c = 0; c < CPB; ++c) any |= live[c];
        if (!any) {
            __syncthreads();
            continue;
        }
        stage_z<CPB>(a, p0, live, sm, per);
        __syncthreads();
        for (int g = warp; g < a.cols.groups; g += kPassWarps) {
            const int base = __ldg(a.cols.off + g);
            const int len = (__ldg(a.cols.off + g + 1) - base) >> 5;
            const int j = __ldg(a.cols.line + (g << 5) + lane);
            float d[CPB];
#pragma unroll
            for (int c = 0; c < CPB; ++c) d[c] = 0.0f;
            for (int t0 = 0; t0 < len; t0 += kSlots) {
                int ii[kSlots];
                float hh[kSlots];
                load_slots<false>(a.cols, base, len, t0, lane, ii, hh, nullptr);
#pragma unroll
                for (int u = 0; u < kSlots; ++u) {
                    if (t0 + u >= len) break;
#pragma unroll
                    for (int c = 0; c < CPB; ++c) d[c] = fmaf(hh[u], sm[c * per + ii[u]], d[c]);
                }
            }
            if (j >= 0) {
#pragma unroll
                for (int c = 0; c < CPB; ++c) sm[c * per + a.ldz + j] = d[c];
            }
        }
        __syncthreads();
        // dx += d in reaction order (the lines above run in column-length order)
        for (int j0 = 0; j0 < a.n; j0 += 2 * kPassThreads) {
            float h[CPB][2], l[CPB][2];
#pragma unroll
            for (int c = 0; c < CPB; ++c)
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const int j = j0 + u * kPassThreads + tid;
                    const size_t o = (size_t)(p0 + c) * (size_t)a.ld + (size_t)j;
                    const bool on = live[c] && j < a.n;
                    h[c][u] = on ? a.dxh[o] : 0.0f;
                    l[c][u] = on ? a.dxl[o] : 0.0f;
                }
#pragma unroll
            for (int c = 0; c < CPB; ++c)
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const int j = j0 + u * kPassThreads + tid;
                    if (!(live[c] && j < a.n)) continue;
                    const size_t o = (size_t)(p0 + c) * (size_t)a.ld + (size_t)j;
                    float s, e;
                    two_sum(h[c][u], sm[c * per + a.ldz + j], s, e);
                    a.dxh[o] = s;
                    a.dxl[o] = __fadd_rn(l[c][u], e);
                }
        }
        float mx[CPB];
#pragma unroll
        for (int c = 0; c < CPB; ++c) mx[c] = 0.0f;
        for (int g = warp; g < a.rows.groups; g += kPassWarps) {
            const int i = __ldg(a.rows.line + (g << 5) + lane);
            float rold[CPB];
#pragma unroll
            for (int c = 0; c < CPB; ++c)
                rold[c] = (i >= 0 && live[c]) ? a.r[(size_t)(p0 + c) * (size_t)a.ldz + (size_t)i] : 0.0f;
            const int base = __ldg(a.rows.off + g);
            const int len = (__ldg(a.rows.off + g + 1) - base) >> 5;
            float acc[CPB];
#pragma unroll
            for (int c = 0; c < CPB; ++c) acc[c] = 0.0f;
            for (int t0 = 0; t0 < len; t0 += kSlots) {
                int ii[kSlots];
                float hh[kSlots];
                load_slots<false>(a.rows, base, len, t0, lane, ii, hh, nullptr);
#pragma unroll
                for (int u = 0; u < kSlots; ++u) {
                    if (t0 + u >= len) break;
#pragma unroll
                    for (int c = 0; c < CPB; ++c) acc[c] = fmaf(hh[u], sm[c * per + a.ldz + ii[u]], acc[c]);
                }
            }
            if (i >= 0) {
#pragma unroll
                for (int c = 0; c < CPB; ++c) {
                    if (!live[c]) continue;
                    const size_t o = (size_t)(p0 + c) * (size_t)a.ldz + (size_t)i;
                    const float rn = __fsub_rn(rold[c], acc[c]);
                    a.r[o] = rn;
                    mx[c] = fmaxf(mx[c], fabsf(rn));
                    if (!a.last)
                        split_store(rn, a.Rh + (size_t)(p0 + c) * (size_t)a.kpad,
                                    a.Rl + (size_t)(p0 + c) * (size_t)a.kpad, i);
                }
            }
        }
        warp_max_to<CPB>(mx, redm);
        __syncthreads();
        if (tid == 0) {
#pragma unroll
            for (int c = 0; c < CPB; ++c)
                if (live[c]) pass_verdict(a, p0 + c, over_warps(redm[c]), a.r0[p0 + c]);
        }
        __syncthreads();
    }
}

// The pass kernels and their shared memory for a model: the most chains per
// CTA (4, 2 or 1) whose shared memory fits.
struct PassPlan {
    void (*pass1)(PassArgs);
    void (*pass)(PassArgs);
    size_t smem1, smem;
    int cpb1, cpb;
};

PassPlan plan_passes(long long ld, long long ldz, bool exact32) {
    PassPlan pl{};
    const size_t per1 = sizeof(float) * pass1_floats(ldz, ld), per = sizeof(float) * pass_floats(ldz, ld);
    // First pass: two CTAs of two chains per SM where their shared memory fits and the
    // coefficients are exact in FP32 (the variant with lo parts would spill at the 64 registers
    // two CTAs of 512 threads allow); measured at 2766 x 3742: 0.44 ms per 9728 chains against
    // 0.49 ms for one CTA of four chains, whose 16 warps hide less of the load latency.  Else
    // the most chains one CTA holds.
    const bool two_ctas = exact32 && per1 * 2 * 2 <= kPassSmemMax;
    pl.cpb1 = two_ctas ? 2 : per1 * 4 <= kPassSmemMax ? 4 : per1 * 2 <= kPassSmemMax ? 2 : 1;
    pl.cpb = per * 4 <= kPassSmemMax ? 4 : per * 2 <= kPassSmemMax ? 2 : 1;
    pl.smem1 = per1 * (size_t)pl.cpb1;
    pl.smem = per * (size_t)pl.cpb;
    if (two_ctas)
        pl.pass1 = defer_pass1_kernel<2, true, 2>;
    else if (exact32)
        pl.pass1 = pl.cpb1 == 4 ? defer_pass1_kernel<4, true, 1> : pl.cpb1 == 2 ? defer_pass1_kernel<2, true, 1>
                                                                                 : defer_pass1_kernel<1, true, 1>;
    else
        pl.pass1 = pl.cpb1 == 4 ? defer_pass1_kernel<4, false, 1> : pl.cpb1 == 2 ? defer_pass1_kernel<2, false, 1>
                                                                                  : defer_pass1_kernel<1, false, 1>;
    pl.pass = pl.cpb == 4 ? defer_pass_kernel<4> : pl.cpb == 2 ? defer_pass_kernel<2> : defer_pass_kernel<1>;
    return pl;
}

// Sliced-ELL block of the lines of a sparse matrix given as CSR-like
// (ptr, idx, val) over n_lines lines; with `sort`, lines sorted by length,
// longest first, else line l of the block is line l of the matrix.
achr_status build_ell(SlicedEll &E, int n_lines, const std::vector<int> &ptr, const std::vector<int> &idx,
                      const std::vector<double> &val, bool &exact32, bool sort) {
    std::vector<int> order((size_t)n_lines);
    for (int l = 0; l < n_lines; ++l) order[(size_t)l] = l;
    if (sort)
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
            return ptr[(size_t)a + 1] - ptr[(size_t)a] > ptr[(size_t)b + 1] - ptr[(size_t)b];
        });
    const int groups = (n_lines + 31) / 32;
    std::vector<int> off((size_t)groups + 1, 0), line((size_t)groups * 32, -1);
    std::vector<unsigned short> eidx;
    std::vector<float> vh, vl;
    for (int g = 0; g < groups; ++g) {
        int len = 0;
        for (int l = 0; l < 32 && 32 * g + l < n_lines; ++l) {
            const int L = order[(size_t)(32 * g + l)];
            line[(size_t)(32 * g + l)] = L;
            len = std::max(len, ptr[(size_t)L + 1] - ptr[(size_t)L]);
        }
        off[(size_t)g + 1] = off[(size_t)g] + 32 * len;
        for (int t = 0; t < len; ++t)
            for (int l = 0; l < 32; ++l) {
                const int L = line[(size_t)(32 * g + l)];
                const bool real = L >= 0 && t < ptr[(size_t)L + 1] - ptr[(size_t)L];
                const double v = real ? val[(size_t)ptr[(size_t)L] + t] : 0.0;
                const float h = (float)v;
                const float lo = (float)(v - (double)h);
                if (lo != 0.0f) exact32 = false;
                eidx.push_back((unsigned short)(real ? idx[(size_t)ptr[(size_t)L] + t] : 0));
                vh.push_back(h);
                vl.push_back(lo);
            }
    }
    E.groups = groups;
    DEFER_TRY(E.off.upload(off.data(), off.size()));
    DEFER_TRY(E.line.upload(line.data(), line.size()));
    DEFER_TRY(E.idx.upload(eidx.data(), eidx.size()));
    DEFER_TRY(E.vh.upload(vh.data(), vh.size()));
    DEFER_TRY(E.vl.upload(vl.data(), vl.size()));
    return ACHR_OK;
}

// B in the device row order: Bd[q][q'] = B[order[q]][order[q']] (q' < m; the K padding stays
// zero), so that the chain kernel's residual rows, R, Z and r all use the row order in which the
// chain kernel computes S x and every access to them is coalesced.
__global__ void permute_pinv(int m, int kpad, const int *__restrict__ order, const __nv_bfloat16 *__restrict__ Bh,
                             const __nv_bfloat16 *__restrict__ Bl, __nv_bfloat16 *__restrict__ Dh,
                             __nv_bfloat16 *__restrict__ Dl) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)m * kpad) return;
    const int q = (int)(t / kpad), k = (int)(t % kpad);
    if (k >= m) {
        Dh[t] = __float2bfloat16_rn(0.0f);
        Dl[t] = __float2bfloat16_rn(0.0f);
        return;
    }
    const size_t src = (size_t)__ldg(order + q) * (size_t)kpad + (size_t)__ldg(order + k);
    Dh[t] = Bh[src];
    Dl[t] = Bl[src];
}

EllView view(const SlicedEll &E) {
    return EllView{E.groups, E.off.p, E.line.p, E.idx.p, E.vh.p, E.vl.p};
}

// The per-model part of the state (B in the device row order, the sliced-ELL
// blocks); the context takes it only once all of it is built.
achr_status init_defer(const achr_ctx *ctx, DeferState *D) {
    {
        const ReprojState &R = *ctx->reproj;
        D->kpad = R.kpad;
        D->ld = (ctx->n + 1) & ~1;
        D->ldz = (ctx->m + 3) & ~3;
        const int n = ctx->n, m = ctx->m;
        const std::vector<int> &order = ctx->h_row_order;  // device row q = model row order[q]
        {
            DevBuf<int> ord;
            DEFER_TRY(ord.upload(order.data(), order.size()));
            const size_t cnt = (size_t)m * (size_t)D->kpad;
            DEFER_TRY(D->Bh.alloc(cnt));
            DEFER_TRY(D->Bl.alloc(cnt));
            permute_pinv<<<(unsigned)((cnt + 255) / 256), 256>>>(m, D->kpad, ord.p, R.Bh.p, R.Bl.p, D->Bh.p, D->Bl.p);
            DEFER_TRY(cudaGetLastError());
            DEFER_TRY(cudaDeviceSynchronize());
        }
        // S (rows) and S^T (columns of S), rows in the device order: longest first, the order
        // the chain kernel computes S x in, so the rows block keeps that order.
        std::vector<int> rp((size_t)m + 1, 0), ci;
        std::vector<double> rv;
        ci.reserve(ctx->h_colidx.size());
        rv.reserve(ctx->h_val.size());
        for (int q = 0; q < m; ++q) {
            const int r = order[(size_t)q];
            for (int t = ctx->h_rowptr[(size_t)r]; t < ctx->h_rowptr[(size_t)r + 1]; ++t) {
                ci.push_back(ctx->h_colidx[(size_t)t]);
                rv.push_back(ctx->h_val[(size_t)t]);
            }
            rp[(size_t)q + 1] = (int)ci.size();
        }
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
        bool exact = true;
        achr_status st = build_ell(D->cols, n, cp, ri, cv, exact, true);
        if (st != ACHR_OK) return st;
        st = build_ell(D->rows, m, rp, ci, rv, exact, false);  // line q is device row q
        if (st != ACHR_OK) return st;
        D->exact32 = exact;
    }
    return ACHR_OK;
}

achr_status ensure_defer(achr_ctx *ctx, int chains, int segments) {
    DeferState *D = ctx->defer;
    if (!D) {
        std::unique_ptr<DeferState> nd(new (std::nothrow) DeferState());
        if (!nd) return set_err(ACHR_ERR_NOMEM, "allocation failed");
        const achr_status st = init_defer(ctx, nd.get());
        if (st != ACHR_OK) return st;
        D = ctx->defer = nd.release();
    }
    if (D->cap < chains) {
        D->cap = 0;
        const size_t c = (size_t)chains;
        DEFER_TRY(D->x.alloc(c * (size_t)D->ld));
        DEFER_TRY(D->A.alloc(c * (size_t)D->ld));
        DEFER_TRY(D->flags.alloc(c));
        DEFER_TRY(D->Rh.alloc(c * (size_t)D->kpad));
        DEFER_TRY(D->Rl.alloc(c * (size_t)D->kpad));
        // the K padding of R (rows m..kpad) is never written and must be zero
        DEFER_TRY(cudaMemset(D->Rh.p, 0, sizeof(unsigned short) * c * (size_t)D->kpad));
        DEFER_TRY(cudaMemset(D->Rl.p, 0, sizeof(unsigned short) * c * (size_t)D->kpad));
        DEFER_TRY(D->rd.alloc(c * (size_t)D->ldz));
        DEFER_TRY(D->Z.alloc(c * (size_t)D->ldz));
        DEFER_TRY(D->r.alloc(c * (size_t)D->ldz));
        DEFER_TRY(D->dxh.alloc(c * (size_t)D->ld));
        DEFER_TRY(D->dxl.alloc(c * (size_t)D->ld));
        DEFER_TRY(D->r0.alloc(c));
        D->cap = chains;
    }
    if (D->any_cap < segments) {
        D->any_cap = 0;
        DEFER_TRY(D->any.alloc((size_t)segments));
        D->any_cap = segments;
    }
    return ACHR_OK;
}

}  // namespace

bool defer_selected(const achr_ctx *ctx) {
    const achr_options &o = ctx->opt;
    if (o.check_period <= 0 || ctx->m <= 0) return false;
    const int np = chain_padded_length(ctx->n, o.threads_per_chain);
    // S x is staged in the chain kernel's column buffer, below its zero padding (the padding
    // beyond the column's ldw entries must stay zero: padded reactions read it as their w)
    if (np == 0 || ctx->m > ctx->ldw) return false;
    // Each BF16-split pass multiplies the remaining error by roughly 1.5e-6 times the
    // condition number of S S^T (measured: 1.9e-3 at 1265); beyond 2e4 the passes
    // converge too slowly to be worth it, and far beyond they diverge.
    if (ctx->kappa_sst > kDeferMaxKappa) return false;
    if (o.reproject_form == 3) return true;
    if (o.reproject_form != 0 || ctx->n_dirs > 0) return false;
    return ctx->warmup_residual > o.residual_tol / 8.0 && (double)ctx->n * (double)ctx->d >= 2.5e5;
}

achr_status defer_sample(achr_ctx *ctx, const ChainArgs &a_in, int threads_per_chain, cudaStream_t s, bool timed) {
    achr_status st = ensure_reproj(ctx);
    if (st != ACHR_OK) return st;
    // Steps [S0, E) of every chain (S0 > 0: chains resumed from a_in.x_in / A_in).
    const int P = a_in.P, S0 = a_in.step0, E = a_in.step0 + a_in.T, k = a_in.check_period;
    if (P <= 0) return ACHR_OK;
    const int cap = std::min(P, kDeferChunk);
    const int segments = E / k - S0 / k + 3;
    // one gate word per launch and pass: [seg * (kMaxPasses + 1) + pass]
    st = ensure_defer(ctx, cap, segments * (kMaxPasses + 1));
    if (st != ACHR_OK) return st;
    DeferState &D = *ctx->defer;
    const ReprojState &R = *ctx->reproj;
    D.ev_used = 0;
    D.chains_per_sweep = (double)P / (double)((P + cap - 1) / cap);
    auto mark = [&]() -> cudaError_t {  // record the next timing event on the stream
        if (!timed) return cudaSuccess;
        if (D.ev_used == (int)D.ev.size()) {
            cudaEvent_t e = nullptr;
            cudaError_t ce = cudaEventCreate(&e);
            if (ce != cudaSuccess) return ce;
            D.ev.push_back(e);
        }
        return cudaEventRecord(D.ev[(size_t)D.ev_used++], s);
    };
    const int passes = ctx->opt.reprojection_passes > 0 ? ctx->opt.reprojection_passes : kMaxPasses;
    const double fine_tol = ctx->opt.residual_tol * 1e-3;

    int dev = 0, sms = 0, per_sm = 0, per_sm1 = 0;
    DEFER_TRY(cudaGetDevice(&dev));
    DEFER_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const PassPlan pl = plan_passes(D.ld, D.ldz, D.exact32);
    if (pl.smem1 > kPassSmemMax || pl.smem > kPassSmemMax)
        return set_err(ACHR_ERR_UNSUPPORTED, "model too large for the batched reprojection's shared memory");
    DEFER_TRY(cudaFuncSetAttribute(pl.pass, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pl.smem));
    DEFER_TRY(cudaFuncSetAttribute(pl.pass1, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pl.smem1));
    DEFER_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pl.pass, kPassThreads, pl.smem));
    DEFER_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm1, pl.pass1, kPassThreads, pl.smem1));
    if (per_sm < 1 || per_sm1 < 1)
        return set_err(ACHR_ERR_UNSUPPORTED, "model too large for the batched reprojection's update");

    ctx->last_segments = 0;
    ctx->last_launches = 0;
    for (int c0 = 0; c0 < P; c0 += cap) {
        const int pc = std::min(cap, P - c0);
        DEFER_TRY(cudaMemsetAsync(D.flags.p, 0, sizeof(unsigned) * (size_t)pc, s));
        DEFER_TRY(cudaMemsetAsync(D.any.p, 0, sizeof(unsigned long long) * (size_t)segments * (kMaxPasses + 1), s));
        ChainArgs a = a_in;
        a.P = pc;
        a.chain_offset = a_in.chain_offset + (unsigned long long)c0;
        a.out = a_in.out + c0;  // columns c0.. of the n x P row-major output (and state, when resumed)
        if (a_in.x_in) a.x_in = a_in.x_in + c0;
        if (a_in.A_in) a.A_in = a_in.A_in + c0;
        if (a_in.A_out) a.A_out = a_in.A_out + c0;
        a.pinv32 = nullptr;     // no reprojection inside the chain kernel
        a.seg = 1;
        a.seg_x = D.x.p;
        a.seg_A = D.A.p;
        a.ld_seg = D.ld;
        a.seg_flags = D.flags.p;
        a.seg_Rh = D.Rh.p;
        a.seg_Rl = D.Rl.p;
        a.kpad = D.kpad;
        a.seg_rd = D.rd.p;
        a.ld_r = D.ldz;
        a.seg_dxh = D.dxh.p;
        a.seg_dxl = D.dxl.p;
        const int pass_grid = (int)std::min<long long>((long long)sms * per_sm, (pc + pl.cpb - 1) / pl.cpb);
        const int pass1_grid = (int)std::min<long long>((long long)sms * per_sm1, (pc + pl.cpb1 - 1) / pl.cpb1);
        PassArgs pa{};
        pa.n = ctx->n;
        pa.m = ctx->m;
        pa.kpad = D.kpad;
        pa.P = pc;
        pa.ld = D.ld;
        pa.ldz = D.ldz;
        pa.flags = D.flags.p;
        pa.Z = D.Z.p;
        pa.rd = D.rd.p;
        pa.r = D.r.p;
        pa.dxh = D.dxh.p;
        pa.dxl = D.dxl.p;
        pa.r0 = D.r0.p;
        pa.Rh = reinterpret_cast<__nv_bfloat16 *>(D.Rh.p);
        pa.Rl = reinterpret_cast<__nv_bfloat16 *>(D.Rl.p);
        pa.cols = view(D.cols);
        pa.rows = view(D.rows);
        pa.fine_tol = (float)fine_tol;
        pa.rel_tol = kRelTol;
        pa.residual_tol = (float)ctx->opt.residual_tol;
        pa.counters = a_in.counters;
        int s0 = S0, seg = 0;
        for (;;) {
            // The launch runs to the first check step at or after s0 (the reference
            // checks at steps that are multiples of the period, ACHRCuda.cu:325).
            const int c = (int)(((long long)s0 + k - 1) / k * k);
            const bool ends_on_check = c <= E - 1;
            a.step0 = s0;
            a.T = ends_on_check ? c - s0 + 1 : E - s0;
            a.seg_final = ends_on_check ? 0 : 1;
            unsigned long long *gate = D.any.p + (size_t)seg * (kMaxPasses + 1);
            a.seg_any = gate;  // pass 0 is needed when some chain's check fired
            DEFER_TRY(mark());
            DEFER_TRY(launch_chains(a, threads_per_chain, s));
            DEFER_TRY(mark());
            ++ctx->last_segments;
            ++ctx->last_launches;
            if (!ends_on_check) break;
            for (int pass = 0; pass < passes; ++pass) {
                TcGemm g{pc, R.m, R.kpad, 3, D.Rh.p, D.Rl.p, (long long)R.kpad, D.Bh.p, D.Bl.p, (long long)R.kpad,
                         D.Z.p, (long long)D.ldz};
                g.gate = gate + pass;  // skipped when no chain needs this pass
                g.gate_max = 0;
                if (const char *why = tc_gemm_check(g)) return set_err(ACHR_ERR_INVALID, why);
                DEFER_TRY(launch_tc_gemm(g, a_in.counters + CNT_ERROR, s));
                pa.pass = pass;
                pa.last = pass + 1 == passes ? 1 : 0;
                pa.this_gate = gate + pass;
                pa.next_any = gate + pass + 1;
                if (pass == 0) pl.pass1<<<(unsigned)pass1_grid, kPassThreads, pl.smem1, s>>>(pa);
                else pl.pass<<<(unsigned)pass_grid, kPassThreads, pl.smem, s>>>(pa);
                DEFER_TRY(cudaGetLastError());
                ctx->last_launches += 2;
            }
            ++seg;
            s0 = c + 1;
            if (s0 >= E) {  // the run's last step was a check step: a launch that only finishes it
                a.step0 = E;
                a.T = 0;
                a.seg_final = 1;
                a.seg_any = D.any.p + (size_t)seg * (kMaxPasses + 1);
                DEFER_TRY(mark());
                DEFER_TRY(launch_chains(a, threads_per_chain, s));
                DEFER_TRY(mark());
                ++ctx->last_segments;
                ++ctx->last_launches;
                break;
            }
        }
    }
    DEFER_TRY(mark());
    return ACHR_OK;
}

achr_status defer_times(achr_ctx *ctx, double *chain_ms, double *pass_ms, double *chains_per_sweep) {
    DeferState *D = ctx->defer;
    double c = 0.0, q = 0.0;
    if (D) {
        // events: (before, after) of every chain-kernel launch, then one at the end
        for (int k = 0; k + 1 < D->ev_used; ++k) {
            float ms = 0.0f;
            DEFER_TRY(cudaEventElapsedTime(&ms, D->ev[(size_t)k], D->ev[(size_t)k + 1]));
            if (k % 2 == 0) c += ms;
            else q += ms;
        }
    }
    *chain_ms = c;
    *pass_ms = q;
    *chains_per_sweep = D ? D->chains_per_sweep : 0.0;
    return ACHR_OK;
}

}  // namespace achr
