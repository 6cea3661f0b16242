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
// residual exceeds the tolerance, r = S x in FP32 and split into BF16 hi + lo
// (chain-major block R).  The batched passes then apply the same orthogonal
// projector to all of those chains at once,
//
//     x <- x - S^T z,   z = B r,   B = (S S^T)^+,
//
// z for every chain as one tensor-core GEMM Z = R B^T (three BF16 split
// products, FP32 accumulation, achr_tc_gemm.cu).  The first pass applies
// S^T z to the point in FP64 and recomputes the true residual S x in FP64, so
// its update leaves the null-space part of x alone to FP64 rounding and what
// is left of the residual is measured exactly (about 1e-4 of it on the
// generator-law models).  Later passes only move the point by that remainder:
// they form d = S^T z, add it to a correction dx and track r <- r - S d, all in
// FP32, and the next launch subtracts dx from the point in FP64.  A chain takes
// passes until max|r| falls to max(residual_tol / 100, 1e-7 of the residual its
// check found), so the corrected point is within about 1e-7 of the
// correction's own size of the FP64 projection; models whose S S^T has a
// condition number above 2e4 reproject in the chain kernel instead.  The next
// launch also clips the point and adds it to its centre accumulator before the
// chain's next step, the order the reference uses.  The decisions (which
// chains reproject) are the chain kernel's own FP64 residual, identical to the
// check it makes when it reprojects in place.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "achr_ctx.h"

extern "C" void achr_io_set_error(const char *msg);

namespace achr {

struct DeferState {
    int cap = 0;             // chains the buffers hold
    long long ld = 0;        // leading dimension of the chain-major state (n rounded up to even)
    int ldz = 0;             // leading dimension of Z and r (m rounded up to a multiple of 4)
    int kpad = 0;            // K of the GEMM: m rounded up to a multiple of 64
    DevBuf<double> x, A;     // cap x ld: points and centre accumulators between launches
    DevBuf<unsigned> flags;  // cap: SEG_* bits
    DevBuf<unsigned short> Rh, Rl;  // cap x kpad BF16 bits: S x of the chains that reproject
    DevBuf<float> Z;         // cap x ldz: B (S x)
    DevBuf<float> r;         // cap x ldz: S x in FP32, tracked through the passes
    DevBuf<float> dx;        // cap x ld: the passes' summed correction S^T z
    DevBuf<float> r0;        // cap: max|S x| of the chain when its check fired
    DevBuf<float> cv32, rv32;  // CSC and CSR values of S in FP32 (model row order)
    DevBuf<int> row_orig;    // m: device row order of S -> the model's row order
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
constexpr int kCorrThreads = 256;
constexpr int kMaxPasses = 8;              // passes of one deferred reprojection at most
// A chain's passes end once max|S x| <= max(residual_tol / 100, kRelTol times the residual its
// check found): the point is then within about that fraction of the correction's size of the
// FP64 projection (the correction is the residual's preimage).
constexpr float kRelTol = 1e-7f;

achr_status set_err(achr_status st, const std::string &msg) {
    achr_io_set_error(msg.c_str());
    return st;
}

#define DEFER_TRY(expr)                                                                                        \
    do {                                                                                                       \
        cudaError_t e_ = (expr);                                                                               \
        if (e_ != cudaSuccess) return set_err(ACHR_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

__global__ void to_f32_kernel(long long count, const double *__restrict__ in, float *__restrict__ out) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < count) out[t] = __double2float_rn(in[t]);
}

// The first pass, in FP64, for every chain flagged SEG_REPROJ (a CTA per chain
// at a time, chain-major rows): x <- x - S^T z1 and r1 = S x, both FP64, with z1
// the GEMM's row of that chain.  This pass removes nearly all of the residual
// (what is left is ~1e-4 of it), so its update must not leak into the null
// space and r1 must be the true residual of the new point: both are FP64 here,
// and the later passes, which only move the point by what is left, run in FP32.
// r1 goes to Rf (FP32) and R (BF16 hi/lo); max|r| of the chain's check (from
// Rf before the update) to r0; convergence as in defer_pass_kernel.
__global__ void __launch_bounds__(kCorrThreads)
    defer_first_pass_kernel(int n, int m, int kpad, int P, unsigned *__restrict__ flags, const float *__restrict__ Z,
                            float *__restrict__ Rf, long long ldz, double *__restrict__ X, long long ldx,
                            float *__restrict__ r0, const int *__restrict__ cp, const int *__restrict__ ri,
                            const double *__restrict__ cv, const int *__restrict__ rp, const int *__restrict__ ci,
                            const double *__restrict__ rv, __nv_bfloat16 *__restrict__ Rh,
                            __nv_bfloat16 *__restrict__ Rl, float fine_tol, float rel_tol, float residual_tol,
                            int last, const unsigned long long *this_gate, unsigned long long *next_any,
                            unsigned long long *counters) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ float wmax[kCorrThreads / 32][2];
    double *zd = reinterpret_cast<double *>(smem_raw);
    double *xs = zd + ldz;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (*this_gate == 0ull) return;  // no chain's check fired (the GEMM did not run either)
    if (blockIdx.x == 0 && tid == 0) atomicAdd(counters + CNT_GEMMS, 1ull);
    for (int p = blockIdx.x; p < P; p += gridDim.x) {
        if (!(flags[p] & SEG_REPROJ)) continue;  // uniform over the block
        const float *zp = Z + (size_t)p * (size_t)ldz;
        float *rp_ = Rf + (size_t)p * (size_t)ldz;
        float m0 = 0.0f;
        for (int i = tid; i < m; i += kCorrThreads) {
            zd[i] = (double)zp[i];
            m0 = fmaxf(m0, fabsf(rp_[i]));
        }
        __syncthreads();
        double *xp = X + (size_t)p * (size_t)ldx;
        for (int j = tid; j < n; j += kCorrThreads) {
            double dl = 0.0;
            const int q1 = __ldg(cp + j + 1);
            for (int q = __ldg(cp + j); q < q1; ++q) dl = fma(__ldg(cv + q), zd[__ldg(ri + q)], dl);
            const double xv = xp[j] - dl;
            xp[j] = xv;
            xs[j] = xv;
        }
        __syncthreads();
        __nv_bfloat16 *rh = Rh + (size_t)p * (size_t)kpad, *rl = Rl + (size_t)p * (size_t)kpad;
        float mx = 0.0f;
        for (int i = tid; i < m; i += kCorrThreads) {
            double acc = 0.0;
            const int q1 = __ldg(rp + i + 1);
            for (int q = __ldg(rp + i); q < q1; ++q) acc = fma(__ldg(rv + q), xs[__ldg(ci + q)], acc);
            const float rn = __double2float_rn(acc);
            rp_[i] = rn;
            mx = fmaxf(mx, fabsf(rn));
            if (!last) {
                const __nv_bfloat16 hi = __float2bfloat16_rn(rn);
                rh[i] = hi;
                rl[i] = __float2bfloat16_rn(rn - __bfloat162float(hi));
            }
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            m0 = fmaxf(m0, __shfl_xor_sync(0xffffffffu, m0, o));
        }
        if (lane == 0) {
            wmax[warp][0] = mx;
            wmax[warp][1] = m0;
        }
        __syncthreads();
        if (tid == 0) {
            for (int w = 1; w < kCorrThreads / 32; ++w) {
                mx = fmaxf(mx, wmax[w][0]);
                m0 = fmaxf(m0, wmax[w][1]);
            }
            atomicAdd(counters + CNT_PASSES, 1ull);
            r0[p] = m0;  // the residual the chain's check found
            if (mx <= fmaxf(fine_tol, rel_tol * m0)) {
                flags[p] &= ~SEG_REPROJ;  // converged
            } else if (!last) {
                if (*next_any == 0ull) atomicOr(next_any, 1ull);
            } else if (mx > residual_tol) {
                atomicOr(counters + CNT_ERROR, (unsigned long long)ERR_DEFER_DIVERGED);
            }
        }
        __syncthreads();
    }
}

// A later pass (pass >= 1) for every chain still flagged SEG_REPROJ (a CTA
// per chain at a time; chain-major rows, so every load and store is coalesced):
//     d = S^T z,  dx += d,  r <- r - S d,
// z the chain's row of the GEMM's B r.  Everything here is FP32: after the
// first pass the residual is ~1e-4 of what the check found, d is of that size,
// and r is tracked from the first pass's FP64 residual, so FP32 rounding stays
// relative to what is left, not to x; the point is touched once, in FP64, when
// the next launch subtracts dx (SEG_CORR).  A chain whose max|r| falls to
// max(fine_tol, rel_tol max|r0|) is done (flag cleared); any other has r split
// into R for the next pass and marks that pass as needed.  After the last pass
// a chain still above residual_tol raises ERR_DEFER_DIVERGED.  S is read in the
// model's row order (CSC for S^T z, CSR for S d), matching B.
__global__ void __launch_bounds__(kCorrThreads)
    defer_pass_kernel(int n, int m, int kpad, int P, int pass, unsigned *__restrict__ flags,
                      const float *__restrict__ Z, float *__restrict__ Rf, long long ldz, float *__restrict__ DX,
                      long long ldx, float *__restrict__ r0, const int *__restrict__ cp, const int *__restrict__ ri,
                      const float *__restrict__ cv, const int *__restrict__ rp, const int *__restrict__ ci,
                      const float *__restrict__ rv, __nv_bfloat16 *__restrict__ Rh, __nv_bfloat16 *__restrict__ Rl,
                      float fine_tol, float rel_tol, float residual_tol, int last,
                      const unsigned long long *this_gate, unsigned long long *next_any,
                      unsigned long long *counters) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ float wmax[kCorrThreads / 32];
    float *zs = reinterpret_cast<float *>(smem_raw);
    float *ds = zs + ldz;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (*this_gate == 0ull) return;  // no chain needed this pass (its GEMM did not run either)
    if (blockIdx.x == 0 && tid == 0) atomicAdd(counters + CNT_GEMMS, 1ull);
    for (int p = blockIdx.x; p < P; p += gridDim.x) {
        if (!(flags[p] & SEG_REPROJ)) continue;  // uniform over the block
        const float *zp = Z + (size_t)p * (size_t)ldz;
        for (int i = tid; i < m; i += kCorrThreads) zs[i] = zp[i];
        __syncthreads();
        float *dxp = DX + (size_t)p * (size_t)ldx;
        for (int j = tid; j < n; j += kCorrThreads) {
            float dl = 0.0f;
            const int q1 = __ldg(cp + j + 1);
            for (int q = __ldg(cp + j); q < q1; ++q) dl = fmaf(__ldg(cv + q), zs[__ldg(ri + q)], dl);
            ds[j] = dl;
            dxp[j] = pass == 1 ? dl : dxp[j] + dl;
        }
        __syncthreads();
        float *rp_ = Rf + (size_t)p * (size_t)ldz;
        __nv_bfloat16 *rh = Rh + (size_t)p * (size_t)kpad, *rl = Rl + (size_t)p * (size_t)kpad;
        float mx = 0.0f;
        for (int i = tid; i < m; i += kCorrThreads) {
            const float ro = rp_[i];
            float acc = 0.0f;
            const int q1 = __ldg(rp + i + 1);
            for (int q = __ldg(rp + i); q < q1; ++q) acc = fmaf(__ldg(rv + q), ds[__ldg(ci + q)], acc);
            const float rn = ro - acc;
            rp_[i] = rn;
            mx = fmaxf(mx, fabsf(rn));
            if (!last) {
                const __nv_bfloat16 hi = __float2bfloat16_rn(rn);
                rh[i] = hi;
                rl[i] = __float2bfloat16_rn(rn - __bfloat162float(hi));
            }
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if (lane == 0) wmax[warp] = mx;
        __syncthreads();
        if (tid == 0) {
            for (int w = 1; w < kCorrThreads / 32; ++w) mx = fmaxf(mx, wmax[w]);
            atomicAdd(counters + CNT_PASSES, 1ull);
            if (pass == 1) flags[p] |= SEG_CORR;  // dx now holds a correction for the next launch
            if (mx <= fmaxf(fine_tol, rel_tol * r0[p])) {
                flags[p] &= ~SEG_REPROJ;  // converged
            } else if (!last) {
                if (*next_any == 0ull) atomicOr(next_any, 1ull);
            } else if (mx > residual_tol) {
                atomicOr(counters + CNT_ERROR, (unsigned long long)ERR_DEFER_DIVERGED);
            }
        }
        __syncthreads();
    }
}

achr_status ensure_defer(achr_ctx *ctx, int chains, int segments) {
    DeferState *D = ctx->defer;
    if (!D) {
        D = new (std::nothrow) DeferState();
        if (!D) return set_err(ACHR_ERR_NOMEM, "allocation failed");
        ctx->defer = D;
        const ReprojState &R = *ctx->reproj;
        D->kpad = R.kpad;
        D->ld = (ctx->n + 1) & ~1;
        D->ldz = (ctx->m + 3) & ~3;
        DEFER_TRY(D->row_orig.upload(ctx->h_row_order.data(), ctx->h_row_order.size()));
        const long long nnz = (long long)R.cv.count;
        DEFER_TRY(D->cv32.alloc((size_t)nnz));
        DEFER_TRY(D->rv32.alloc((size_t)nnz));
        to_f32_kernel<<<(unsigned)((nnz + 255) / 256), 256>>>(nnz, R.cv.p, D->cv32.p);
        to_f32_kernel<<<(unsigned)((nnz + 255) / 256), 256>>>(nnz, R.rv.p, D->rv32.p);
        DEFER_TRY(cudaGetLastError());
        DEFER_TRY(cudaDeviceSynchronize());
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
        DEFER_TRY(D->Z.alloc(c * (size_t)D->ldz));
        DEFER_TRY(D->r.alloc(c * (size_t)D->ldz));
        DEFER_TRY(D->dx.alloc(c * (size_t)D->ld));
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
    if (np == 0 || ctx->m > np) return false;  // S x is staged in the chain kernel's column buffer
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
    const double fine_tol = ctx->opt.residual_tol * 0.01;

    int dev = 0, sms = 0, per_sm = 0;
    DEFER_TRY(cudaGetDevice(&dev));
    DEFER_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const size_t corr_smem = sizeof(float) * ((size_t)D.ldz + (size_t)D.ld);
    const size_t first_smem = sizeof(double) * ((size_t)D.ldz + (size_t)D.ld);
    int per_sm1 = 0;
    DEFER_TRY(cudaFuncSetAttribute(defer_pass_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)corr_smem));
    DEFER_TRY(cudaFuncSetAttribute(defer_first_pass_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)first_smem));
    DEFER_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, defer_pass_kernel, kCorrThreads, corr_smem));
    DEFER_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm1, defer_first_pass_kernel, kCorrThreads,
                                                            first_smem));
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
        a.row_orig = D.row_orig.p;
        a.seg_Rh = D.Rh.p;
        a.seg_Rl = D.Rl.p;
        a.kpad = D.kpad;
        a.seg_r = D.r.p;
        a.ld_r = D.ldz;
        a.seg_dx = D.dx.p;
        const int corr_grid = (int)std::min<long long>((long long)sms * per_sm, pc);
        const int first_grid = (int)std::min<long long>((long long)sms * per_sm1, pc);
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
                TcGemm g{pc, R.m, R.kpad, 3, D.Rh.p, D.Rl.p, (long long)R.kpad, R.Bh.p, R.Bl.p, (long long)R.kpad,
                         D.Z.p, (long long)D.ldz};
                g.gate = gate + pass;  // skipped when no chain needs this pass
                g.gate_max = 0;
                if (const char *why = tc_gemm_check(g)) return set_err(ACHR_ERR_INVALID, why);
                DEFER_TRY(launch_tc_gemm(g, a_in.counters + CNT_ERROR, s));
                if (pass == 0)
                    defer_first_pass_kernel<<<(unsigned)first_grid, kCorrThreads, first_smem, s>>>(
                        ctx->n, ctx->m, R.kpad, pc, D.flags.p, D.Z.p, D.r.p, D.ldz, D.x.p, D.ld, D.r0.p, R.cp.p,
                        R.ri.p, R.cv.p, R.rp.p, R.ci.p, R.rv.p, reinterpret_cast<__nv_bfloat16 *>(D.Rh.p),
                        reinterpret_cast<__nv_bfloat16 *>(D.Rl.p), (float)fine_tol, kRelTol,
                        (float)ctx->opt.residual_tol, passes == 1 ? 1 : 0, gate, gate + 1, a_in.counters);
                else
                    defer_pass_kernel<<<(unsigned)corr_grid, kCorrThreads, corr_smem, s>>>(
                        ctx->n, ctx->m, R.kpad, pc, pass, D.flags.p, D.Z.p, D.r.p, D.ldz, D.dx.p, D.ld, D.r0.p,
                        R.cp.p, R.ri.p, D.cv32.p, R.rp.p, R.ci.p, D.rv32.p,
                        reinterpret_cast<__nv_bfloat16 *>(D.Rh.p), reinterpret_cast<__nv_bfloat16 *>(D.Rl.p),
                        (float)fine_tol, kRelTol, (float)ctx->opt.residual_tol, pass + 1 == passes ? 1 : 0,
                        gate + pass, gate + pass + 1, a_in.counters);
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
