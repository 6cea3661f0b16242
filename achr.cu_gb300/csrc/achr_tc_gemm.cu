// Tensor-core GEMM for sm_103a: tcgen05.mma (kind::f16, BF16 operands, FP32
// accumulator in tensor memory), operands staged by 2-D TMA with 128-byte
// swizzle through a 4-stage mbarrier pipeline.
//
//   C (M x N, FP32, row-major) = sum over split terms  A_s (M x K) * B_t (N x K)^T
//
// Operands are BF16, row-major with K contiguous ("K-major").  nsplit = 1
// computes A0 B0^T; nsplit = 3 computes A0 B0^T + A0 B1^T + A1 B0^T, the three
// leading products of hi/lo BF16 splits (A = A0 + A1, B = B0 + B1), all
// accumulated in the same FP32 tensor-memory accumulator.  This contraction is
// the dense part of the batched null-space reprojection.  The reference has
// no counterpart: its reprojection (ACHRcu/ACHRCuda.cu:208-230) is a per-chain
// FP64 GEMV pair.
//
// A persistent CTA per SM computes 128 x 256 tiles with six warps:
//   warp 0      one thread issues the TMA loads of A and B k-blocks (64 wide);
//   warp 1      allocates 512 tensor-memory columns (two accumulators); one
//               thread issues four 128x256x16 MMAs per k-block, commits each
//               stage back to the producer and each finished accumulator to
//               the epilogue;
//   warps 2..5  read an accumulator (tcgen05.ld, 32 lanes each: warp w sees
//               lanes 32 (w mod 4) .. +31), store FP32 rows of C and hand the
//               accumulator back, while the MMAs of the next tile run.
// Every mbarrier wait is bounded (2 s); on expiry the kernel records an error
// bit and skips the rest of its work.  Before the CTA leaves, the producer
// waits for every TMA load it issued to land (so no copy writes into shared
// memory the CTA no longer owns) and the MMA thread waits for every MMA it
// issued to complete before tensor memory is freed.  An MMA is issued only
// after its operands have landed, so it depends on nothing but the tensor
// pipe and always completes; that wait is repeated, bounded each time, until
// it does.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <mutex>

#include "achr_internal.h"

namespace achr {
namespace {

constexpr int kBM = 128, kBN = 256, kBK = 64, kStages = 4;
constexpr unsigned kABytes = kBM * kBK * 2;  // 16 KB
constexpr unsigned kBBytes = kBN * kBK * 2;  // 32 KB
constexpr unsigned kStageBytes = kABytes + kBBytes;
constexpr unsigned kTmemCols = 512;  // two 256-column FP32 accumulators
constexpr int kThreads = 192;
constexpr size_t kSmemBytes = (size_t)kStages * kStageBytes + 1024 + 160;
constexpr unsigned long long kTcWaitNs = 2000000000ull;

// Instruction descriptor of tcgen05.mma kind::f16: D FP32 (bits 4-5 = 1),
// A and B BF16 (bits 7-9 = 1, 10-12 = 1), both K-major (bits 15, 16 = 0),
// N >> 3 in bits 17-22, M >> 4 in bits 24-28.
constexpr unsigned kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(kBN >> 3) << 17) |
                            ((unsigned)(kBM >> 4) << 24);

__device__ __forceinline__ unsigned s_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long tc_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void bar_init(unsigned bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void bar_expect_tx(unsigned bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool bar_try(unsigned bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool bar_wait(unsigned bar, unsigned parity) {
    if (bar_try(bar, parity)) return true;
    const unsigned long long t0 = tc_ns();
    for (;;) {
        if (bar_try(bar, parity)) return true;
        if (tc_ns() - t0 > kTcWaitNs) return false;
    }
}

// 2-D tiled TMA load of the box at (x = k element, y = row) into shared memory.
__device__ __forceinline__ void tma_2d(unsigned dst, const CUtensorMap *map, int x, int y, unsigned bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
            "r"(dst),
        "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

// Shared-memory matrix descriptor, K-major with 128-byte swizzle: start
// address >> 4 (bits 0-13), stride between 8-row groups 1024 B >> 4 (bits
// 32-45), descriptor version 1 (bits 46-47), swizzle mode 2 = 128 B (bits
// 61-63); the leading-dimension offset is unused for this layout.
__device__ __forceinline__ uint64_t sw128_desc(unsigned saddr) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(1024u >> 4) << 32) | (1ull << 46) | (2ull << 61);
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tc_mma(unsigned d_tmem, uint64_t adesc, uint64_t bdesc, unsigned accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
        : "memory");
}

// Arrive on `bar` once every tcgen05.mma this thread issued so far has completed.
__device__ __forceinline__ void tc_commit(unsigned bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

// 16 consecutive FP32 accumulator columns of this thread's tensor-memory lane.
__device__ __forceinline__ void tmem_ld16(unsigned taddr, float (&v)[16]) {
    unsigned r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
        "%14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    // The wait names the destination registers so that no use moves above it.
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]),
                   "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]),
                   "+r"(r[14]), "+r"(r[15])
                 :
                 : "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

struct GemmParams {
    int M, N, K, nsplit;
    float *C;
    long long ldc;
    int vec;  // 1: rows of C are 16-byte aligned (float4 stores)
    int n_fast;  // tile order: 1 = N fastest (A, the larger operand, streamed once), 0 = M fastest
    unsigned long long *err;
    const unsigned long long *gate;  // non-NULL: skip the whole GEMM when *gate <= gate_max
    unsigned long long gate_max;
};

__device__ __forceinline__ void bar_arrive(unsigned bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// Persistent: one CTA per SM walks the output tiles tile = blockIdx.x + k *
// gridDim.x, along the dimension of the smaller operand fastest: the CTAs
// working at the same time then share the tiles of the larger operand, which
// leaves DRAM once, while the smaller one stays in L2 (with M fastest and
// 100,000 rows of A, A would be read again for every 256 columns of B).
// Two 256-column accumulators in tensor memory let the epilogue of one tile
// overlap the MMAs of the next; the k-block ring runs on across tiles.
__global__ void __launch_bounds__(kThreads, 1)
    tc_gemm_bf16_kernel(const __grid_constant__ CUtensorMap mA0, const __grid_constant__ CUtensorMap mA1,
                        const __grid_constant__ CUtensorMap mB0, const __grid_constant__ CUtensorMap mB1,
                        const GemmParams p) {
    if (p.gate && *p.gate <= p.gate_max) return;  // uniform over the grid: written by an earlier kernel
    extern __shared__ unsigned char smem_raw[];
    const unsigned raw = s_addr(smem_raw);
    const unsigned base = (raw + 1023u) & ~1023u;  // 128-byte swizzle atoms repeat every 1024 B
    const unsigned bar_full = base + kStages * kStageBytes;
    const unsigned bar_empty = bar_full + 8 * kStages;
    const unsigned bar_accf = bar_empty + 8 * kStages;  // 2: accumulator b holds a finished tile
    const unsigned bar_acce = bar_accf + 16;            // 2: the epilogue has drained accumulator b
    const unsigned bar_done = bar_acce + 16;            // every MMA of this CTA has completed
    const unsigned tmem_slot = bar_done + 8;
    const unsigned *tmem_slot_ptr = reinterpret_cast<const unsigned *>(smem_raw + (tmem_slot - raw));

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m_tiles = (p.M + kBM - 1) / kBM, n_tiles = (p.N + kBN - 1) / kBN;
    const int tiles = m_tiles * n_tiles;
    const int kb_split = p.K / kBK;
    const int total = kb_split * p.nsplit;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            bar_init(bar_full + 8 * s, 1);
            bar_init(bar_empty + 8 * s, 1);
        }
        for (int b = 0; b < 2; ++b) {
            bar_init(bar_accf + 8 * b, 1);
            bar_init(bar_acce + 8 * b, 4);  // one arrival per epilogue warp
        }
        bar_init(bar_done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tmem_slot),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = *(volatile const unsigned *)tmem_slot_ptr;
    bool ok = true;

    if (warp == 0) {
        if (lane == 0) {
            int it = 0;  // k-blocks issued by this CTA so far (the ring position)
            for (int tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
                const int m0 = (p.n_fast ? tile / n_tiles : tile % m_tiles) * kBM;
                const int n0 = (p.n_fast ? tile % n_tiles : tile / m_tiles) * kBN;
                for (int kb = 0; kb < total; ++kb, ++it) {
                    const int s = it % kStages;
                    const unsigned round = (unsigned)(it / kStages);
                    if (it >= kStages && !bar_wait(bar_empty + 8 * s, (round - 1u) & 1u)) {
                        ok = false;
                        break;
                    }
                    const int split = kb / kb_split;
                    const int kx = (kb - split * kb_split) * kBK;
                    const CUtensorMap *ma = split == 2 ? &mA1 : &mA0;
                    const CUtensorMap *mb = split == 1 ? &mB1 : &mB0;
                    const unsigned sa = base + (unsigned)s * kStageBytes;
                    bar_expect_tx(bar_full + 8 * s, kStageBytes);
                    tma_2d(sa, ma, kx, m0, bar_full + 8 * s);
                    tma_2d(sa + kABytes, mb, kx, n0, bar_full + 8 * s);
                }
            }
            // Drain: the last load armed on each stage (use it/kStages - 1 or the
            // round below it) must have landed before shared memory is released.
            // Each stage is at most one phase ahead of its last arming, so the
            // parity names that phase unambiguously.
            for (int j = (it > kStages ? it - kStages : 0); j < it; ++j) {
                const int s = j % kStages;
                const unsigned round = (unsigned)(j / kStages);
                if (!bar_wait(bar_full + 8 * s, round & 1u)) ok = false;
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            int it = 0, t = 0;
            for (int tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x, ++t) {
                const int b = t & 1;
                const unsigned use = (unsigned)(t >> 1);
                if (t >= 2 && !bar_wait(bar_acce + 8 * b, (use - 1u) & 1u)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const unsigned acc = tmem + (unsigned)(b * (int)kBN);
                for (int kb = 0; kb < total; ++kb, ++it) {
                    const int s = it % kStages;
                    const unsigned round = (unsigned)(it / kStages);
                    if (!bar_wait(bar_full + 8 * s, round & 1u)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const unsigned sa = base + (unsigned)s * kStageBytes;
#pragma unroll
                    for (int k = 0; k < kBK / 16; ++k)  // 16 BF16 = 32 bytes of K per MMA
                        tc_mma(acc, sw128_desc(sa + 32u * k), sw128_desc(sa + kABytes + 32u * k),
                               (kb | k) != 0 ? 1u : 0u);
                    tc_commit(bar_empty + 8 * s);
                }
                if (ok) tc_commit(bar_accf + 8 * b);
            }
            // Before tensor memory is freed: every MMA issued above has completed.
            // (Their operands had landed when they were issued, so they finish;
            // the bounded wait is repeated rather than abandoned.)
            tc_commit(bar_done);
            for (int tries = 0; tries < 8 && !bar_wait(bar_done, 0); ++tries) ok = false;
        }
        __syncwarp();
    } else {
        const int q = warp & 3;  // tensor-memory lanes 32q .. 32q + 31
        int t = 0;
        for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x, ++t) {
            const int b = t & 1;
            const unsigned use = (unsigned)(t >> 1);
            bool got = bar_wait(bar_accf + 8 * b, use & 1u);
            got = __all_sync(0xffffffffu, got);
            if (!got) {
                ok = false;
                break;
            }
            tc_fence_after();
            const int m0 = (p.n_fast ? tile / n_tiles : tile % m_tiles) * kBM;
            const int n0 = (p.n_fast ? tile % n_tiles : tile / m_tiles) * kBN;
            const int row = m0 + q * 32 + lane;
            float *crow = p.C + (long long)row * p.ldc;
            const unsigned acc = tmem + (unsigned)(b * (int)kBN) + ((unsigned)(q * 32) << 16);
#pragma unroll 1
            for (int c = 0; c < kBN; c += 16) {
                float v[16];
                tmem_ld16(acc + (unsigned)c, v);
                const int col = n0 + c;
                if (row < p.M && col < p.N) {
                    if (p.vec && col + 16 <= p.N) {
                        float4 *d4 = reinterpret_cast<float4 *>(crow + col);
#pragma unroll
                        for (int j = 0; j < 4; ++j) d4[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
                    } else {
#pragma unroll
                        for (int j = 0; j < 16; ++j)
                            if (col + j < p.N) crow[col + j] = v[j];
                    }
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) bar_arrive(bar_acce + 8 * b);
        }
    }
    if (!ok) atomicOr(p.err, (unsigned long long)ERR_TC_TIMEOUT);
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
    }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_tiled() {
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    });
    return fn;
}

// Row-major BF16 matrix (rows x K, leading dimension ld elements) as a TMA
// map with boxes of 64 K-elements (128 bytes, one swizzle row) x box_rows.
bool bf16_map(CUtensorMap *m, const void *ptr, long long rows, long long K, long long ld, int box_rows) {
    PFN_cuTensorMapEncodeTiled_v12000 fn = encode_tiled();
    if (!fn) return false;
    cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)box_rows};
    cuuint32_t es[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(ptr), dims, strides, box, es,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

const char *tc_gemm_check(const TcGemm &g) {
    if (g.M <= 0 || g.N <= 0 || g.K <= 0) return "M, N and K must be positive";
    if (g.K % kBK) return "K must be a multiple of 64";
    if (g.nsplit != 1 && g.nsplit != 3) return "nsplit must be 1 or 3";
    if (!g.A0 || !g.B0 || !g.C || (g.nsplit == 3 && (!g.A1 || !g.B1))) return "null operand";
    if (g.lda < g.K || g.ldb < g.K || g.ldc < g.N) return "leading dimension below the matrix extent";
    if (g.lda % 8 || g.ldb % 8) return "operand leading dimensions must be multiples of 8 elements";
    const uintptr_t al = (uintptr_t)g.A0 | (uintptr_t)g.B0 | (g.nsplit == 3 ? ((uintptr_t)g.A1 | (uintptr_t)g.B1) : 0);
    if (al & 15u) return "operands must be 16-byte aligned";
    if ((long long)((g.M + kBM - 1) / kBM) * ((g.N + kBN - 1) / kBN) > 2147483647ll) return "too many tiles";
    return nullptr;
}

cudaError_t launch_tc_gemm(const TcGemm &g, unsigned long long *err, cudaStream_t stream) {
    static std::once_flag attr_once;
    static cudaError_t attr_err = cudaSuccess;
    std::call_once(attr_once, [] {
        attr_err = cudaFuncSetAttribute(tc_gemm_bf16_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)kSmemBytes);
    });
    if (attr_err != cudaSuccess) return attr_err;
    CUtensorMap a0, a1, b0, b1;
    const void *A1 = g.nsplit == 3 ? g.A1 : g.A0;
    const void *B1 = g.nsplit == 3 ? g.B1 : g.B0;
    if (!bf16_map(&a0, g.A0, g.M, g.K, g.lda, kBM) || !bf16_map(&a1, A1, g.M, g.K, g.lda, kBM) ||
        !bf16_map(&b0, g.B0, g.N, g.K, g.ldb, kBN) || !bf16_map(&b1, B1, g.N, g.K, g.ldb, kBN))
        return cudaErrorInvalidValue;
    GemmParams p;
    p.M = g.M;
    p.N = g.N;
    p.K = g.K;
    p.nsplit = g.nsplit;
    p.C = g.C;
    p.ldc = g.ldc;
    p.vec = (((uintptr_t)g.C & 15u) == 0 && (g.ldc % 4) == 0) ? 1 : 0;
    p.n_fast = g.M > g.N ? 1 : 0;
    p.err = err;
    p.gate = g.gate;
    p.gate_max = g.gate_max;
    static int sms = 0;
    if (sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    const long long tiles = (long long)((g.M + kBM - 1) / kBM) * ((g.N + kBN - 1) / kBN);
    const unsigned grid = (unsigned)std::min<long long>(tiles, sms);
    tc_gemm_bf16_kernel<<<grid, kThreads, kSmemBytes, stream>>>(a0, a1, b0, b1, p);
    return cudaGetLastError();
}

double tc_gemm_flops(const TcGemm &g) { return 2.0 * g.M * (double)g.N * (double)g.K * g.nsplit; }

}  // namespace achr
