// Counter-based randomness of the sampler (host and device).
//
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), 10 rounds of
//   (hi0,lo0) = mulhilo(M0, c0), (hi1,lo1) = mulhilo(M1, c2)
//   c <- (hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0), k <- k + (W0, W1).
//
// Stream of one chain step (replaces the per-thread cuRAND XORWOW state seeded
// from clock64() in ACHRcu/ACHRCuda.cu:371, which cannot be reproduced):
//   key     = (seed_lo, seed_hi)
//   counter = (step, attempt, chain_lo, chain_hi)
//   warmup index  r = (w0 * W) >> 32                          (every attempt)
//   step uniform  U = ((((w2 << 32) | w3) >> 12) + 0.5) 2^-52  (attempt 0)
// One uniform per accepted step is reused by all redraws of the warmup index,
// as the reference pre-draws randVector[step] (ACHRCuda.cu:314, 382) while a
// rejected attempt draws a new index (ACHRCuda.cu:309-319).
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define ACHR_HD __host__ __device__ __forceinline__
#else
#define ACHR_HD inline
#endif

namespace achr {

struct Philox4 {
    uint32_t v[4];
};

ACHR_HD void mulhilo32(uint32_t a, uint32_t b, uint32_t &hi, uint32_t &lo) {
#if defined(__CUDA_ARCH__)
    hi = __umulhi(a, b);
    lo = a * b;
#else
    uint64_t p = (uint64_t)a * (uint64_t)b;
    hi = (uint32_t)(p >> 32);
    lo = (uint32_t)p;
#endif
}

ACHR_HD Philox4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo32(0xD2511F53u, c0, hi0, lo0);
        mulhilo32(0xCD9E8D57u, c2, hi1, lo1);
        const uint32_t n0 = hi1 ^ c1 ^ k0;
        const uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    Philox4 out;
    out.v[0] = c0;
    out.v[1] = c1;
    out.v[2] = c2;
    out.v[3] = c3;
    return out;
}

ACHR_HD Philox4 step_draw(uint64_t seed, uint64_t chain, uint32_t step, uint32_t attempt) {
    return philox4x32_10(step, attempt, (uint32_t)chain, (uint32_t)(chain >> 32), (uint32_t)seed,
                         (uint32_t)(seed >> 32));
}

ACHR_HD uint32_t warmup_index(const Philox4 &w, uint32_t n_warmup) {
    return (uint32_t)(((uint64_t)w.v[0] * (uint64_t)n_warmup) >> 32);
}

ACHR_HD double step_uniform(const Philox4 &w) {
    const uint64_t bits = ((uint64_t)w.v[2] << 32) | (uint64_t)w.v[3];
    return ((double)(bits >> 12) + 0.5) * 2.220446049250313080847263336181640625e-16;  // 2^-52
}

}  // namespace achr
