// Test helper (not part of the library): cuRAND's device Philox4_32_10 for a
// batch of (seed, subsequence, offset) triples, so the tests can pin the
// sampler's own Philox4x32-10 against the library.  With offset = 4 * (c1:c0)
// and subsequence = (c3:c2), curand_init + curand4 returns the Philox
// function of the counter (c0, c1, c2, c3) under the key (seed lo, seed hi).
#include <curand_kernel.h>
#include <stdint.h>

__global__ void philox_batch(int n, const unsigned long long *seed, const unsigned long long *subseq,
                             const unsigned long long *offset, uint4 *out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    curandStatePhilox4_32_10_t st;
    curand_init(seed[t], subseq[t], offset[t], &st);
    out[t] = curand4(&st);
}

extern "C" int curand_philox_batch(int n, const unsigned long long *seed, const unsigned long long *subseq,
                                   const unsigned long long *offset, unsigned *out) {
    unsigned long long *d_in = nullptr;
    uint4 *d_out = nullptr;
    const size_t b = sizeof(unsigned long long) * (size_t)n;
    if (cudaMalloc(&d_in, 3 * b) != cudaSuccess) return 1;
    if (cudaMalloc(&d_out, sizeof(uint4) * (size_t)n) != cudaSuccess) return 2;
    cudaMemcpy(d_in, seed, b, cudaMemcpyHostToDevice);
    cudaMemcpy(d_in + n, subseq, b, cudaMemcpyHostToDevice);
    cudaMemcpy(d_in + 2 * n, offset, b, cudaMemcpyHostToDevice);
    philox_batch<<<(n + 127) / 128, 128>>>(n, d_in, d_in + n, d_in + 2 * n, d_out);
    const cudaError_t e = cudaMemcpy(out, d_out, sizeof(uint4) * (size_t)n, cudaMemcpyDeviceToHost);
    cudaFree(d_in);
    cudaFree(d_out);
    return e == cudaSuccess ? 0 : 3;
}
