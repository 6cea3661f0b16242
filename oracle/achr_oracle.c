/*
 * CPU oracle for the ACHR sampling step -- TEST INFRASTRUCTURE ONLY.
 *
 * This file is the checker, not the product.  Only tests/, the smoke()
 * entry point and the CPU-baseline / reference arm of bench.py may load it.
 * The product path (the CUDA library and the ACHRCuda CLI) never links it.
 *
 * PARITY UNPINNED: the reference sampler (ACHRcu/ACHRCuda.cu) cannot be
 * built here (its device-side cudaDeviceSynchronize() is rejected by CUDA 13,
 * sm_37 is unsupported, GLPK/GSL are absent) and the reference ships no
 * golden outputs or known-answer tests for the sampler.  This restatement
 * therefore follows the reference source line by line and is pinned only by
 * (a) the published Philox4x32-10 known-answer vectors, (b) an independent
 * pure-Python/numpy restatement whose outputs are committed as fixtures, and
 * (c) invariants (bounds, ||Sv||_inf).
 *
 * What it restates (file:line in the reference project):
 *   - per-chain driver, centre copy, T steps            ACHRcu/ACHRCuda.cu:361-385
 *   - accepted-step loop, reject/redraw                 ACHRcu/ACHRCuda.cu:297-359
 *   - direction + ratio test                            ACHRcu/ACHRCuda.cu:251-289
 *   - x = prev + t u                                    ACHRcu/ACHRCuda.cu:242-249
 *   - every 10th step: r = S x, max|r| > 1e-9 check     ACHRcu/ACHRCuda.cu:232-240, 325-338
 *   - reprojection x <- N (N^T x)                       ACHRcu/ACHRCuda.cu:208-230, 338-343
 *   - clip, prev = x, centre EMA with pre-increment t   ACHRcu/ACHRCuda.cu:193-206, 346-351
 *   - tolerances maxMinTol=uTol=1e-9, dTol=1e-14         ACHRcu/ACHRCuda.cu:505, 508, 512
 * Semantic cross-check: VFWarmup/ACHRSamplerMOD.m:65-191 (MATLAB centre
 * weight uses the post-increment count; selectable with centre_offset=1).
 *
 * Deliberate, documented deviations from the reference:
 *   - randomness is the counter-based Philox4x32-10 stream defined below,
 *     keyed by (seed, chain, step, attempt), instead of cuRAND XORWOW seeded
 *     from clock64() (ACHRCuda.cu:371), which is not reproducible;
 *   - an empty candidate set in the ratio test (the reference dereferences
 *     thrust's end() iterator, ACHRCuda.cu:283-288) counts as a rejection;
 *   - a step that is rejected max_attempts times in a row stops the chain and
 *     is reported (the reference loops forever).
 * Extension without a reference counterpart: hit_and_run = 1 runs the same
 * loop with the warmup matrix read as a pool of directions (u = w_r/|w_r|,
 * no centre), the form the learned direction pool is sampled with.
 *
 * Build: oracle/build_oracle.sh (gcc -O2 -fopenmp -ffp-contract=off).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---------------------------------------------------------------------
 * Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
 * easy as 1, 2, 3", SC'11), restated from the paper: 10 rounds of
 *   (hi0,lo0) = mulhilo(M0, c0); (hi1,lo1) = mulhilo(M1, c2)
 *   c' = (hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0);  k += (W0, W1)
 * ------------------------------------------------------------------- */
#define PHILOX_M0 0xD2511F53u
#define PHILOX_M1 0xCD9E8D57u
#define PHILOX_W0 0x9E3779B9u
#define PHILOX_W1 0xBB67AE85u

void oracle_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4])
{
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int round = 0; round < 10; ++round) {
        uint64_t p0 = (uint64_t)PHILOX_M0 * (uint64_t)c0;
        uint64_t p1 = (uint64_t)PHILOX_M1 * (uint64_t)c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += PHILOX_W0; k1 += PHILOX_W1;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* The random stream of one chain step (shared contract with the CUDA path):
 *   key = (seed_lo, seed_hi); counter = (step, attempt, chain_lo, chain_hi)
 *   warmup index  r = (w0 * W) >> 32                        (attempt a)
 *   step uniform  U = ((((w2<<32)|w3) >> 12) + 0.5) * 2^-52  (attempt 0 only)
 * The step uniform is drawn once per accepted step and reused by every
 * redraw of the warmup index, as the reference pre-draws randVector[step]
 * (ACHRCuda.cu:314, 382) while rejected attempts redraw the index (:309). */
static void draw(uint64_t seed, uint64_t chain, uint32_t step, uint32_t attempt, uint32_t out[4])
{
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t ctr[4] = {step, attempt, (uint32_t)chain, (uint32_t)(chain >> 32)};
    oracle_philox4x32_10(ctr, key, out);
}

uint32_t oracle_warmup_index(uint64_t seed, uint64_t chain, uint32_t step, uint32_t attempt, uint32_t n_warmup)
{
    uint32_t w[4];
    draw(seed, chain, step, attempt, w);
    return (uint32_t)(((uint64_t)w[0] * (uint64_t)n_warmup) >> 32);
}

double oracle_step_uniform(uint64_t seed, uint64_t chain, uint32_t step)
{
    uint32_t w[4];
    draw(seed, chain, step, 0, w);
    uint64_t bits = ((uint64_t)w[2] << 32) | (uint64_t)w[3];
    return ((double)(bits >> 12) + 0.5) * 0x1p-52;
}

/* ---------------------------------------------------------------------
 * Problem description (host arrays, FP64).
 * ------------------------------------------------------------------- */
typedef struct {
    int32_t n;              /* reactions (columns of S) */
    int32_t m;              /* metabolites (rows of S) */
    int32_t n_warmup;       /* W */
    const double *warmup;   /* n x W, column-major: point j at warmup + j*n (ACHRCuda.cu:409) */
    const double *lb, *ub;  /* n */
    const int32_t *row_ptr; /* CSR of S: m+1 */
    const int32_t *col_idx; /* nnz */
    const double *val;      /* nnz */
    int32_t d;              /* null-space dimension n - istart */
    const double *N;        /* n x d, column-major (ACHRCuda.cu:484-489) */
    const double *centre;   /* n: mean of the warmup points (ACHRCuda.cu:414-434) */
} oracle_problem;

typedef struct {
    int32_t check_period;   /* 10 (ACHRCuda.cu:325); 0 = never */
    int32_t max_attempts;   /* redraws of one step before the chain is declared stuck */
    int32_t centre_offset;  /* 0: CUDA weights (ACHRCuda.cu:347-348); 1: MATLAB (ACHRSamplerMOD.m:174) */
    int32_t threads;        /* OpenMP threads over chains (<=0: library default) */
    int32_t hit_and_run;    /* 1: `warmup` holds directions, u = w_r / |w_r|, no centre (c = 0, never updated) */
    int32_t reserved;
    double residual_tol;    /* 1e-9 (ACHRCuda.cu:338) */
    double max_min_tol;     /* 1e-9 (ACHRCuda.cu:505) */
    double u_tol;           /* 1e-9 (ACHRCuda.cu:508) */
    double d_tol;           /* 1e-14 (ACHRCuda.cu:512) */
} oracle_options;

typedef struct {
    int64_t accepted;       /* accepted steps over all chains */
    int64_t rejected;       /* rejected attempts */
    int64_t checks;         /* residual checks */
    int64_t reprojections;  /* reprojections triggered */
    int64_t stuck_chains;   /* chains that hit max_attempts */
} oracle_stats;

/* One chain: restates stepPointProgress + createPoint for chain `chain`.
 * Work arrays: u, prev, c (n each), r (m), tmp (d). */
static void run_chain(const oracle_problem *pb, const oracle_options *op, uint64_t seed,
                      uint64_t chain, int32_t T, double *x_out, int64_t out_stride,
                      double *u, double *prev, double *c, double *x, double *r, double *tmp,
                      oracle_stats *st)
{
    const int n = pb->n, W = pb->n_warmup;
    const double uTol = op->u_tol, dTol = op->d_tol, maxMinTol = op->max_min_tol;
    /* ACHRCuda.cu:376-379: per-chain centre and prevPoint start at the global centre;
     * ACHRCuda.cu:739: the output points start at zero. */
    for (int i = 0; i < n; ++i) { c[i] = op->hit_and_run ? 0.0 : pb->centre[i]; prev[i] = pb->centre[i]; x[i] = 0.0; }
    int stuck = 0;
    for (int32_t s = 0; s < T && !stuck; ++s) {
        const double Ustep = oracle_step_uniform(seed, chain, (uint32_t)s);
        for (int32_t a = 0;; ++a) {
            if (a >= op->max_attempts) { stuck = 1; break; }
            const uint32_t rid = oracle_warmup_index(seed, chain, (uint32_t)s, (uint32_t)a, (uint32_t)W);
            const double *w = pb->warmup + (size_t)rid * (size_t)n;
            /* fillrandPoint, ACHRCuda.cu:260-267 */
            double ss = 0.0;
            for (int i = 0; i < n; ++i) { u[i] = w[i] - c[i]; }
            for (int i = 0; i < n; ++i) { ss += u[i] * u[i]; }
            const double norm = sqrt(ss);
            /* ACHRCuda.cu:266-281 */
            int k = 0;
            double minStep = 0.0, maxStep = 0.0;
            for (int i = 0; i < n; ++i) {
                u[i] = u[i] / norm;
                const double distUb = pb->ub[i] - prev[i];
                const double distLb = prev[i] - pb->lb[i];
                if (distUb > dTol && distLb > dTol) {
                    double mn, mx;
                    if (u[i] > uTol) { mn = -distLb / u[i]; mx = distUb / u[i]; }
                    else if (u[i] < -uTol) { mn = distUb / u[i]; mx = -distLb / u[i]; }
                    else continue;
                    /* thrust::max_element / min_element over the candidates (ACHRCuda.cu:283-288) */
                    if (k == 0 || mn > minStep) minStep = mn;
                    if (k == 0 || mx < maxStep) maxStep = mx;
                    ++k;
                }
            }
            /* ACHRCuda.cu:314-319 (empty candidate set: rejection, see header) */
            const double stepDist = Ustep * (maxStep - minStep) + minStep;
            if (k == 0 || (fabs(minStep) < maxMinTol && fabs(maxStep) < maxMinTol) || minStep > maxStep) {
                st->rejected++;
                continue;
            }
            /* advNextStep, ACHRCuda.cu:242-249 */
            for (int i = 0; i < n; ++i) x[i] = prev[i] + stepDist * u[i];
            /* ACHRCuda.cu:325-344: residual check every check_period steps */
            if (op->check_period > 0 && s % op->check_period == 0) {
                st->checks++;
                double mx = 0.0;
                for (int row = 0; row < pb->m; ++row) {
                    double acc = 0.0;
                    for (int32_t q = pb->row_ptr[row]; q < pb->row_ptr[row + 1]; ++q)
                        acc += pb->val[q] * x[pb->col_idx[q]];
                    r[row] = acc;
                    if (fabs(acc) > mx) mx = fabs(acc);
                }
                if (mx > op->residual_tol) {
                    st->reprojections++;
                    /* reprojectPoint: tmp = N^T x (ACHRCuda.cu:208-218) */
                    for (int j = 0; j < pb->d; ++j) {
                        const double *Nj = pb->N + (size_t)j * (size_t)n;
                        double acc = 0.0;
                        for (int i = 0; i < n; ++i) acc += Nj[i] * x[i];
                        tmp[j] = acc;
                    }
                    /* reprojectPoint2: x = N tmp (ACHRCuda.cu:220-230) */
                    for (int i = 0; i < n; ++i) {
                        double acc = 0.0;
                        for (int j = 0; j < pb->d; ++j) acc += pb->N[(size_t)j * (size_t)n + i] * tmp[j];
                        x[i] = acc;
                    }
                }
            }
            /* correctBounds with alpha/beta, ACHRCuda.cu:193-206, 347-350 */
            const double tc = (double)s + (double)op->centre_offset;
            const double alpha = ((double)W + tc) / ((double)W + tc + 1.0);
            const double beta = 1.0 / ((double)W + tc + 1.0);
            for (int i = 0; i < n; ++i) {
                if (x[i] > pb->ub[i]) x[i] = pb->ub[i];
                else if (x[i] < pb->lb[i]) x[i] = pb->lb[i];
                prev[i] = x[i];
                if (!op->hit_and_run) c[i] = alpha * c[i] + beta * x[i];
            }
            st->accepted++;
            break;
        }
    }
    if (stuck) st->stuck_chains++;
    for (int i = 0; i < n; ++i) x_out[(int64_t)i * out_stride] = x[i];
}

/* Sample P chains (ids chain_offset .. chain_offset+P-1) of T steps each.
 * out: n x P row-major (row = reaction, column = chain), the layout of the
 * reference's points array and File<ii> (ACHRCuda.cu:247, 749-755).
 * Returns 0 on success, -1 on allocation failure, -2 on bad arguments. */
int oracle_sample(const oracle_problem *pb, const oracle_options *op, uint64_t seed,
                  uint64_t chain_offset, int32_t P, int32_t T, double *out, oracle_stats *stats_out)
{
    if (!pb || !op || !out || pb->n <= 0 || pb->n_warmup <= 0 || P < 0 || T < 0 || op->check_period < 0)
        return -2;
    oracle_stats total = {0, 0, 0, 0, 0};
    int failed = 0;
#ifdef _OPENMP
    int nth = op->threads > 0 ? op->threads : omp_get_max_threads();
#pragma omp parallel num_threads(nth)
#endif
    {
        const int n = pb->n;
        double *buf = (double *)malloc(sizeof(double) * ((size_t)4 * n + (size_t)pb->m + (size_t)(pb->d > 0 ? pb->d : 1)));
        oracle_stats st = {0, 0, 0, 0, 0};
        if (!buf) {
#ifdef _OPENMP
#pragma omp atomic write
#endif
            failed = 1;
        } else {
            double *u = buf, *prev = u + n, *c = prev + n, *x = c + n, *r = x + n, *tmp = r + pb->m;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
            for (int32_t p = 0; p < P; ++p)
                run_chain(pb, op, seed, chain_offset + (uint64_t)p, T, out + p, P, u, prev, c, x, r, tmp, &st);
            free(buf);
        }
#ifdef _OPENMP
#pragma omp critical
#endif
        {
            total.accepted += st.accepted; total.rejected += st.rejected; total.checks += st.checks;
            total.reprojections += st.reprojections; total.stuck_chains += st.stuck_chains;
        }
    }
    if (stats_out) *stats_out = total;
    return failed ? -1 : 0;
}

/* Centre of the warmup points, c = (1/W) * Wmat * 1 (ACHRCuda.cu:414-434). */
void oracle_centre(int32_t n, int32_t W, const double *warmup, double *centre)
{
    const double alpha = 1.0 / (double)W;
    for (int i = 0; i < n; ++i) {
        double acc = 0.0;
        for (int j = 0; j < W; ++j) acc += warmup[(size_t)j * (size_t)n + i];
        centre[i] = alpha * acc;
    }
}

/* Byte-level "%f" formatting of one File<ii> (ACHRCuda.cu:744-756) is checked
 * in the tests with Python's own printf-style formatting; nothing here. */
int oracle_version(void) { return 1; }
