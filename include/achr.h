/*
 * achr.h -- C ABI of the GB300 ACHR sampler (Artificial-Centering Hit-and-Run
 * over the flux polytope {v : S v = 0, lb <= v <= ub}).
 *
 * Plain pointers and sizes only; every call returns an achr_status and never
 * throws or exits.  achr_last_error() gives a message for the calling thread.
 * One context owns device copies of one model and its warmup points on one GPU.
 * A context is used by one host thread at a time (its counters and scratch
 * buffers are shared by its calls); distinct contexts may be used concurrently.
 *
 * Each entry point names the part of the reference program it replaces
 * (ACHRcu/ACHRCuda.cu in marouenbg/ACHR.cu).  The reference exposes a CLI,
 * not a library; the CLI built from this library (ACHRCuda) keeps its
 * arguments and output files.
 */
#ifndef ACHR_GB300_H
#define ACHR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    ACHR_OK = 0,
    ACHR_ERR_INVALID = 1,     /* bad argument or malformed input */
    ACHR_ERR_CUDA = 2,        /* CUDA runtime / library failure */
    ACHR_ERR_NOMEM = 3,       /* host or device allocation failed */
    ACHR_ERR_IO = 4,          /* file could not be opened, read or written */
    ACHR_ERR_PARSE = 5,       /* MPS or CSV content does not parse */
    ACHR_ERR_NUMERIC = 6,     /* null space / solver failure */
    ACHR_ERR_TIMEOUT = 7,     /* a bounded device-side wait ran out */
    ACHR_ERR_UNSUPPORTED = 8  /* size or option outside what this build handles */
} achr_status;

/* Stoichiometric model: S as COO triplets (any order, duplicates summed),
 * bounds per reaction.  Mirrors what the reference keeps from the MPS file:
 * S, lb and ub only (ACHRCuda.cu:567-597, COO build :642-663). */
typedef struct {
    int32_t n_rxns;           /* n: columns of S */
    int32_t n_mets;           /* m: rows of S */
    int64_t nnz;
    const int32_t *row;       /* nnz metabolite indices in [0, m) */
    const int32_t *col;       /* nnz reaction indices in [0, n) */
    const double *val;        /* nnz coefficients */
    const double *lb;         /* n lower bounds (may be -inf) */
    const double *ub;         /* n upper bounds (may be +inf) */
} achr_model;

/* Reprojection / warmup handling. */
enum {
    /* Reference semantics: warmups used as given; every check_period-th step
     * x <- N (N^T x) in FP64 when max|S x| > residual_tol (ACHRCuda.cu:325-343). */
    ACHR_MODE_REFERENCE = 0,
    /* Same loop, but warmup points and centre are first projected onto null(S)
     * in FP64 (warmup CSVs are %f-rounded, so S w != 0 at ~1e-6), and every
     * emitted point is projected, clipped and verified against feasibility_tol. */
    ACHR_MODE_FEASIBLE = 1
};

/* Null-space basis construction. */
enum {
    ACHR_NULL_SVD_STS = 0,    /* SVD of S^T S, cutoff n*sigma0*2.2204e-16 (ACHRCuda.cu:436-502) */
    ACHR_NULL_SVD_S = 1,      /* SVD of S itself (better conditioned), same cutoff rule on sigma(S) */
    ACHR_NULL_FIXED = 2       /* as SVD_STS on S with a unit row appended for every reaction with lb == ub:
                                 the basis spans {v : S v = 0, v_i = 0 where lb_i = ub_i}, so a
                                 reprojection never moves a fixed (blocked) reaction off its value.
                                 Not the reference's basis; reprojections then stay in the chain kernel. */
};

typedef struct {
    int32_t mode;             /* ACHR_MODE_* (default REFERENCE) */
    int32_t null_space;       /* ACHR_NULL_* (default SVD_STS) */
    int32_t check_period;     /* residual check every k-th step (default 10, ACHRCuda.cu:325); 0 = never
                                 (for runs that reproject in batches, achr_sample_periodic) */
    int32_t max_attempts;     /* rejected redraws of one step before a chain stops (default 100000) */
    int32_t centre_offset;    /* 0: centre weights of ACHRCuda.cu:347-348; 1: ACHRSamplerMOD.m:174 */
    int32_t exact_ratio;      /* 1: evaluate every ratio-test candidate in FP64 (diagnostic, slower) */
    int32_t threads_per_chain;/* 0: chosen by size; else 32, 64, 128, 256, 320, 384 or 512 threads per chain
                                 (320 and 384 hold up to 3840 reactions) */
    int32_t reproject_form;   /* per-chain reprojection x <- N (N^T x) (ACHRCuda.cu:208-230) computed as
                                 0: chosen by the inputs: deferred (3) when the warmup points carry a
                                    residual max|S w| > residual_tol / 8 (a %f-rounded CSV: nearly every
                                    check then reprojects), n_rxns x null_dim >= 2.5e5 and form 3's
                                    conditions hold; otherwise in the chain kernel, as 2 when
                                    n_rxns x null_dim >= 4e6, else as 1,
                                 1: N (N^T x) in FP64 in the chain kernel,
                                 2: x - S^T (S S^T)^+ S x in the chain kernel, the pseudo-inverse product
                                    in FP32 on the residual (equal in exact arithmetic; m^2 FP32 instead
                                    of 4 n d FP64 operations); needs n_mets <= 8192,
                                 3: deferred: every chain's launch stops after a check step's update,
                                    and the chains whose residual exceeds residual_tol are reprojected
                                    together, x <- x - S^T (S S^T)^+ S x with S x and the update in FP64
                                    and the dense product on the tensor cores (three BF16 split
                                    products); the first pass's update S^T z and new residual are
                                    exact to double-float (~48 bits), later ones (FP32, on what is left)
                                    run per chain until max|S x| <= residual_tol / 1000; then the clip
                                    and the centre update of
                                    that step, as the reference orders them; needs n_mets <= the chain
                                    kernel's padded length and a condition number of S S^T <= 2e4
                                    (achr_sample,
                                    achr_sample_device and achr_sample_resume; batched launches
                                    reproject in the chain kernel, and so does choice 0 with a
                                    hit-and-run pool) */
    double residual_tol;      /* 1e-9 (ACHRCuda.cu:338) */
    double max_min_tol;       /* 1e-9 (ACHRCuda.cu:505) */
    double u_tol;             /* 1e-9 (ACHRCuda.cu:508) */
    double d_tol;             /* 1e-14 (ACHRCuda.cu:512) */
    double feasibility_tol;   /* 1e-8: ||S v||_inf bound for emitted points in FEASIBLE mode */
    int32_t wait_limit_ns;    /* bound on the chain kernel's wait for a staged warmup column; on expiry
                                 the launch stops, drains its copy and returns ACHR_ERR_TIMEOUT
                                 (0: the default of 2 s).  A negative value -L is a test of that
                                 path: the wait is on a barrier nothing completes and runs out after
                                 L ns every time. */
    int32_t bracket_pass;     /* FP32 ratio-test brackets (ACHRCuda.cu:266-281): 0: formed in the same pass
                                 as the direction, before its norm is known, with the candidacy threshold
                                 bounded through the box (or the longest hit-and-run direction); a step
                                 whose threshold exceeds the bound, or a model with an infinite bound,
                                 uses a separate pass.  1: always a separate pass.  Results are equal. */
    int32_t reprojection_passes; /* most passes of one deferred reprojection, 1..8 (0: 8); a chain still
                                    above residual_tol after the last pass is an ACHR_ERR_NUMERIC */
} achr_options;

typedef struct {
    int64_t accepted;         /* accepted steps over all chains */
    int64_t rejected;         /* rejected attempts (reference ACHRCuda.cu:316-319) */
    int64_t checks;           /* residual checks performed */
    int64_t reprojections;    /* reprojections triggered (max|Sx| > residual_tol) */
    int64_t stuck_chains;     /* chains that stopped after max_attempts rejections */
    int64_t exact_evals;      /* ratio-test candidates evaluated in FP64 */
    int64_t final_projections;/* emitted points that needed the FEASIBLE-mode projection */
    double max_residual;      /* max ||S v||_inf over emitted points (FEASIBLE mode) */
    double max_bound_violation; /* max over emitted points of max(lb - v, v - ub, 0) */
    double kernel_ms;         /* device time of the sampling launch(es) */
    int64_t segments;         /* chain-kernel launches of deferred-reprojection sampling (reproject_form 3,
                                 or 0 choosing it); 0 when reprojections ran inside the chain kernel */
    int64_t reprojection_passes; /* deferred: passes summed over the reprojected chains */
    int64_t reprojection_gemms;  /* deferred: tensor-core GEMMs that ran (each over all chains of a sweep) */
    double chain_ms;          /* device time of the chain-kernel launches alone (= kernel_ms when the
                                 reprojections ran inside the chain kernel) */
    double reprojection_ms;   /* deferred: device time of the batched passes (GEMMs and updates) */
    double reprojection_flops;/* deferred: FLOPs of the GEMMs that ran (three BF16 split products) */
    int64_t kernel_launches;  /* kernels the call launched (chain kernel, and when deferred the GEMMs and
                                 pass kernels, including those a device-side gate then skipped) */
} achr_stats;

typedef struct achr_ctx achr_ctx;

/* Fill *opt with the reference's constants (see field comments). */
void achr_default_options(achr_options *opt);

/* Build a context: upload S (CSR), bounds and the n x W column-major warmup
 * matrix (point j at warmup + j*n), compute the null-space basis N and the
 * warmup centre.  Replaces ACHRCuda.cu:642-729 (COO build and upload,
 * computeKernelCuda :436-502, createCenterPt :414-434, buffer set-up). */
achr_status achr_create(const achr_model *model, const double *warmup, int32_t n_warmup,
                        const achr_options *opt, achr_ctx **out);

/* Replace the context's null-space basis with a caller-supplied one (n x d,
 * column-major, host memory).  The reference computes it internally
 * (ACHRCuda.cu:698-704); this lets a caller pin N across implementations.
 * In ACHR_MODE_FEASIBLE the warmup points are projected onto the new basis
 * and the centre is recomputed. */
achr_status achr_set_null_space(achr_ctx *ctx, const double *N, int32_t d);

/* Null-space dimension d and the basis itself (n x d column-major, host). */
achr_status achr_get_null_space_dim(const achr_ctx *ctx, int32_t *d);
achr_status achr_get_null_space(const achr_ctx *ctx, double *N_out);

/* Centre of the warmup points as used by the sampler (n doubles, host). */
achr_status achr_get_centre(const achr_ctx *ctx, double *centre_out);

/* Run P independent chains of T accepted steps each and copy the final
 * points to host memory, n x P row-major (row = reaction, column = chain),
 * the layout of the reference's points array (ACHRCuda.cu:247, 743).
 * Chains are numbered chain_offset .. chain_offset+P-1 in the random stream
 * keyed by seed; file ii of the CLI uses chain_offset = ii*P.
 * Replaces one iteration of the per-file loop, ACHRCuda.cu:736-743
 * (stepPointProgress launch :741 and the device-to-host copy :743). */
achr_status achr_sample(achr_ctx *ctx, uint64_t seed, uint64_t chain_offset, int32_t n_points,
                        int32_t n_steps, double *points_out, achr_stats *stats);

/* Same as achr_sample, but the output is device memory (n x P row-major,
 * leading dimension ld_out >= P) and the work is queued on `stream`
 * (a cudaStream_t; NULL = legacy default stream).  Returns after the launch
 * is queued; stats (if non-NULL) are filled after synchronising the stream. */
achr_status achr_sample_device(achr_ctx *ctx, uint64_t seed, uint64_t chain_offset, int32_t n_points,
                               int32_t n_steps, double *d_points_out, int64_t ld_out, void *stream,
                               achr_stats *stats);

/* Start (resume = 0) or continue (resume = 1) chains in segments: the
 * checkpoint/resume the reference lacks (its MATLAB counterpart keeps the last
 * point, ACHRSamplerMOD.m:176-183).  d_points and d_centre_acc are device
 * buffers n x P row-major (leading dimension ld): the chains' points and
 * their centre accumulators (W + t + centre_offset) * centre after step t.
 * A fresh start begins at step0 = 0 and writes both; a resumed launch reads
 * both as the state after step0 steps and overwrites them with the state
 * after step0 + n_steps.  Running T1 then T2 steps this way gives the same
 * points as one launch of T1 + T2 steps (the random stream is keyed by the
 * global step index), except in ACHR_MODE_FEASIBLE, where every segment ends
 * with the feasibility projection.  Queued on `stream`; stats synchronise. */
achr_status achr_sample_resume(achr_ctx *ctx, uint64_t seed, uint64_t chain_offset, int32_t n_points, int32_t step0,
                               int32_t n_steps, int32_t resume, double *d_points, double *d_centre_acc, int64_t ld,
                               void *stream, achr_stats *stats);

/* Release every device and host resource of the context. */
void achr_destroy(achr_ctx *ctx);

/* ---- Hit-and-run along a pool of directions (no reference counterpart) ----
 * Replaces ACHR's direction (a random warmup point minus the running centre,
 * ACHRCuda.cu:260-264) by a random column of a fixed pool: each step draws a
 * pool index from the same Philox stream as the warmup index, moves along
 * that column with the reference's ratio test and step draw, clips, and keeps
 * no centre.  The direction distribution is symmetric and independent of the
 * state, so the chain keeps the uniform target.  dirs is n x n_dirs
 * column-major (leading dimension ld >= n), host or device memory; every
 * column should lie in the null space of S.  n_dirs = 0 returns the context
 * to ACHR.  Chains start at the warmup centre in either mode. */
achr_status achr_set_directions(achr_ctx *ctx, const double *dirs, int64_t ld, int32_t n_dirs);

/* The installed pool: its size (0 in ACHR mode) and a copy, n x K
 * column-major (ld = n), to host or device memory. */
int32_t achr_get_n_directions(const achr_ctx *ctx);
achr_status achr_get_directions(const achr_ctx *ctx, double *dirs_out);

/* ---- Learned direction preconditioner (no reference counterpart) ----
 * A low-rank-plus-diagonal linear map L = [diag(exp(s)), U] (d x (d + r)) in
 * the coordinates below, fitted to samples y = B^T (x - mu) of the plain
 * sampler by the Gaussian KL loss 1/2 tr(C^-1 Sigma) + 1/2 log det C with
 * C = L L^T = diag(exp(2 s)) + U U^T (minibatch Sigma, Adam), all on the GPU.
 * Its directions N L z, z ~ N(0, I), drive hit-and-run (achr_set_directions)
 * through a pool of K of them.  s is d floats, U is d x r row-major, Y is
 * d x n_samples row-major (leading dimension ldy), all device memory. */
typedef struct achr_precond_options {
    int32_t iterations;    /* Adam steps (2000) */
    int32_t batch;         /* samples per step (4096) */
    float learning_rate;   /* 0.01 */
    float beta1, beta2;    /* 0.9, 0.999 */
    float eps;             /* 1e-8 */
    uint64_t seed;         /* order in which minibatches are visited */
    int32_t init;          /* 1: start from the probabilistic-PCA fit of the samples (overwrites s, U);
                              0: start from the s, U passed in */
    int32_t standardize;   /* 1: train in coordinates scaled to unit RMS (results returned unscaled) */
    int32_t full_batch;    /* 1 (default): every step's loss and gradients are those of all n_samples
                              samples: the samples are replaced by d columns with the same covariance,
                              V Lambda^1/2 sqrt(d) from its eigen-decomposition, so a step costs a d-sample
                              minibatch and carries no sampling noise; batch and seed are then unused.
                              0: minibatches of `batch` consecutive samples in a seeded order */
} achr_precond_options;

typedef struct achr_precond_stats {
    double loss_first;     /* mean loss over the first 20 steps (the full-sample loss with full_batch) */
    double loss_last;      /* mean loss over the last 20 steps */
    double train_ms;
    int32_t iterations;
} achr_precond_stats;

void achr_precond_default_options(achr_precond_options *opt);

/* The preconditioner's coordinates.  Hit-and-run directions must stay in the
 * polytope's affine hull, not just the null space of S: a reaction that has
 * the same value in every warmup point (blocked, or pinned at a bound by the
 * other constraints) must not move, or almost every random direction leaves
 * the polytope at once.  The basis (n x d, column-major, orthonormal) spans
 * {v : S v = 0, v_i = 0 for those reactions}; d and the number of pinned
 * reactions come from achr_precond_dim, the basis from achr_get_precond_basis
 * (host or device memory).  Built on first use. */
achr_status achr_precond_dim(achr_ctx *ctx, int32_t *d_out, int32_t *n_frozen_out);
achr_status achr_get_precond_basis(achr_ctx *ctx, double *basis_out);

/* Y (d x P, row-major, leading dimension ldy, FP32) = B^T (x - mu), B the
 * preconditioner's basis above, for the chains of an n x P row-major block of
 * points (mu: n doubles or NULL), as a tensor-core GEMM with three BF16 split
 * products.  Synchronises `stream`. */
achr_status achr_null_coords(achr_ctx *ctx, int32_t n_points, const double *d_points, int64_t ld, const double *d_mu,
                             float *d_Y, int64_t ldy, void *stream);

/* Loss and gradients (ds: d floats, dU: d x r) for one minibatch Y (d x B). */
achr_status achr_precond_loss_grad(int32_t d, int32_t r, int32_t B, const float *d_s, const float *d_U,
                                   const float *d_Y, int64_t ldy, float *loss_out, float *d_gs, float *d_gU,
                                   void *stream);

/* opt.iterations Adam steps over minibatches of consecutive columns of Y
 * (centred samples), from the probabilistic-PCA fit of Y (opt.init = 1) or
 * from the s, U passed in; s and U are updated in place.  Synchronises
 * `stream`. */
achr_status achr_precond_train(int32_t d, int32_t r, int32_t n_samples, const float *d_Y, int64_t ldy,
                               const achr_precond_options *opt, float *d_s, float *d_U, void *stream,
                               achr_precond_stats *stats);

/* Pool of n_dirs directions B (exp(s) z1 + U z2), z ~ N(0, I) from Philox
 * keyed by seed, computed in FP64 (the directions lie in the null space of S
 * to rounding), installed with achr_set_directions. */
achr_status achr_precond_pool(achr_ctx *ctx, int32_t r, const float *d_s, const float *d_U, int32_t n_dirs,
                              uint64_t seed);

/* Pilot run of the installed direction pool and the fallback to plain ACHR.
 * `chains` chains start at random warmup points (Philox keyed by seed), run
 * `burnin` steps along the pool, then `draws` draws `gap` steps apart; the
 * split-R-hat of every moving flux (Gelman et al., BDA3 11.4: halves of every
 * chain, sqrt(((n-1)/n W + B/n) / W)) is computed on the GPU.  When its maximum
 * is at or above rhat_limit (1.01 in the usual practice) the pool is removed and
 * the context returns to the reference's direction rule (ACHRCuda.cu:260-264),
 * so a preconditioner that does not mix never replaces plain ACHR.  The chains
 * use ids 0 .. chains-1 of seed. */
typedef struct {
    double rhat_max;          /* largest split-R-hat over the moving fluxes */
    int32_t fluxes;           /* fluxes that moved in the pilot (the others are left out) */
    int32_t kept;             /* 1: the pool stays installed; 0: removed (plain ACHR) */
    double sampling_ms;       /* device time of the pilot's sampling launches */
} achr_direction_check;

achr_status achr_check_directions(achr_ctx *ctx, int32_t chains, int32_t burnin, int32_t draws, int32_t gap,
                                  uint64_t seed, double rhat_limit, achr_direction_check *out);

/* ---- Batched reprojection on the tensor cores and periodic-reprojection
 * sampling.  The reference reprojects one chain at a time when its residual
 * check fires (reprojectPoint(2), ACHRCuda.cu:208-230, :338-343); these
 * reproject every chain of a block at once. ---- */

typedef struct achr_reproj_stats {
    double residual_before;  /* max |S x|_inf over the chains before the first round */
    double residual_after;   /* after the last round (measured only when stats are requested) */
    double gemm_ms;          /* tensor-core GEMM time, summed over chunks and rounds */
    double total_ms;         /* the whole reprojection on the stream */
    double gemm_flops;       /* FLOPs of the three BF16 split products */
    int32_t rounds;          /* passes in which some block of chains was corrected */
    int32_t rank;            /* rank of S kept by the pseudo-inverse */
    double lambda_min;       /* smallest kept and largest eigenvalue of S S^T */
    double lambda_max;
} achr_reproj_stats;

/* x <- clip(x - S^T (S S^T)^+ S x, lb, ub) for chains 0..P-1 of an n x P
 * row-major device block (leading dimension ld); the centre accumulators (if
 * d_centre_acc is non-NULL, same layout) move with the points.  Up to
 * max_rounds (1..16) passes; a block of chains whose max |S x| is already
 * within opt.residual_tol is left as it is.  Equals the reference's N (N^T x) followed by its clip; the
 * residual S x and the update are FP64, the dense (S S^T)^+ product runs on
 * the tensor cores as three BF16 split products with FP32 accumulation.  The
 * operator is built on the first call (FP64 eigen-decomposition of S S^T).
 * Synchronises `stream`. */
achr_status achr_reproject_batch(achr_ctx *ctx, int32_t n_points, double *d_points, double *d_centre_acc,
                                 int64_t ld, int32_t max_rounds, void *stream, achr_reproj_stats *stats);

/* T steps of P chains in segments of `period` steps with achr_sample_resume,
 * each segment followed by achr_reproject_batch over all chains (max_rounds).
 * d_points and d_centre_acc as for achr_sample_resume; they hold the final
 * points (feasible to the reprojection's accuracy) and accumulators.  With
 * opt.check_period = 0 the chain kernel performs no per-chain checks. */
achr_status achr_sample_periodic(achr_ctx *ctx, uint64_t seed, uint64_t chain_offset, int32_t n_points,
                                 int32_t n_steps, int32_t period, int32_t max_rounds, double *d_points,
                                 double *d_centre_acc, int64_t ld, void *stream, achr_stats *stats,
                                 achr_reproj_stats *rstats);

/* The tensor-core GEMM on its own: C (M x N, FP32, row-major, ldc) = A0 B0^T
 * (nsplit 1) or A0 B0^T + A0 B1^T + A1 B0^T (nsplit 3, hi/lo split products).
 * A_s are M x K and B_s are N x K BF16 device matrices, row-major with K
 * contiguous (leading dimensions lda, ldb in elements, multiples of 8; base
 * addresses 16-byte aligned); K is a multiple of 64.  No reference
 * counterpart.  Synchronises `stream`. */
achr_status achr_gemm_bf16(int32_t M, int32_t N, int32_t K, int32_t nsplit, const void *A0, const void *A1,
                           int64_t lda, const void *B0, const void *B1, int64_t ldb, float *C, int64_t ldc,
                           void *stream);

/* ---- Tuning and batched sampling (no counterpart in the reference, which
 * hard-codes 8-thread blocks, ACHRCuda.cu:715, and runs one model per process) ---- */

/* Time the chain kernel's candidate configurations (threads per chain x
 * reactions per thread) on a short run of this context and keep the fastest in
 * its options; the choice is cached per padded model size and device for the
 * rest of the process.  Writes the chosen threads per chain if non-NULL. */
achr_status achr_autotune(achr_ctx *ctx, int32_t *threads_per_chain_out);

typedef struct {
    double graph_ms;            /* device time of the whole batched launch */
    double load_imbalance;      /* per work queue, (max - mean) / max of its CTAs' exit times (the
                                   share of its CTA slots left idle at its end), averaged over the
                                   queues weighted by their predicted work */
    int64_t accepted, rejected, reprojections, stuck_chains;
    double max_residual, max_bound_violation;
} achr_batch_stats;

/* Sample several models at once in one CUDA-graph launch.  Models are grouped
 * by chain-kernel configuration (threads per chain x reactions per thread,
 * from the context's options, e.g. as achr_autotune chose them); each group is
 * one persistent kernel, one CTA per resident slot of the GPU, whose CTAs take
 * (model, first chain, end chain) items from a device work queue until it is
 * empty.  Items run in order of predicted chain time (the throughput
 * achr_autotune measured for the model, else steps x padded reactions),
 * longest model first, and each item holds about a quarter of the work still
 * queued behind it over the CTAs, so the tiles shrink to single chains at the
 * end of the queue.  Groups run on their own streams, largest total work
 * first.  Model k runs n_points[k] chains of n_steps into d_points_out[k]
 * (device, n_k x P_k, leading dimension ld_out[k]); its chain ids start at the
 * sum of the earlier models' n_points, so achr_sample_device on model k alone
 * with that chain_offset gives the same points.  Synchronises `stream`;
 * per-model finish times (ms from the launch) go to model_ms_out[k] if
 * non-NULL. */
achr_status achr_sample_batch(achr_ctx *const *ctxs, int32_t n_models, const int32_t *n_points, int32_t n_steps,
                              uint64_t seed, double *const *d_points_out, const int64_t *ld_out, void *stream,
                              achr_batch_stats *stats, double *model_ms_out);

/* Tile size of the batched work queues: each item holds the work still queued
 * behind it divided by tiles x the queue's CTAs (default 4; 1..1024).  The
 * setting is process-wide. */
achr_status achr_set_batch_tiles(int32_t tiles);
int32_t achr_get_batch_tiles(void);

/* Time achr_sample_batch for n_steps (a short probe, into the caller's output
 * buffers, which it overwrites) with tiles = 1, 2, 4, 8 and 16, keep the
 * fastest as the process-wide setting and write it to tiles_out if non-NULL. */
achr_status achr_autotune_batch(achr_ctx *const *ctxs, int32_t n_models, const int32_t *n_points, int32_t n_steps,
                                uint64_t seed, double *const *d_points_out, const int64_t *ld_out, void *stream,
                                int32_t *tiles_out);

/* ---- Sampling without any allocation ---- */

/* Largest model (reactions) achr_sample_noalloc accepts: its working data sits
 * in a fixed array of about 40 bytes per reaction plus 1.3 KB (322 KB) that
 * every GPU loading the library keeps until the process exits. */
#define ACHR_NOALLOC_MAX_RXNS 8192

/* A model already resident in device memory (all pointers are device pointers). */
typedef struct {
    int32_t n_rxns;           /* n, at most ACHR_NOALLOC_MAX_RXNS */
    int32_t n_mets;           /* m */
    int32_t n_warmup;         /* W */
    int32_t null_dim;         /* d, columns of N */
    int64_t ld_warmup;        /* leading dimension of warmup in doubles: even and >= n_rxns */
    const double *warmup;     /* ld_warmup x W, column j = warmup point j; 16-byte aligned */
    const double *lb, *ub;    /* n bounds */
    const int32_t *row_ptr;   /* CSR of S: m + 1 offsets, row_ptr[0] = 0, row_ptr[m] = nnz */
    const int32_t *col_idx;   /* nnz column indices in [0, n) */
    const double *val;        /* nnz coefficients */
    const double *N;          /* n x d column-major null-space basis */
    int64_t nnz;              /* entries of col_idx and val */
} achr_device_model;

/* No counterpart in the reference (which allocates all its buffers itself).
 * The points of achr_sample_device (same seed, chains and options), for
 * callers that may not allocate GPU memory (code inside another framework's
 * memory pool or a pre-sized arena, or a repeated path that must not add
 * allocations): inputs and the n x P output (leading dimension ld_out) are the
 * caller's device buffers, and the library calls no cudaMalloc, cudaFree or
 * allocating library routine.  Its working data lives in one fixed device
 * array shared by all calls; the first call on each device looks up that
 * array's address (make it before any stream capture); calls whose GPU work
 * overlaps race on it and must be serialised.  Models above
 * ACHR_NOALLOC_MAX_RXNS reactions are rejected with ACHR_ERR_UNSUPPORTED.
 * The model is checked on the device before sampling (CSR offsets and column
 * indices, finite coefficients and warmup values, lb <= ub); a bad model gives
 * ACHR_ERR_INVALID.  What differs from a context: the null space is the
 * caller's (as with achr_set_null_space); the residual check reads the
 * caller's CSR rather than a sliced-ELL copy (same sums); reprojection is
 * N (N^T x) in FP64 (reproject_form 2 or 3 gives ACHR_ERR_UNSUPPORTED); in
 * ACHR_MODE_FEASIBLE only the final projection of emitted points is applied
 * (the warmup points are used as given).  Synchronises the stream and reports
 * an expired column wait as ACHR_ERR_TIMEOUT; stats->kernel_ms is 0. */
achr_status achr_sample_noalloc(const achr_device_model *model, const achr_options *opt, uint64_t seed,
                                uint64_t chain_offset, int32_t n_points, int32_t n_steps, double *d_points_out,
                                int64_t ld_out, void *stream, achr_stats *stats);

/* ---- Host input/output used by the ACHRCuda CLI (ACHRCuda.cu:558-689, 744-756) ---- */

/* Parsed model owned by the library (free with achr_free_model). */
typedef struct {
    achr_model model;         /* pointers into the arrays below */
    int32_t *row_buf, *col_buf;
    double *val_buf, *lb_buf, *ub_buf;
} achr_model_buf;

/* Read a fixed-format MPS file and keep S, lb, ub, as the reference does with
 * glp_read_mps(GLP_MPS_DECK) (ACHRCuda.cu:560-597).  The first N row is the
 * objective and is dropped; RHS and RANGES are ignored. */
achr_status achr_read_mps(const char *path, achr_model_buf *out);
void achr_free_model(achr_model_buf *m);

/* Read a warmup CSV (n lines of W comma-separated values, ACHRCuda.cu:387-412,
 * 675-689) into a malloc'd n x W column-major matrix (free with achr_free).
 * No line-length limit; rows or columns that disagree are an error. */
achr_status achr_read_warmup_csv(const char *path, int32_t n_rxns, double **warmup_out, int32_t *n_warmup_out);

/* Write an n x P row-major matrix as the reference's File<ii> does:
 * one line per reaction, "%f" values separated by ',' (ACHRCuda.cu:744-756).
 * Byte-identical to fprintf("%f") output; formats with `threads` host threads. */
achr_status achr_write_points_csv(const char *path, const double *points, int32_t n_rxns,
                                  int32_t n_points, int32_t threads);

/* Format one value exactly as printf("%f") into buf (>= 320 bytes); returns length.
 * Exposed for testing the writer against the C library. */
int32_t achr_format_f(double v, char *buf);

void achr_free(void *p);

/* Message describing the last failure on the calling thread ("" if none). */
const char *achr_last_error(void);

/* Library version (major*10000 + minor*100 + patch). */
int32_t achr_version(void);

#ifdef __cplusplus
}
#endif

#endif /* ACHR_GB300_H */
