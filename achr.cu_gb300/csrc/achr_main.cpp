// ACHRCuda: drop-in replacement for the reference program's command line.
//
//   ACHRCuda model.mps warmuppoints.csv nFiles nPoints nSteps [options]
//
// Same positional arguments, same File0..File{nFiles-1} outputs (n lines of
// nPoints "%f" values separated by commas) and the same progress lines on
// stdout as ACHRcu/ACHRCuda.cu:504-802.  Optional trailing flags:
//   --seed S            64-bit seed of the Philox stream (default: time-based, printed)
//   --mode reference|feasible
//   --null sts|svd|fixed  null-space construction (default sts, the reference's rule; fixed also
//                       holds the reactions with lb == ub)
//   --centre cuda|matlab  centre weights (ACHRCuda.cu:347-348 or ACHRSamplerMOD.m:174)
//   --threads-per-chain N
//   --check-period N    residual check every N steps (default 10, ACHRCuda.cu:325; 0 = never)
//   --reproject auto|nnt|residual|deferred  reprojection as N (N^T x) or through the residual in
//                             the chain kernel, or deferred to a batched tensor-core pass
//   --reprojection-passes N   passes of the deferred reprojection (default 2)
//                       (default: chosen by model size)
//   --bracket-pass merged|separate  ratio-test brackets in the direction pass (default) or in a
//                       pass of their own; the points are the same
//   --writer-threads N  host threads formatting File<ii>
//   --report path.json  write sampling statistics
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <thread>
#include <vector>

#include "../../include/achr.h"

namespace {

double now_s() {
    return std::chrono::duration<double>(std::chrono::system_clock::now().time_since_epoch()).count();
}

int die(const char *what) {
    std::fprintf(stderr, "ACHRCuda: %s: %s\n", what, achr_last_error());
    return 2;
}

bool parse_int(const char *s, long long &v) {
    char *e = nullptr;
    v = std::strtoll(s, &e, 10);
    return e && *e == '\0' && e != s;
}

}  // namespace

int main(int argc, char **argv) {
    const double t0 = now_s();
    if (argc < 6) {
        std::fprintf(stderr,
                     "usage: %s model.mps warmuppoints.csv nFiles nPoints nSteps [--seed S] [--mode reference|feasible]"
                     " [--null sts|svd|fixed] [--centre cuda|matlab] [--threads-per-chain N] [--check-period N]"
                     " [--reproject auto|nnt|residual|deferred] [--reprojection-passes N] [--bracket-pass merged|separate]"
                     " [--writer-threads N]"
                     " [--report file.json]\n",
                     argv[0]);
        return 2;
    }
    achr_options opt;
    achr_default_options(&opt);
    unsigned long long seed = (unsigned long long)std::time(nullptr) * 2654435761ull ^ (unsigned long long)clock();
    int writer_threads = 0;
    const char *report = nullptr;
    for (int a = 6; a < argc; ++a) {
        std::string f = argv[a];
        auto need = [&](void) -> const char * {
            if (a + 1 >= argc) {
                std::fprintf(stderr, "ACHRCuda: %s needs a value\n", f.c_str());
                std::exit(2);
            }
            return argv[++a];
        };
        long long v;
        if (f == "--seed") {
            if (!parse_int(need(), v)) return std::fprintf(stderr, "ACHRCuda: bad --seed\n"), 2;
            seed = (unsigned long long)v;
        } else if (f == "--mode") {
            std::string m = need();
            if (m == "reference") opt.mode = ACHR_MODE_REFERENCE;
            else if (m == "feasible") opt.mode = ACHR_MODE_FEASIBLE;
            else return std::fprintf(stderr, "ACHRCuda: bad --mode\n"), 2;
        } else if (f == "--null") {
            std::string m = need();
            if (m == "sts") opt.null_space = ACHR_NULL_SVD_STS;
            else if (m == "svd") opt.null_space = ACHR_NULL_SVD_S;
            else if (m == "fixed") opt.null_space = ACHR_NULL_FIXED;
            else return std::fprintf(stderr, "ACHRCuda: bad --null\n"), 2;
        } else if (f == "--centre") {
            std::string m = need();
            if (m == "cuda") opt.centre_offset = 0;
            else if (m == "matlab") opt.centre_offset = 1;
            else return std::fprintf(stderr, "ACHRCuda: bad --centre\n"), 2;
        } else if (f == "--threads-per-chain") {
            if (!parse_int(need(), v)) return std::fprintf(stderr, "ACHRCuda: bad --threads-per-chain\n"), 2;
            opt.threads_per_chain = (int32_t)v;
        } else if (f == "--check-period") {
            if (!parse_int(need(), v) || v < 0) return std::fprintf(stderr, "ACHRCuda: bad --check-period\n"), 2;
            opt.check_period = (int32_t)v;
        } else if (f == "--reproject") {
            std::string m = need();
            if (m == "nnt") opt.reproject_form = 1;
            else if (m == "residual") opt.reproject_form = 2;
            else if (m == "deferred") opt.reproject_form = 3;
            else if (m == "auto") opt.reproject_form = 0;
            else return std::fprintf(stderr, "ACHRCuda: bad --reproject\n"), 2;
        } else if (f == "--reprojection-passes") {
            if (!parse_int(need(), v) || v < 1 || v > 8)
                return std::fprintf(stderr, "ACHRCuda: bad --reprojection-passes\n"), 2;
            opt.reprojection_passes = (int32_t)v;
        } else if (f == "--bracket-pass") {
            std::string m = need();
            if (m == "merged") opt.bracket_pass = 0;
            else if (m == "separate") opt.bracket_pass = 1;
            else return std::fprintf(stderr, "ACHRCuda: bad --bracket-pass\n"), 2;
        } else if (f == "--writer-threads") {
            if (!parse_int(need(), v)) return std::fprintf(stderr, "ACHRCuda: bad --writer-threads\n"), 2;
            writer_threads = (int)v;
        } else if (f == "--report") {
            report = need();
        } else {
            std::fprintf(stderr, "ACHRCuda: unknown option %s\n", f.c_str());
            return 2;
        }
    }

    // Device report (ACHRCuda.cu:540-549).
    int ndev = 0;
    cudaGetDeviceCount(&ndev);
    for (int i = 0; i < ndev; ++i) {
        cudaDeviceProp prop;
        cudaGetDeviceProperties(&prop, i);
        int mem_khz = 0, bus = 0;
        cudaDeviceGetAttribute(&mem_khz, cudaDevAttrMemoryClockRate, i);
        cudaDeviceGetAttribute(&bus, cudaDevAttrGlobalMemoryBusWidth, i);
        std::printf("Device Number: %d\n", i);
        std::printf("Device name: %s\n", prop.name);
        std::printf("Memory clock rate (Khz): %d\n", mem_khz);
        std::printf("Memory Bus Width (bits): %d\n", bus);
        std::printf("Peak Memory Bandwidth (GB/s): %f\n\n", 2.0 * mem_khz * (bus / 8) / 1.0e6);
    }

    long long nFiles, nPoints, nSteps;
    if (!parse_int(argv[3], nFiles) || !parse_int(argv[4], nPoints) || !parse_int(argv[5], nSteps) || nFiles < 0 ||
        nPoints < 0 || nSteps < 0 || nPoints > 2147483647LL || nSteps > 2147483647LL) {
        std::fprintf(stderr, "ACHRCuda: nFiles, nPoints and nSteps must be non-negative integers\n");
        return 2;
    }
    std::printf("Total count is %lld \n", nFiles * nPoints * nSteps);
    std::printf("Seed is %llu \n", seed);

    std::printf("\nThe model supplied is %s\n", argv[1]);
    achr_model_buf mb;
    if (achr_read_mps(argv[1], &mb) != ACHR_OK) {
        std::printf("Error reading MPS file %s\n", argv[1]);
        std::fprintf(stderr, "%s\n", achr_last_error());
        return 1;  // reference exit code for an unreadable model (ACHRCuda.cu:563-566)
    }
    const int n = mb.model.n_rxns;
    std::printf("nRxns egale a %d  \n", n);
    std::printf("nMets egale a %d  \n", mb.model.n_mets);
    std::printf("nnz is %lld \n", (long long)mb.model.nnz);

    double *warm = nullptr;
    int32_t W = 0;
    if (achr_read_warmup_csv(argv[2], n, &warm, &W) != ACHR_OK) {
        achr_free_model(&mb);
        return die("reading warmup points");
    }
    std::printf("nWrmup egale a %d \n", W);

    achr_ctx *ctx = nullptr;
    if (achr_create(&mb.model, warm, W, &opt, &ctx) != ACHR_OK) {
        achr_free(warm);
        achr_free_model(&mb);
        return die("set-up");
    }
    int32_t d = 0;
    achr_get_null_space_dim(ctx, &d);
    std::printf("Null space dimension is %d \n", d);
    std::printf("Null space done in %.5f seconds.\n", now_s() - t0);

    // Two host buffers: File<ii> is formatted and written by a writer thread
    // while the GPU samples file ii + 1 (the reference samples and writes in
    // turn, ACHRCuda.cu:736-756).
    std::vector<double> pts[2];
    pts[0].resize((size_t)n * (size_t)nPoints);
    if (nFiles > 1) pts[1].resize((size_t)n * (size_t)nPoints);
    std::thread writer;
    bool write_ok = true;
    std::string write_err;
    auto join_writer = [&]() -> bool {
        if (writer.joinable()) writer.join();
        return write_ok;
    };
    auto fail_run = [&](const char *what) -> int {
        join_writer();
        achr_destroy(ctx);
        achr_free(warm);
        achr_free_model(&mb);
        if (!write_ok) {
            std::fprintf(stderr, "ACHRCuda: writing points: %s\n", write_err.c_str());
            return 2;
        }
        return die(what);
    };
    achr_stats total{};
    for (long long ii = 0; ii < nFiles; ++ii) {
        std::printf("File %lld\n", ii);
        std::fflush(stdout);
        achr_stats st{};
        std::vector<double> &buf = pts[ii & 1];
        if (achr_sample(ctx, seed, (uint64_t)ii * (uint64_t)nPoints, (int32_t)nPoints, (int32_t)nSteps, buf.data(),
                        &st) != ACHR_OK)
            return fail_run("sampling");
        total.accepted += st.accepted;
        total.rejected += st.rejected;
        total.checks += st.checks;
        total.reprojections += st.reprojections;
        total.stuck_chains += st.stuck_chains;
        total.exact_evals += st.exact_evals;
        total.final_projections += st.final_projections;
        if (st.max_residual > total.max_residual) total.max_residual = st.max_residual;
        if (st.max_bound_violation > total.max_bound_violation) total.max_bound_violation = st.max_bound_violation;
        total.kernel_ms += st.kernel_ms;
        if (!join_writer()) return fail_run("writing points");
        writer = std::thread([&, ii, bufp = buf.data()]() {
            char name[64];
            std::snprintf(name, sizeof name, "File%lld", ii);
            if (achr_write_points_csv(name, bufp, n, (int32_t)nPoints, writer_threads) != ACHR_OK) {
                write_ok = false;
                write_err = achr_last_error();  // the message is per thread
            }
        });
    }
    if (!join_writer()) return fail_run("writing points");
    const double elapsed = now_s() - t0;
    std::printf("Sampling done in %.5f seconds.\n", elapsed);
    if (total.stuck_chains)
        std::printf("Warning: %lld chains stopped after %d rejected attempts in a row\n", (long long)total.stuck_chains,
                    opt.max_attempts);
    if (report) {
        FILE *f = std::fopen(report, "w");
        if (f) {
            std::fprintf(f,
                         "{\"n_rxns\": %d, \"n_mets\": %d, \"n_warmup\": %d, \"null_dim\": %d, \"files\": %lld, "
                         "\"points\": %lld, \"steps\": %lld, \"seed\": %llu, \"accepted\": %lld, \"rejected\": %lld, "
                         "\"checks\": %lld, \"reprojections\": %lld, \"stuck_chains\": %lld, \"exact_evals\": %lld, "
                         "\"final_projections\": %lld, \"max_residual\": %.6e, \"max_bound_violation\": %.6e, "
                         "\"kernel_ms\": %.3f, \"wall_s\": %.5f, \"chain_steps_per_s_kernel\": %.6e}\n",
                         n, mb.model.n_mets, W, d, nFiles, nPoints, nSteps, seed, (long long)total.accepted,
                         (long long)total.rejected, (long long)total.checks, (long long)total.reprojections,
                         (long long)total.stuck_chains, (long long)total.exact_evals,
                         (long long)total.final_projections, total.max_residual, total.max_bound_violation,
                         total.kernel_ms, elapsed,
                         total.kernel_ms > 0 ? (double)total.accepted / (total.kernel_ms * 1e-3) : 0.0);
            std::fclose(f);
        }
    }
    achr_destroy(ctx);
    achr_free(warm);
    achr_free_model(&mb);
    return 0;
}
