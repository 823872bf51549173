// lmm_bench: the benchmark driver of the reference's LiborMarketModel sample,
// rebuilt on the library's reference-signature entry points.
//
// It replaces three reference pieces:
//   main.cpp         (LiborMarketModel/main.cpp:40-110): numPaths from argv[1],
//                    z[NMAT*numPaths], one timed liborSwaptionGreeks call,
//                    then "Result: value=..., lambda=...", "Total time: X ms"
//                    and "Paths/sec: ... KPaths/sec";
//   runbatch.sh      (MPTest/runbatch.sh): PR copies of the program run at
//                    once, one per core, each writing its own results file;
//   getresults.sh    (MPTest/getresults.sh): the mean of the PR "Total time"
//                    values.
// Throughput follows LiborMarketModel/README.txt:113-114 (paths x loops x
// processes / total time), with every simulated path counted once: the
// reference's call repeats its Monte Carlo NLOOPS = 10 times
// (liborSwaptionGreeks.cpp:27) but main.cpp divides by numPaths alone.
//
// Usage: lmm_bench [numPaths] [--loops N] [--processes PR] [--f32]
//                  [--rng philox|mrg32k3a] [--quiet]
// Processes are forked before any CUDA call; each one times --loops calls
// of lmm_swaption_greeks[_mrg32k3a][_f32] (after one untimed warm-up call)
// and reports to the parent through a pipe.
#include <sys/types.h>
#include <sys/wait.h>
#include <unistd.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "lmm_gb300.h"

namespace {

struct Options {
    int paths = 65536;
    int loops = 1;
    int processes = 1;
    bool f32 = false;
    bool mrg = false;
    bool quiet = false;
};

void usage(const char *argv0)
{
    std::printf(
        "usage: %s [numPaths] [--loops N] [--processes PR] [--f32] [--rng philox|mrg32k3a] [--quiet]\n"
        "  numPaths     Monte Carlo paths per call (default 65536)\n"
        "  --loops N    timed calls per process after one warm-up call (default 1)\n"
        "  --processes  PR processes running at once, each on the same GPU (default 1)\n"
        "  --f32        the FP32 build of the reference call (default FP64)\n"
        "  --rng        normal stream written into z: the library's Philox stream (default)\n"
        "               or the MRG32k3a/AS241 stream (the reference's generator family)\n",
        argv0);
}

bool parse(int argc, char **argv, Options *o)
{
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        auto need = [&](const char *what) -> const char * {
            if (i + 1 >= argc) {
                std::fprintf(stderr, "%s needs a value\n", what);
                return nullptr;
            }
            return argv[++i];
        };
        if (a == "-h" || a == "--help") {
            usage(argv[0]);
            std::exit(0);
        } else if (a == "--loops") {
            const char *v = need("--loops");
            if (!v) return false;
            o->loops = std::atoi(v);
        } else if (a == "--processes") {
            const char *v = need("--processes");
            if (!v) return false;
            o->processes = std::atoi(v);
        } else if (a == "--f32") {
            o->f32 = true;
        } else if (a == "--rng") {
            const char *v = need("--rng");
            if (!v) return false;
            if (std::strcmp(v, "mrg32k3a") == 0) o->mrg = true;
            else if (std::strcmp(v, "philox") == 0) o->mrg = false;
            else {
                std::fprintf(stderr, "unknown --rng %s\n", v);
                return false;
            }
        } else if (a == "--quiet") {
            o->quiet = true;
        } else if (!a.empty() && a[0] != '-') {
            o->paths = std::atoi(a.c_str());
        } else {
            std::fprintf(stderr, "unknown option %s\n", a.c_str());
            return false;
        }
    }
    if (o->paths < 1 || o->loops < 1 || o->processes < 1 || o->processes > 256 ||
        (long long)o->paths * 40 > 0x7fffffffLL) {
        std::fprintf(stderr, "need 1 <= numPaths <= %d, loops >= 1, 1 <= processes <= 256\n",
                     0x7fffffff / 40);
        return false;
    }
    return true;
}

struct Result {
    int status;
    double value, lambda, mean_ms;
};

// One process: a warm-up call, then `loops` timed calls; main.cpp's lines per call.
Result run_one(const Options &o, int id)
{
    Result r{LMM_OK, 0.0, 0.0, 0.0};
    const int num = 40 * o.paths;
    std::vector<double> z64;
    std::vector<float> z32;
    if (o.f32) z32.resize(num); else z64.resize(num);
    auto call = [&](double *v, double *lb) -> int {
        if (o.f32) {
            float fv = 0.f, flb = 0.f;
            const int rc = o.mrg ? lmm_swaption_greeks_mrg32k3a_f32(z32.data(), num, 0.f, 1.f, 1234, &fv, &flb, o.paths)
                                 : lmm_swaption_greeks_f32(z32.data(), num, 0.f, 1.f, 1234, &fv, &flb, o.paths);
            *v = fv;
            *lb = flb;
            return rc;
        }
        return o.mrg ? lmm_swaption_greeks_mrg32k3a(z64.data(), num, 0.0, 1.0, 1234, v, lb, o.paths)
                     : lmm_swaption_greeks(z64.data(), num, 0.0, 1.0, 1234, v, lb, o.paths);
    };
    double v = 0.0, lb = 0.0;
    r.status = call(&v, &lb);
    if (r.status != LMM_OK) return r;
    double total = 0.0;
    for (int l = 0; l < o.loops; ++l) {
        const auto t0 = std::chrono::steady_clock::now();
        r.status = call(&v, &lb);
        const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (r.status != LMM_OK) return r;
        total += ms;
        if (!o.quiet) {
            std::printf("[process %d] Number of paths: %d\n", id, o.paths);
            std::printf("[process %d] Result: value=%.10g,\tlambda=%.10g\n", id, v, lb);
            std::printf("[process %d] Total time: %.6f ms\n", id, ms);
            std::printf("[process %d] Paths/sec: %.6f KPaths/sec\n", id, o.paths / ms);
            std::fflush(stdout);
        }
    }
    r.value = v;
    r.lambda = lb;
    r.mean_ms = total / o.loops;
    return r;
}

}  // namespace

int main(int argc, char **argv)
{
    Options o;
    if (!parse(argc, argv, &o)) {
        usage(argv[0]);
        return 2;
    }
    std::printf("lmm_bench: %d paths, %d loop(s), %d process(es), %s, %s normals (library %s)\n", o.paths,
                o.loops, o.processes, o.f32 ? "FP32" : "FP64", o.mrg ? "MRG32k3a/AS241" : "Philox", lmm_version());
    std::fflush(stdout);

    std::vector<pid_t> kids;
    std::vector<int> fds;
    const auto wall0 = std::chrono::steady_clock::now();
    for (int p = 0; p < o.processes; ++p) {
        int fd[2];
        if (pipe(fd) != 0) {
            std::perror("pipe");
            return 1;
        }
        const pid_t pid = fork();
        if (pid < 0) {
            std::perror("fork");
            return 1;
        }
        if (pid == 0) {
            close(fd[0]);
            const Result r = run_one(o, p);
            if (r.status != LMM_OK)
                std::fprintf(stderr, "[process %d] %s: %s\n", p, lmm_status_string(r.status), lmm_last_error());
            const ssize_t w = write(fd[1], &r, sizeof(r));
            close(fd[1]);
            _exit(w == (ssize_t)sizeof(r) && r.status == LMM_OK ? 0 : 1);
        }
        close(fd[1]);
        kids.push_back(pid);
        fds.push_back(fd[0]);
    }
    std::vector<Result> res(o.processes);
    int failed = 0;
    for (int p = 0; p < o.processes; ++p) {
        const ssize_t got = read(fds[p], &res[p], sizeof(Result));
        close(fds[p]);
        int st = 0;
        waitpid(kids[p], &st, 0);
        if (got != (ssize_t)sizeof(Result) || !WIFEXITED(st) || WEXITSTATUS(st) != 0) ++failed;
    }
    const double wall_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - wall0).count();
    if (failed) {
        std::fprintf(stderr, "lmm_bench: %d process(es) failed\n", failed);
        return 1;
    }
    double sum = 0.0;
    for (const Result &r : res) sum += r.mean_ms;
    const double avg = sum / o.processes;  // getresults.sh: mean "Total time" over processes
    std::printf("Result: value=%.10g,\tlambda=%.10g\n", res[0].value, res[0].lambda);
    std::printf("Average total time per call: %.6f ms (mean over %d process(es))\n", avg, o.processes);
    std::printf("LiborMarketModel throughput: %.6g paths/s (paths x processes / average time per call)\n",
                (double)o.paths * o.processes / (avg * 1e-3));
    std::printf("Wall time: %.3f ms for %lld paths\n", wall_ms,
                (long long)o.paths * o.processes * (o.loops + 1));
    return 0;
}
