// flock_gb300: command-line drop-in for the reference's CUDA backend
// (cuda/flock.cu:374-523). Same flags, same .flk input/output, same stdout
// table, so scripts that drive `flock_cuda` (scripts/parity.sh) can point at
// this binary instead.
//
//   flock_gb300 --in FILE [--steps K] [--warmup W] [--out FILE] [--decide-smem N]
//
// --decide-smem N reserves N more bytes of dynamic shared memory per decide
// CTA, the reference's occupancy experiment (cuda/flock.cu:377,385); the
// "# decide occupancy" header line reports the resulting launch, in the
// reference's format (cuda/flock.cu:440-445).
//
// Exit codes: 0 ok, 1 CUDA / IO / device error, 2 usage.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <string>

#include "../../include/flock_gb300.h"

static int die(const char* what) {
    std::fprintf(stderr, "flock_gb300: %s: %s\n", what, flk_last_error());
    return 1;
}

int main(int argc, char** argv) {
    const char *in = nullptr, *out = nullptr;
    int steps = 1, warmup = 0;
    unsigned long long decide_smem = 0;
    for (int k = 1; k < argc; ++k) {
        const std::string a = argv[k];
        auto val = [&]() -> const char* {
            if (k + 1 >= argc) {
                std::fprintf(stderr, "missing value for %s\n", a.c_str());
                std::exit(2);
            }
            return argv[++k];
        };
        if (a == "--in") in = val();
        else if (a == "--out") out = val();
        else if (a == "--steps") steps = std::atoi(val());
        else if (a == "--warmup") warmup = std::atoi(val());
        else if (a == "--decide-smem") decide_smem = std::strtoull(val(), nullptr, 10);
        else {
            std::fprintf(stderr,
                         "usage: flock_gb300 --in FILE [--steps K] [--warmup W] [--out FILE] [--decide-smem N]\n"
                         "(the first W steps are not timed)\n");
            return 2;
        }
    }
    if (!in) {
        std::fprintf(stderr, "missing --in\n");
        return 2;
    }
    steps = std::max(steps, 0);
    warmup = std::min(std::max(warmup, 0), steps);

    flk_flock* f = nullptr;
    if (flk_open_file(-1, in, &f) != FLK_OK) return die(in);
    uint32_t n = 0;
    flk_size(f, &n, nullptr);

    int dev = 0, drv = 0, rt = 0;
    cudaDeviceProp prop{};
    cudaGetDevice(&dev);
    cudaGetDeviceProperties(&prop, dev);
    cudaDriverGetVersion(&drv);
    cudaRuntimeGetVersion(&rt);
    std::printf("# flock_gb300: %s (sm_%d%d), CUDA driver %d.%d runtime %d.%d\n", prop.name, prop.major, prop.minor,
                drv / 1000, drv % 1000 / 10, rt / 1000, rt % 1000 / 10);
    std::printf("# %u birds, %d steps (%d warm-up, not timed)\n", n, steps, warmup);
    {
        int32_t bps = 0, tpb = 0, tpsm = 0;
        uint64_t smem = 0;
        if (flk_decide_occupancy(f, decide_smem, &bps, &tpb, &tpsm, &smem) != FLK_OK) {
            std::fprintf(stderr, "flock_gb300: --decide-smem %llu: %s\n", decide_smem, flk_last_error());
            flk_close(f);
            return 2;
        }
        std::printf("# decide occupancy: %d blocks/SM of %d threads = %d%% of %d threads/SM (dynamic smem %llu B)\n",
                    bps, tpb, tpsm ? 100 * bps * tpb / tpsm : 0, tpsm, (unsigned long long)smem);
    }

    flk_pass_times pt{};
    if (steps > 0 && flk_step_timed(f, (uint32_t)steps, (uint32_t)warmup, &pt) != FLK_OK) return die("step");
    const int timed = steps - warmup;
    if (timed > 0) {
        std::printf("# %d timed steps (mean GPU ms per pass, CUDA events)\n", timed);
        std::printf("  %-16s %9.4f\n", "grid_histogram", pt.hash_ms);
        std::printf("  %-16s %9.4f\n", "grid_scan", pt.scan_ms);
        std::printf("  %-16s %9.4f\n", "grid_scatter", pt.sort_ms);
        std::printf("  %-16s %9.4f\n", "decide", pt.decide_ms);
        std::printf("  %-16s %9.4f\n", "integrate", pt.integrate_ms);
        std::printf("  %-16s %9.4f\n  bird-steps/s     %9.0f\n", "step total", pt.total_ms,
                    pt.total_ms > 0 ? n / (pt.total_ms / 1000.0) : 0.0);
    }
    if (out && flk_write_file(f, out) != FLK_OK) return die(out);
    flk_close(f);
    return 0;
}
