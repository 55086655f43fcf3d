// ref_callers.cpp -- a main() for the reference's OWN callers of the engine,
// linked against the GPU shim (prothlogic_gb300/compat/fft_engine_gpu.cpp) and
// libprothgpu.so instead of the reference's fft_engine.cpp / llr_fft_pack.cpp.
// Built by oracle/ref/build_ref_callers.sh from the unmodified dcore.cpp,
// worker.cpp, pipeline_proth.cpp, proth_logic.cpp, checkpoint_manager.cpp,
// storage_core.cpp and progress_core.cpp.
//
//   ref_callers autotune <n> <k>          auto_tune_fft_len (dcore.cpp:20-81) through the shim
//   ref_callers test <k> <n>              auto_tune_fft_len, then execute_proth_test_fft
//                                         (proth_logic.cpp:384-580) on a worker-style context and
//                                         limb buffer (dcore.cpp:134-155); prints verdict, RES64, L
//   ref_callers dispatch <n> <workers> <k1,k2,...>
//                                         build_proth_ff_tasks_for_range (pipeline_proth.cpp:21-75)
//                                         + dispatch (dcore.cpp:84-193) over worker threads
#include <sys/mman.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <sstream>
#include <string>
#include <vector>

#include "dcore.h"
#include "fft_engine.h"
#include "pipeline_proth.h"
#include "proth_logic.h"

size_t auto_tune_fft_len(unsigned actual_n, uint64_t sample_k);  // dcore.cpp:20 (not in dcore.h)

int main(int argc, char** argv) {
    if (argc < 4) return 2;
    const std::string mode = argv[1];
    if (mode == "autotune") {
        const unsigned n = (unsigned)strtoul(argv[2], nullptr, 10);
        const uint64_t k = strtoull(argv[3], nullptr, 10);
        printf("L %zu\n", auto_tune_fft_len(n, k));
        return 0;
    }
    if (mode == "test") {
        const uint64_t k = strtoull(argv[2], nullptr, 10);
        const unsigned n = (unsigned)strtoul(argv[3], nullptr, 10);
        const size_t L = auto_tune_fft_len(n, k);
        FFTContext ctx;
        if (!fft_init(ctx, FFTBackend::INTERNAL, L)) return 3;
        const size_t nl = std::max(L, (size_t)((2 * n) / 64 + 64));  // dcore.cpp:143-155
        uint64_t* limbs = (uint64_t*)mmap(nullptr, nl * 8, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
        if (limbs == MAP_FAILED) return 4;
        std::memset(limbs, 0, nl * 8);
        const auto t0 = std::chrono::steady_clock::now();
        const bool prime = execute_proth_test_fft(k, n, limbs, ctx, 0);
        const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        printf("RESULT %d %016llx %zu %.3f\n", prime ? 1 : 0, (unsigned long long)limbs[0], L, s * 1e6 / (n - 1));
        munmap(limbs, nl * 8);
        fft_destroy(ctx);
        return 0;
    }
    if (mode == "dispatch" && argc >= 5) {
        const unsigned n = (unsigned)strtoul(argv[2], nullptr, 10);
        const int workers = atoi(argv[3]);
        std::vector<uint64_t> ks;
        std::stringstream ss(argv[4]);
        for (std::string t; std::getline(ss, t, ',');) ks.push_back(strtoull(t.c_str(), nullptr, 10));
        std::vector<Task> tasks;
        build_proth_ff_tasks_for_range(n, ks, "primes.txt", workers, tasks, 0);
        dispatch(tasks, workers);
        printf("DISPATCHED %zu\n", tasks.size());
        return 0;
    }
    return 2;
}
