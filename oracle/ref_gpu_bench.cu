// ref_gpu_bench.cu -- times the reference's own CUDA NTT on this GPU
// (BASELINE INFRASTRUCTURE, not part of the library).
//
// Built by `make -C oracle ref-gpu` against an unmodified copy of the
// reference sources (src/ and third_party/), for sm_100: the reference's
// cuda::ntt::autoNtt<n> (src/cuda/ntt/ntt_kernel.cuh:153-200) with the
// parameters every reference caller uses, findParams(n, 11)
// (src/ntt/ntt_util.cpp:10-14), batch 1, radix 2, at each block size of the
// reference's own sweep (defaultMaxBlockSizes, ntt_kernel.cuh:27). The same
// call sequence as the reference's benchmark loop (runNttIteration,
// src/bench.cu:26-55), which records autoNtt's return value -- kernel
// milliseconds between two CUDA events -- as "Kernel time", and the wall time
// of the call (allocation, twiddle upload, copies, kernels) as
// "Kernel+transfers time". Only the reporting is this file's: one JSON line
// per (n, block size) on stdout.
//
// Sizes: argv[1] = comma-separated log2 n from {16, 20, 26}; argv[2] = timed
// repetitions (after 2 untimed ones). The reference's arithmetic is int32 with
// wrap-around (exact only for n <= 2^13); the timing does not depend on it.
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "cuda/ntt/ntt_kernel.cuh"
#include "ntt/ntt_util.h"

namespace {

template <size_t LOG>
void run(int reps) {
    constexpr size_t n = size_t(1) << LOG;
    auto [root, mod] = findParams(n, 11);
    // uniform residues in [0, mod) from a fixed 64-bit LCG (the values do not
    // change the reference's work)
    std::vector<int> base(n);
    uint64_t z = 0x5717000100000000ull + LOG;
    for (size_t i = 0; i < n; ++i) {
        z = z * 6364136223846793005ull + 1442695040888963407ull;
        base[i] = (int)((z >> 33) % mod);
    }
    for (unsigned bs : cuda::ntt::defaultMaxBlockSizes) {
        std::vector<int> v = base;
        cuda::ntt::NttArgs args(std::span<int>(v), (unsigned)n, 1u, (unsigned)root, (unsigned)mod, 2u, bs);
        for (int w = 0; w < 2; ++w)
            cuda::ntt::autoNtt<n>(args);
        std::string kms, wms;
        double ksum = 0, wsum = 0, kmin = 1e30;
        for (int r = 0; r < reps; ++r) {
            auto t0 = std::chrono::steady_clock::now();
            const float k = cuda::ntt::autoNtt<n>(args);
            const double w = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
            ksum += k;
            wsum += w;
            kmin = k < kmin ? k : kmin;
            kms += (r ? "," : "") + std::to_string(k);
            wms += (r ? "," : "") + std::to_string(w);
        }
        std::printf("{\"log_n\": %zu, \"block_size\": %u, \"root\": %zu, \"mod\": %zu, \"reps\": %d, "
                    "\"kernel_ms_mean\": %.6f, \"kernel_ms_min\": %.6f, \"wall_ms_mean\": %.6f, "
                    "\"kernel_ms\": [%s], \"wall_ms\": [%s]}\n",
                    LOG, bs, (size_t)root, (size_t)mod, reps, ksum / reps, kmin, wsum / reps, kms.c_str(),
                    wms.c_str());
        std::fflush(stdout);
    }
}

}  // namespace

int main(int argc, char **argv) {
    const std::string sizes = argc > 1 ? argv[1] : "16,20,26";
    const int reps = argc > 2 ? std::atoi(argv[2]) : 5;
    if (reps < 1)
        return 2;
    size_t pos = 0;
    while (pos <= sizes.size()) {
        const size_t comma = sizes.find(',', pos);
        const int lg = std::atoi(sizes.substr(pos, comma == std::string::npos ? std::string::npos : comma - pos).c_str());
        switch (lg) {
        case 16: run<16>(reps); break;
        case 20: run<20>(reps); break;
        case 26: run<26>(reps); break;
        default: std::fprintf(stderr, "unsupported log2 n %d (16, 20 or 26)\n", lg); return 2;
        }
        if (comma == std::string::npos)
            break;
        pos = comma + 1;
    }
    return 0;
}
