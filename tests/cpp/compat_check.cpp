// Exercises include/stntt_compat.hpp the way the reference's doctest suite
// (src/tests/cuda/ntt/st_ntt_test.cu:16-45) uses the reference API: findParams,
// the CPU-style nttStockham and cuda::ntt::autoNtt<n>, on inputs 0..9 read from
// stdin. Prints one line per case: "log_n batch fnv1a64(output)".
#include <cstdint>
#include <cstdio>
#include <iostream>
#include <vector>

#include "stntt_compat.hpp"

static uint64_t fnv1a(const std::vector<int> &v) {
    uint64_t h = 0xcbf29ce484222325ull;
    for (int x : v)
        for (int b = 0; b < 4; ++b) {
            h ^= (uint8_t)((uint32_t)x >> (8 * b));
            h *= 0x100000001b3ull;
        }
    return h;
}

template <size_t I>
static void run(const std::vector<int> &in, int batches) {
    constexpr size_t n = size_t(1) << I;
    auto [root, mod] = findParams(n, 11);
    std::vector<int> a(in.begin(), in.begin() + n * batches);
    std::vector<int> b = a;
    nttStockham(std::span<int>(a), (int)n, (int)root, (int)mod, batches);
    cuda::ntt::NttArgs args(b, n, batches, root, mod, 2, 1024);
    const float ms = cuda::ntt::autoNtt<n>(args);
    if (a != b) {
        std::printf("MISMATCH %zu %d\n", I, batches);
        return;
    }
    if (!(ms > 0.f)) {  // the reference returns the event-timed kernel time
        std::printf("NO-KERNEL-TIME %zu %d\n", I, batches);
        return;
    }
    std::printf("%zu %d %016llx\n", I, batches, (unsigned long long)fnv1a(a));
}

int main() {
    std::vector<int> in;
    int x;
    while (std::cin >> x)
        in.push_back(x);
    for (int batches : {1, 2, 5, 10}) {
        run<4>(in, batches);
        run<10>(in, batches);
        run<14>(in, batches);
        run<16>(in, batches);
    }
    try {
        std::vector<int> bad(12);
        nttStockham(std::span<int>(bad), 12, 1, 13, 1);
        std::printf("NO-THROW\n");
    } catch (const std::invalid_argument &e) {
        std::printf("invalid_argument: %s\n", e.what());
    }
    return 0;
}
