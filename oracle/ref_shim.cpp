// ref_shim.cpp -- C entry points over the UNMODIFIED reference CPU code
// (TEST INFRASTRUCTURE). Compiled by oracle/Makefile together with the
// reference's own src/ntt/ntt_cpu.cpp and src/ntt/ntt_util.cpp, read in
// place from the reference checkout; nothing of the reference is copied.
// The result, oracle/_ref/libstntt_ref.so, generates the golden vectors in
// tests/golden and validates the C restatement in stntt_oracle.c.
#include "ntt/ntt_cpu.h"
#include "ntt/ntt_util.h"
#include "util/rng.h"

#include <cstdint>
#include <cstring>
#include <exception>
#include <optional>
#include <span>
#include <vector>

// Defined in ntt_cpu.cpp:130 with external linkage but not declared in its header.
void inttGs(std::vector<int> &vec, int root, int mod);

extern "C" {

int ref_find_params(uint64_t size, uint64_t min_mod, uint64_t *root, uint64_t *mod) {
    try {
        auto [r, m] = findParams(size, min_mod);
        *root = r;
        *mod = m;
        return 0;
    } catch (const std::exception &) {
        return -1;
    }
}

// nttStockham(int*, size, root, mod, nsteps) -- ntt_cpu.cpp:46
int ref_ntt_stockham(int *vec, int size, int root, int mod, int nsteps) {
    try {
        std::optional<int> ns;
        if (nsteps >= 0)
            ns = nsteps;
        nttStockham(vec, size, root, mod, ns);
        return 0;
    } catch (const std::exception &) {
        return -1;
    }
}

// nttStockham(span, size, root, mod, batches) -- ntt_cpu.cpp:87
int ref_ntt_stockham_batch(int *vec, int size, int root, int mod, int batches) {
    try {
        nttStockham(std::span<int>(vec, (size_t)size * batches), size, root, mod, batches);
        return 0;
    } catch (const std::exception &) {
        return -1;
    }
}

// nttCt -- ntt_cpu.cpp:11 (NO->BO)
int ref_ntt_ct(int *vec, int n, int root, int mod) {
    try {
        std::vector<int> v(vec, vec + n);
        nttCt(v, root, mod);
        std::memcpy(vec, v.data(), sizeof(int) * n);
        return 0;
    } catch (const std::exception &) {
        return -1;
    }
}

// inttGs -- ntt_cpu.cpp:130 (BO->NO, scaled by n^-1)
int ref_intt_gs(int *vec, int n, int root, int mod) {
    try {
        std::vector<int> v(vec, vec + n);
        inttGs(v, root, mod);
        std::memcpy(vec, v.data(), sizeof(int) * n);
        return 0;
    } catch (const std::exception &) {
        return -1;
    }
}

// pwc_convolution -- ntt_cpu.cpp:180
int ref_pwc_convolution(const int *s0, const int *s1, int len, int *out, int *root, int *mod) {
    try {
        auto [v, r, m] = pwc_convolution(std::span<const int>(s0, len), std::span<const int>(s1, len));
        std::memcpy(out, v.data(), sizeof(int) * len);
        *root = r;
        *mod = m;
        return 0;
    } catch (const std::exception &) {
        return -1;
    }
}

// util::Rng(seed).get_vector(n) -- src/util/rng.h:14-30
void ref_rng_vector(int seed, int *out, size_t n) {
    util::Rng rng(seed);
    std::vector<int> v = rng.get_vector(n);
    std::memcpy(out, v.data(), sizeof(int) * n);
}
}
