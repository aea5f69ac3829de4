// stntt_compat.hpp -- the reference's C++ entry points on top of libstntt.
//
// Header-only. Mirrors the names and argument meaning of AlvaroPardoFente/stNTT's
// hot-path interface so its callers can be relinked against libstntt:
//   findParams(size, min_mod) -> (root, mod)          src/ntt/ntt_util.h:11
//   nttStockham(int *vec, size, root, mod, nsteps)     src/ntt/ntt_cpu.h:8
//   nttStockham(std::span<int>, size, root, mod, batches, nsteps)   ntt_cpu.h:9
//   cuda::ntt::NttArgs, cuda::ntt::autoNtt<n>(args)    src/cuda/ntt/ntt_kernel.cuh:41-82,153
// The transforms run on GPU 0 through the C ABI. nttStockham and autoNtt use
// STNTT_FLAG_REF_WRAP, i.e. the reference's own int32 arithmetic, so results are
// identical to the reference at every size; nttStockhamExact gives the exact
// field transform (identical to the reference for size <= 2^13).
// Errors throw std::invalid_argument (bad arguments, as the reference) or
// std::runtime_error (CUDA failures; the reference exits the process).
#pragma once

#include <cstddef>
#include <cstdint>
#include <optional>
#include <span>
#include <stdexcept>
#include <string>
#include <tuple>

#include "stntt.h"

namespace stntt_compat {

inline stntt_ctx *default_ctx() {
    static stntt_ctx *ctx = [] {
        stntt_ctx *c = nullptr;
        if (stntt_init(&c, 0) != STNTT_OK)
            throw std::runtime_error("stntt_init failed: no usable CUDA device 0");
        return c;
    }();
    return ctx;
}

inline void check(int rc, stntt_ctx *ctx) {
    if (rc == STNTT_OK)
        return;
    const std::string msg = ctx ? stntt_last_error(ctx) : stntt_status_string(rc);
    if (rc == STNTT_EINVAL)
        throw std::invalid_argument(msg);
    throw std::runtime_error(msg);
}

inline void stockham(int *vec, int size, int root, int mod, int batches, std::optional<int> nsteps,
                     uint32_t flags) {
    stntt_ctx *ctx = default_ctx();
    check(stntt_ntt_stockham_host(ctx, vec, size, root, mod, batches, nsteps ? *nsteps : -1, flags), ctx);
}

}  // namespace stntt_compat

inline std::tuple<size_t, size_t> findParams(size_t size, size_t min_mod) {
    uint64_t root = 0, mod = 0;
    const int rc = stntt_find_params(size, min_mod, &root, &mod);
    if (rc == STNTT_EINVAL)
        throw std::invalid_argument("findParams: size and min_mod must be positive");
    if (rc)
        throw std::overflow_error("findParams: search range exhausted");
    return {static_cast<size_t>(root), static_cast<size_t>(mod)};
}

inline void nttStockham(int *vec, int size, int root, int mod, std::optional<int> nsteps = std::nullopt) {
    stntt_compat::stockham(vec, size, root, mod, 1, nsteps, STNTT_FLAG_REF_WRAP);
}

inline void nttStockham(std::span<int> vec, int size, int root, int mod, int batches,
                        std::optional<int> nsteps = std::nullopt) {
    if (vec.size() < static_cast<size_t>(size) * static_cast<size_t>(batches))
        throw std::invalid_argument("vec is shorter than size * batches");
    stntt_compat::stockham(vec.data(), size, root, mod, batches, nsteps, STNTT_FLAG_REF_WRAP);
}

inline void nttStockhamExact(std::span<int> vec, int size, int root, int mod, int batches = 1) {
    stntt_compat::stockham(vec.data(), size, root, mod, batches, std::nullopt, 0);
}

namespace cuda::ntt {

constexpr unsigned defaultBlockSize = 1024;

// The arguments autoNtt reads (ntt_kernel.cuh:41-82). Launch geometry
// (radix, blockSize) is accepted and ignored: the library plans its own.
struct NttArgs {
    unsigned n{}, batches{}, root{}, mod{}, radix{2}, blockSize{defaultBlockSize};
    std::span<int> vec;
    NttArgs() = default;
    NttArgs(unsigned n_, unsigned batches_, unsigned root_, unsigned mod_, unsigned radix_,
            unsigned blockSize_ = defaultBlockSize)
        : n(n_), batches(batches_), root(root_), mod(mod_), radix(radix_), blockSize(blockSize_) {}
    NttArgs(std::span<int> vec_, unsigned n_, unsigned batches_, unsigned root_, unsigned mod_, unsigned radix_,
            unsigned blockSize_ = defaultBlockSize)
        : NttArgs(n_, batches_, root_, mod_, radix_, blockSize_) {
        vec = vec_;
    }
};

// In place on args.vec (host memory), like the reference. Returns the device
// time of the transform in milliseconds, measured with CUDA events recorded
// after the copy in and before the copy out, as the reference's autoNtt does
// (ntt_kernel.cuh:167,187-191).
template <size_t n>
float autoNtt(NttArgs args) {
    if (args.n != n)
        throw std::invalid_argument("autoNtt<n>: args.n differs from n");
    ::nttStockham(args.vec, static_cast<int>(n), static_cast<int>(args.root), static_cast<int>(args.mod),
                  static_cast<int>(args.batches));
    stntt_ctx *ctx = stntt_compat::default_ctx();
    float ms = 0.f;
    stntt_compat::check(stntt_last_kernel_ms(ctx, &ms), ctx);
    return ms;
}

}  // namespace cuda::ntt
