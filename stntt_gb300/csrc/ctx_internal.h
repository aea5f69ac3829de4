// ctx_internal.h -- context services shared by the C-ABI translation units
// (api.cu defines them; serve.cu uses them). Not installed.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/stntt.h"

namespace sd {

struct Plan;

// Twiddle tables and pass list for one transform (built and cached on first use).
// kind: kPlanSmall for a call of fewer than kSmallCallElems elements in all,
// kPlanBatched for a job of the persistent batched launch; each uses its own
// shape when stntt_set_plan_small / stntt_set_plan_batched set one, else the
// shape of every call (kPlanAll).
constexpr uint64_t kSmallCallElems = 1ull << 22;
enum : int { kPlanAll = 0, kPlanSmall = 1, kPlanBatched = 2 };
int get_plan(stntt_ctx *ctx, int field, uint32_t log_n, uint32_t p, uint64_t root, int dir, const Plan **out,
             int kind = kPlanAll);
// Run a plan: first pass reads `in`, last pass writes `out`, on stream s.
// in2: optional second input whose product with `in` the first pass transforms.
int run_plan(stntt_ctx *ctx, const Plan &pl, const void *in, void *out, uint64_t batch, cudaStream_t s,
             const void *in2 = nullptr);
// Per-stream scratch of at least `bytes` (grows with a synchronising cudaMalloc);
// *tail (optional): 256 zero-initialised bytes after it that belong to the stream.
int get_workspace(stntt_ctx *ctx, cudaStream_t s, size_t bytes, void **ptr, void **tail = nullptr);
// Free the workspace of a stream that is about to be destroyed.
int release_workspace(stntt_ctx *ctx, cudaStream_t s);
// Cyclic product of two length-2^log_n operands (device pointers) on stream s.
int polymul_impl(stntt_ctx *ctx, int field, const void *a, const void *b, void *out, uint32_t log_n, uint32_t p,
                 uint64_t root, cudaStream_t s);
int check_u32_args(stntt_ctx *ctx, uint32_t log_n, uint32_t p, uint32_t root);
int fail(stntt_ctx *ctx, int status, const std::string &msg);
int ctx_device(const stntt_ctx *ctx);

}  // namespace sd
