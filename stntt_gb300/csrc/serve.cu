// serve.cu -- a request loop on one GPU (continuous batching of NTT requests).
//
// Requests (a transform, or a cyclic polynomial product = two forward
// transforms, a pointwise product and an inverse) arrive on any host thread
// through stntt_server_submit. One scheduler thread owns all CUDA work:
//   - admission: requests are taken in arrival order as soon as a stream slot
//     is free and the device arena can hold their operands (a buddy allocator
//     over one device allocation: "admission by free HBM"); a request that
//     does not fit waits at the head of the queue until memory is released;
//   - execution: each admitted request runs on its own slot stream (H2D of
//     its operands, the transform kernels, D2H of the result, an event), so
//     work of different requests overlaps on the device and requests that
//     arrive while others run join as slots and memory free up;
//   - completion: finished events release the slot and the arena block and
//     produce a completion record with host timestamps.
// Twiddle tables and per-slot workspaces stay resident; the plans for the
// configured size range are built when the server starts.
//
// The reference has no serving path; this composes its operations (nttStockham,
// pwcNtt: src/ntt/ntt_cpu.cpp:46-90, 167-174).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <vector>

#include "../../include/stntt.h"
#include "ctx_internal.h"
#include "internal.h"

namespace {

double now_s() {
    using namespace std::chrono;
    static const steady_clock::time_point t0 = steady_clock::now();
    return duration<double>(steady_clock::now() - t0).count();
}

// Binary buddy allocator over [0, 2^top) bytes, blocks of 2^min_order..2^top.
class Buddy {
  public:
    void init(uint32_t min_order, uint32_t top_order) {
        min_ = min_order;
        top_ = top_order;
        free_.assign(top_ + 1, {});
        free_[top_].insert(0);
        free_bytes_ = 1ull << top_;
    }
    bool alloc(uint32_t order, uint64_t *off) {
        order = std::max(order, min_);
        if (order > top_)
            return false;
        uint32_t o = order;
        while (o <= top_ && free_[o].empty())
            ++o;
        if (o > top_)
            return false;
        uint64_t b = *free_[o].begin();
        free_[o].erase(free_[o].begin());
        while (o > order) {  // split, keep the lower half
            --o;
            free_[o].insert(b + (1ull << o));
        }
        *off = b;
        free_bytes_ -= 1ull << order;
        return true;
    }
    void release(uint64_t off, uint32_t order) {
        order = std::max(order, min_);
        free_bytes_ += 1ull << order;
        while (order < top_) {
            const uint64_t buddy = off ^ (1ull << order);
            auto it = free_[order].find(buddy);
            if (it == free_[order].end())
                break;
            free_[order].erase(it);
            off = std::min(off, buddy);
            ++order;
        }
        free_[order].insert(off);
    }
    uint64_t free_bytes() const { return free_bytes_; }

  private:
    uint32_t min_ = 0, top_ = 0;
    uint64_t free_bytes_ = 0;
    std::vector<std::set<uint64_t>> free_;
};

struct Req {
    stntt_request r;
    double t_submit = 0, t_start = 0;
    uint64_t off = 0;
    uint32_t order = 0;
    int slot = -1;
};

struct Slot {
    cudaStream_t s = nullptr;
    cudaEvent_t ev = nullptr;
    bool busy = false;
    Req req;
};

uint32_t order_of(uint64_t bytes) {
    uint32_t o = 0;
    while ((1ull << o) < bytes)
        ++o;
    return o;
}

}  // namespace

struct stntt_server {
    stntt_ctx *ctx = nullptr;
    stntt_server_config cfg{};
    int device = 0;
    void *arena = nullptr;
    Buddy buddy;
    uint32_t arena_order = 0;
    std::vector<Slot> slots;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Req> submitted;  // mu
    std::deque<Req> pending;    // scheduler thread only
    std::deque<stntt_completion> done;  // mu
    stntt_server_stats stats{};         // mu
    std::atomic<bool> stop{false};
    std::atomic<uint64_t> outstanding{0};
    std::thread th;
};

namespace {

size_t elem_size(uint32_t field) { return field == STNTT_FIELD_GL64 ? 8 : 4; }

uint64_t req_bytes(const stntt_request &r) {
    const uint64_t one = (uint64_t)elem_size(r.field) << r.log_n;
    return r.kind == STNTT_REQ_POLYMUL ? 2 * one : one;
}

void complete(stntt_server *sv, const Req &q, int status) {
    stntt_completion c{};
    c.id = q.r.id;
    c.status = status;
    c.submit_s = q.t_submit;
    c.start_s = q.t_start;
    c.done_s = now_s();
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->done.push_back(c);
    if (status == STNTT_OK)
        sv->stats.completed++;
    else
        sv->stats.failed++;
    sv->outstanding--;
}

int launch(stntt_server *sv, Slot &sl) {
    const Req &q = sl.req;
    const stntt_request &r = q.r;
    const int field = r.field == STNTT_FIELD_GL64 ? stntt::kFieldGL : stntt::kFieldU32;
    const size_t bytes = elem_size(r.field) << r.log_n;
    char *a = static_cast<char *>(sv->arena) + q.off;
    char *b = a + bytes;
    uint64_t root = r.root;
    if (field == stntt::kFieldGL)
        stntt_gl64_root(r.log_n, &root);
    const uint32_t p = field == stntt::kFieldGL ? 0u : r.p;
    cudaError_t e = cudaMemcpyAsync(a, r.in_a, bytes, cudaMemcpyHostToDevice, sl.s);
    if (e != cudaSuccess)
        return STNTT_ECUDA;
    int rc;
    if (r.kind == STNTT_REQ_POLYMUL) {
        e = cudaMemcpyAsync(b, r.in_b, bytes, cudaMemcpyHostToDevice, sl.s);
        if (e != cudaSuccess)
            return STNTT_ECUDA;
        rc = sd::polymul_impl(sv->ctx, field, a, b, a, r.log_n, p, root, sl.s);
    } else {
        const sd::Plan *pl = nullptr;
        rc = sd::get_plan(sv->ctx, field, r.log_n, p, root, (int)r.dir, &pl, (1ull << r.log_n) < sd::kSmallCallElems);
        if (!rc)
            rc = sd::run_plan(sv->ctx, *pl, a, a, 1, sl.s);
    }
    if (rc)
        return rc;
    e = cudaMemcpyAsync(r.out, a, bytes, cudaMemcpyDeviceToHost, sl.s);
    if (e == cudaSuccess)
        e = cudaEventRecord(sl.ev, sl.s);
    return e == cudaSuccess ? STNTT_OK : STNTT_ECUDA;
}

int validate(stntt_server *sv, const stntt_request &r) {
    if (r.kind != STNTT_REQ_NTT && r.kind != STNTT_REQ_POLYMUL)
        return STNTT_EINVAL;
    if (r.field != STNTT_FIELD_U32 && r.field != STNTT_FIELD_GL64)
        return STNTT_EINVAL;
    if (r.dir != STNTT_FORWARD && r.dir != STNTT_INVERSE)
        return STNTT_EINVAL;
    if (!r.in_a || !r.out || (r.kind == STNTT_REQ_POLYMUL && !r.in_b))
        return STNTT_EINVAL;
    if (r.log_n > sv->cfg.max_log_n)
        return STNTT_EUNSUPPORTED;
    if (order_of(req_bytes(r)) > sv->arena_order)
        return STNTT_EUNSUPPORTED;
    if (r.field == STNTT_FIELD_U32) {
        if (r.p < 2 || r.p >= (1u << 31) || r.root == 0 || r.root >= r.p)
            return STNTT_EINVAL;
        if (r.log_n && (r.p - 1) % (1u << r.log_n))
            return STNTT_EINVAL;
    }
    return STNTT_OK;
}

void scheduler(stntt_server *sv) {
    cudaSetDevice(sv->device);
    for (;;) {
        {
            std::lock_guard<std::mutex> lk(sv->mu);
            while (!sv->submitted.empty()) {
                sv->pending.push_back(sv->submitted.front());
                sv->submitted.pop_front();
            }
        }
        bool progress = false, busy = false;
        const double t_poll = now_s();
        // completions
        for (Slot &sl : sv->slots) {
            if (!sl.busy)
                continue;
            const cudaError_t q = cudaEventQuery(sl.ev);
            if (q == cudaErrorNotReady) {
                busy = true;
                continue;
            }
            sv->buddy.release(sl.req.off, sl.req.order);
            sl.busy = false;
            complete(sv, sl.req, q == cudaSuccess ? STNTT_OK : STNTT_ECUDA);
            progress = true;
        }
        double t_issue = now_s();
        {
            std::lock_guard<std::mutex> lk(sv->mu);
            sv->stats.poll_ns += (uint64_t)((t_issue - t_poll) * 1e9);
        }
        // admissions, in arrival order
        while (!sv->pending.empty()) {
            Slot *free_slot = nullptr;
            for (Slot &sl : sv->slots)
                if (!sl.busy) {
                    free_slot = &sl;
                    break;
                }
            if (!free_slot)
                break;
            Req &q = sv->pending.front();
            q.order = order_of(req_bytes(q.r));
            if (!sv->buddy.alloc(q.order, &q.off))
                break;  // wait for memory to be released
            q.t_start = now_s();
            free_slot->req = q;
            free_slot->busy = true;
            sv->pending.pop_front();
            progress = true;
            {
                std::lock_guard<std::mutex> lk(sv->mu);
                const uint64_t used = (1ull << sv->arena_order) - sv->buddy.free_bytes();
                sv->stats.admitted++;
                sv->stats.peak_arena_used = std::max<uint64_t>(sv->stats.peak_arena_used, used);
                uint64_t inflight = 0;
                for (const Slot &s2 : sv->slots)
                    inflight += s2.busy;
                sv->stats.peak_inflight = std::max<uint64_t>(sv->stats.peak_inflight, inflight);
            }
            const int rc = launch(sv, *free_slot);
            if (rc) {
                cudaStreamSynchronize(free_slot->s);
                sv->buddy.release(free_slot->req.off, free_slot->req.order);
                free_slot->busy = false;
                complete(sv, free_slot->req, rc);
            }
            const double t = now_s();
            {
                std::lock_guard<std::mutex> lk(sv->mu);
                sv->stats.issue_ns += (uint64_t)((t - t_issue) * 1e9);
            }
            t_issue = t;
        }
        if (sv->stop.load() && sv->pending.empty() && !busy && !progress) {
            std::lock_guard<std::mutex> lk(sv->mu);
            if (sv->submitted.empty())
                break;
        }
        if (!progress) {
            std::unique_lock<std::mutex> lk(sv->mu);
            sv->cv.wait_for(lk, std::chrono::microseconds(busy ? 10 : 200),
                            [&] { return !sv->submitted.empty() || sv->stop.load(); });
        }
    }
}

}  // namespace

extern "C" {

double stntt_clock_s(void) { return now_s(); }

int stntt_server_create(stntt_ctx *ctx, const stntt_server_config *cfg, stntt_server **out) {
    if (!ctx || !out)
        return STNTT_EINVAL;
    *out = nullptr;
    auto sv = std::make_unique<stntt_server>();
    sv->ctx = ctx;
    stntt_server_config c{};
    if (cfg)
        c = *cfg;
    if (c.streams == 0)
        c.streams = 32;
    if (c.max_log_n == 0)
        c.max_log_n = 22;
    if (c.streams > 128 || c.max_log_n > 26)
        return sd::fail(ctx, STNTT_EINVAL, "server: streams <= 128 and max_log_n <= 26");
    sv->cfg = c;
    sv->device = sd::ctx_device(ctx);
    cudaSetDevice(sv->device);
    // arena: requested size, else a quarter of free HBM capped at 8 GiB; a power of two
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess)
        return sd::fail(ctx, STNTT_ECUDA, "server: cudaMemGetInfo failed");
    uint64_t want = c.arena_bytes ? c.arena_bytes : std::min<uint64_t>(fr / 4, 8ull << 30);
    uint32_t order = 0;
    while ((2ull << order) <= want)
        ++order;
    if (order < 16)
        return sd::fail(ctx, STNTT_ENOMEM, "server: arena smaller than 64 KiB");
    if ((1ull << order) > fr)
        return sd::fail(ctx, STNTT_ENOMEM, "server: not enough free HBM for the arena");
    if (cudaMalloc(&sv->arena, 1ull << order) != cudaSuccess)
        return sd::fail(ctx, STNTT_ENOMEM, "server: arena allocation failed");
    sv->arena_order = order;
    sv->buddy.init(16, order);
    sv->stats.arena_bytes = 1ull << order;
    sv->slots.resize(c.streams);
    const size_t ws = (size_t)2 * 8 << c.max_log_n;  // polymul on Goldilocks at the largest size
    for (Slot &sl : sv->slots) {
        if (cudaStreamCreateWithFlags(&sl.s, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming) != cudaSuccess) {
            stntt_server_destroy(sv.release());
            return sd::fail(ctx, STNTT_ECUDA, "server: stream creation failed");
        }
        void *p = nullptr;
        if (sd::get_workspace(ctx, sl.s, ws, &p)) {
            stntt_server_destroy(sv.release());
            return STNTT_ENOMEM;
        }
    }
    // resident twiddle tables for both fields, both directions, the size range:
    // the very plans a request of that size looks up (a request is one call of
    // one transform, so sizes below 2^22 take the small-call plans). A plan
    // built in the middle of a trace stalls the scheduler thread while its
    // tables are allocated and generated.
    for (uint32_t lg = c.prewarm_min_log_n; c.prewarm_max_log_n && lg <= c.prewarm_max_log_n; ++lg) {
        const int kind = (1ull << lg) < sd::kSmallCallElems ? sd::kPlanSmall : sd::kPlanAll;
        for (int dir = 0; dir < 2; ++dir) {
            uint32_t p32 = 0, r32 = 0;
            uint64_t rg = 0;
            const sd::Plan *pl = nullptr;
            stntt_gl64_root(lg, &rg);
            int rc = sd::get_plan(ctx, stntt::kFieldGL, lg, 0, rg, dir, &pl, kind);
            if (!rc)
                rc = stntt_params_u32(lg, &p32, &r32);
            if (!rc)
                rc = sd::get_plan(ctx, stntt::kFieldU32, lg, p32, r32, dir, &pl, kind);
            if (rc) {
                stntt_server_destroy(sv.release());
                return rc;
            }
        }
    }
    stntt_server *raw = sv.release();
    raw->th = std::thread(scheduler, raw);
    *out = raw;
    return STNTT_OK;
}

int stntt_server_submit(stntt_server *sv, const stntt_request *req) {
    return stntt_server_submit_at(sv, req, now_s());
}

int stntt_server_submit_at(stntt_server *sv, const stntt_request *req, double t_submit) {
    if (!sv || !req)
        return STNTT_EINVAL;
    Req q;
    q.r = *req;
    q.t_submit = t_submit;
    const int v = validate(sv, q.r);
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->stats.submitted++;
        sv->outstanding++;
        if (v == STNTT_OK)
            sv->submitted.push_back(q);
        else
            sv->stats.rejected++;
    }
    if (v != STNTT_OK) {
        q.t_start = now_s();
        complete(sv, q, v);
        return v;
    }
    sv->cv.notify_one();
    return STNTT_OK;
}

int stntt_server_poll(stntt_server *sv, stntt_completion *out, size_t max, size_t *got) {
    if (!sv || !got || (!out && max))
        return STNTT_EINVAL;
    std::lock_guard<std::mutex> lk(sv->mu);
    size_t k = 0;
    while (k < max && !sv->done.empty()) {
        out[k++] = sv->done.front();
        sv->done.pop_front();
    }
    *got = k;
    return STNTT_OK;
}

int stntt_server_wait_idle(stntt_server *sv, double timeout_s) {
    if (!sv)
        return STNTT_EINVAL;
    const double t_end = now_s() + timeout_s;
    while (sv->outstanding.load() > 0) {
        if (now_s() > t_end)
            return STNTT_ETIMEOUT;
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    return STNTT_OK;
}

int stntt_server_stats_get(stntt_server *sv, stntt_server_stats *out) {
    if (!sv || !out)
        return STNTT_EINVAL;
    std::lock_guard<std::mutex> lk(sv->mu);
    *out = sv->stats;
    return STNTT_OK;
}

int stntt_server_run_trace(stntt_server *sv, const stntt_request *reqs, const double *arrival_s, size_t n,
                           double timeout_s, stntt_completion *out) {
    if (!sv || (n && (!reqs || !arrival_s || !out)))
        return STNTT_EINVAL;
    const double t0 = now_s() + 1e-3;
    double late_max = 0;
    uint64_t late_count = 0;
    for (size_t i = 0; i < n; ++i) {
        const double t = t0 + arrival_s[i];
        double now;
        while ((now = now_s()) < t) {
        }
        late_max = std::max(late_max, now - t);
        late_count += now - t > 0.5e-3;
        stntt_server_submit_at(sv, &reqs[i], t);
    }
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->stats.trace_late_max_ns = std::max<uint64_t>(sv->stats.trace_late_max_ns, (uint64_t)(late_max * 1e9));
        sv->stats.trace_late_count += late_count;
    }
    int rc = stntt_server_wait_idle(sv, timeout_s);
    // gather: completions carry the request ids; place by position among reqs
    std::vector<stntt_completion> all;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        all.assign(sv->done.begin(), sv->done.end());
        sv->done.clear();
    }
    for (size_t i = 0; i < n; ++i)
        out[i] = stntt_completion{};
    for (const stntt_completion &c : all)
        if (c.id < n)
            out[c.id] = c;
    return rc;
}

int stntt_server_destroy(stntt_server *sv) {
    if (!sv)
        return STNTT_EINVAL;
    if (sv->th.joinable()) {
        sv->stop.store(true);
        sv->cv.notify_all();
        sv->th.join();
    }
    cudaSetDevice(sv->device);
    for (Slot &sl : sv->slots) {
        if (sl.s) {
            cudaStreamSynchronize(sl.s);
            sd::release_workspace(sv->ctx, sl.s);
        }
        if (sl.ev)
            cudaEventDestroy(sl.ev);
        if (sl.s)
            cudaStreamDestroy(sl.s);
    }
    if (sv->arena)
        cudaFree(sv->arena);
    delete sv;
    return STNTT_OK;
}

}  // extern "C"
