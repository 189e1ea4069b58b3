// Host<->device copies of many caller arrays through a page-locked staging ring.
//
// A copy from pageable memory is staged by the driver through its own bounce buffers with one
// host thread (a few GB/s on GB300's Grace host), and page-locking the caller's arrays instead
// costs about a millisecond per registration call, which dominates for hundreds of small
// arrays.  Here host threads move the data between the caller's arrays and 64 MB page-locked
// slots while the link drains or fills the neighbouring slot.
#include <algorithm>
#include <condition_variable>
#include <cstring>
#include <functional>
#include <mutex>
#include <thread>

#include "staging.cuh"

namespace jues {

namespace {

// A fixed set of worker threads running one parallel loop at a time; the caller takes tasks too.
class WorkerPool {
  public:
    explicit WorkerPool(int workers) {
        for (int i = 0; i < workers; ++i) threads_.emplace_back([this] { run(); });
    }
    ~WorkerPool() {
        {
            std::lock_guard<std::mutex> l(m_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto &t : threads_) t.join();
    }
    // fn(k) for every k in [0, n); returns when all have finished
    void parallel_for(int n, const std::function<void(int)> &fn) {
        if (n <= 0) return;
        {
            std::lock_guard<std::mutex> l(m_);
            fn_ = &fn;
            n_ = n;
            next_ = 0;
            done_ = 0;
            ++gen_;
        }
        cv_.notify_all();
        work();
        std::unique_lock<std::mutex> l(m_);
        done_cv_.wait(l, [&] { return done_ == n_; });
        fn_ = nullptr;
    }

  private:
    void work() {
        for (;;) {
            int k;
            const std::function<void(int)> *fn;
            {
                std::lock_guard<std::mutex> l(m_);
                if (!fn_ || next_ >= n_) return;
                k = next_++;
                fn = fn_;
            }
            (*fn)(k);
            std::lock_guard<std::mutex> l(m_);
            if (++done_ == n_) done_cv_.notify_all();
        }
    }
    void run() {
        unsigned long long seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> l(m_);
                cv_.wait(l, [&] { return stop_ || gen_ != seen; });
                if (stop_) return;
                seen = gen_;
            }
            work();
        }
    }
    std::vector<std::thread> threads_;
    std::mutex m_;
    std::condition_variable cv_, done_cv_;
    const std::function<void(int)> *fn_ = nullptr;
    int n_ = 0, next_ = 0, done_ = 0;
    unsigned long long gen_ = 0;
    bool stop_ = false;
};

constexpr size_t kSlot = size_t(64) << 20;
constexpr int kSlots = 3;
constexpr size_t kTask = size_t(1) << 20;   // host copy granule

// one slot's worth of ranges: stage[i] in the slot <-> host[i] / dev[i]
struct Fill {
    struct Piece {
        size_t at;   // offset in the slot
        const char *src;
        char *dst;
        size_t bytes;
    };
    std::vector<Piece> pcs;
    size_t used = 0;
};

// cut the ranges into slot-sized fills, in order
std::vector<Fill> plan_fills(const std::vector<HostSeg> &segs) {
    std::vector<Fill> fills(1);
    for (const HostSeg &s : segs) {
        size_t off = 0;
        while (off < s.bytes) {
            if (fills.back().used == kSlot) fills.emplace_back();
            Fill &f = fills.back();
            const size_t take = std::min(s.bytes - off, kSlot - f.used);
            f.pcs.push_back({f.used, static_cast<const char *>(s.src) + off, static_cast<char *>(s.dst) + off, take});
            f.used += take;
            off += take;
        }
    }
    if (fills.back().used == 0) fills.pop_back();
    return fills;
}

}  // namespace

struct Staging {
    char *host = nullptr;   // kSlots x kSlot, page-locked
    cudaEvent_t done[kSlots] = {};
    bool busy[kSlots] = {};
    WorkerPool *pool = nullptr;
};

static Staging *staging_of(Ctx *ctx) {
    if (ctx->staging) return ctx->staging;
    Staging *st = new Staging;
    ctx->staging = st;   // released by staging_destroy, also when a step below fails
    JUES_CHECK_CUDA(cudaHostAlloc(reinterpret_cast<void **>(&st->host), kSlot * kSlots, cudaHostAllocDefault));
    for (int k = 0; k < kSlots; ++k) JUES_CHECK_CUDA(cudaEventCreateWithFlags(&st->done[k], cudaEventDisableTiming));
    const unsigned hw = std::thread::hardware_concurrency();
    st->pool = new WorkerPool((int)std::min(15u, hw > 1 ? hw - 1 : 0u));
    return st;
}

// host side of one fill: copy the pieces' bytes between the slot and the caller's arrays in 1 MB
// tasks over the workers (to_slot: caller -> slot)
static void host_copy(Staging *st, const Fill &f, char *slot, bool to_slot) {
    const int ntask = (int)((f.used + kTask - 1) / kTask);
    st->pool->parallel_for(ntask, [&](int k) {
        const size_t lo = (size_t)k * kTask, hi = std::min(f.used, lo + kTask);
        // pieces are in slot order: start at the last one beginning at or before lo
        auto it = std::upper_bound(f.pcs.begin(), f.pcs.end(), lo,
                                   [](size_t x, const Fill::Piece &p) { return x < p.at; });
        for (--it; it != f.pcs.end() && it->at < hi; ++it) {
            const size_t a = std::max(lo, it->at), b = std::min(hi, it->at + it->bytes);
            if (a >= b) continue;
            if (to_slot)
                std::memcpy(slot + a, it->src + (a - it->at), b - a);
            else
                std::memcpy(it->dst + (a - it->at), slot + a, b - a);
        }
    });
}

void staged_h2d(Ctx *ctx, const std::vector<HostSeg> &segs) {
    const std::vector<Fill> fills = plan_fills(segs);
    if (fills.empty()) return;
    Staging *st = staging_of(ctx);
    for (size_t i = 0; i < fills.size(); ++i) {
        const int k = (int)(i % kSlots);
        if (st->busy[k]) JUES_CHECK_CUDA(cudaEventSynchronize(st->done[k]));   // its last copy has left
        char *slot = st->host + k * kSlot;
        host_copy(st, fills[i], slot, true);
        for (const Fill::Piece &p : fills[i].pcs)
            JUES_CHECK_CUDA(cudaMemcpyAsync(p.dst, slot + p.at, p.bytes, cudaMemcpyHostToDevice, ctx->stream));
        JUES_CHECK_CUDA(cudaEventRecord(st->done[k], ctx->stream));
        st->busy[k] = true;
    }
}

void staged_d2h(Ctx *ctx, const std::vector<HostSeg> &segs) {
    const std::vector<Fill> fills = plan_fills(segs);
    if (fills.empty()) return;
    Staging *st = staging_of(ctx);
    // the link fills slot i while the host empties slot i - 1
    auto issue = [&](size_t i) {
        const int k = (int)(i % kSlots);
        if (st->busy[k]) JUES_CHECK_CUDA(cudaEventSynchronize(st->done[k]));
        char *slot = st->host + k * kSlot;
        for (const Fill::Piece &p : fills[i].pcs)
            JUES_CHECK_CUDA(cudaMemcpyAsync(slot + p.at, p.src, p.bytes, cudaMemcpyDeviceToHost, ctx->stream));
        JUES_CHECK_CUDA(cudaEventRecord(st->done[k], ctx->stream));
        st->busy[k] = true;
    };
    issue(0);
    for (size_t i = 0; i < fills.size(); ++i) {
        if (i + 1 < fills.size()) issue(i + 1);
        const int k = (int)(i % kSlots);
        JUES_CHECK_CUDA(cudaEventSynchronize(st->done[k]));
        host_copy(st, fills[i], st->host + k * kSlot, false);
    }
}

void staging_destroy(Staging *st) {
    if (!st) return;
    for (int k = 0; k < kSlots; ++k)
        if (st->done[k]) {
            cudaEventSynchronize(st->done[k]);
            cudaEventDestroy(st->done[k]);
        }
    if (st->host) cudaFreeHost(st->host);
    delete st->pool;
    delete st;
}

}  // namespace jues
