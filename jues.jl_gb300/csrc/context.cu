// Context: stream, memory accounting, per-kernel event timing, error flags.
#include <nvtx3/nvToolsExt.h>

#include <chrono>
#include <cstdint>
#include <cstring>

#include <algorithm>

#include "common.cuh"
#include "staging.cuh"

namespace jues {

static thread_local std::string g_last_error;
void set_last_error(const std::string &msg) { g_last_error = msg; }
const std::string &last_error() { return g_last_error; }

Ctx::Ctx() {}

Ctx::~Ctx() {
    if (stream) cudaStreamSynchronize(stream);
    PackCache *pk = pack;
    pack = nullptr;   // the cache's own buffers are freed below; no lookups into it meanwhile
    pack_cache_destroy(pk);
    batch_cache_destroy(batch);
    batch = nullptr;
    staging_destroy(staging);
    staging = nullptr;
    for (auto &kv : prof) {
        for (auto &e : kv.second.pending) { cudaEventDestroy(e.first); cudaEventDestroy(e.second); }
        for (auto &e : kv.second.pool) { cudaEventDestroy(e.first); cudaEventDestroy(e.second); }
    }
    if (splitk_ws) free(splitk_ws, splitk_bytes);
    splitk_ws = nullptr;
    if (stream) cudaStreamSynchronize(stream);
    if (pool) cudaMemPoolDestroy(pool);   // returns everything the pool still holds
    if (d_flags) cudaFree(d_flags);
    if (d_red) cudaFree(d_red);
    if (stream) cudaStreamDestroy(stream);
}

void *Ctx::alloc(size_t bytes) {
    if (bytes == 0) return nullptr;
    if (mem_limit && mem_used + bytes > mem_limit)
        throw Error(JUES_ENOMEM, "device allocation of " + std::to_string(bytes) +
                                     " bytes exceeds the context memory limit (" +
                                     std::to_string(mem_limit) + " bytes, " +
                                     std::to_string(mem_used) + " in use)");
    // Stream-ordered allocation from the context's own pool.  Freed blocks stay in the pool
    // (release threshold = unlimited) and are handed out again in stream order, so the large
    // per-call buffers (AO integrals, packed operands, transform scratch) cost no
    // cudaMalloc/cudaFree round trips and no implicit device synchronisation after warm-up.
    if (!pool) {
        cudaMemPoolProps props;
        std::memset(&props, 0, sizeof(props));
        props.allocType = cudaMemAllocationTypePinned;
        props.handleTypes = cudaMemHandleTypeNone;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        JUES_CHECK_CUDA(cudaMemPoolCreate(&pool, &props));
        uint64_t keep = UINT64_MAX;
        JUES_CHECK_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    }
    void *p = nullptr;
    cudaError_t e = cudaMallocFromPoolAsync(&p, bytes, pool, stream);
    if (e != cudaSuccess) {
        // give the pool's idle blocks back and try once more (fragmentation)
        cudaGetLastError();
        cudaStreamSynchronize(stream);
        cudaMemPoolTrimTo(pool, 0);
        e = cudaMallocFromPoolAsync(&p, bytes, pool, stream);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw Error(JUES_ENOMEM, "device allocation of " + std::to_string(bytes) + " bytes failed: " +
                                     cudaGetErrorString(e));
    }
    mem_used += bytes;
    return p;
}

void Ctx::free(void *p, size_t bytes) {
    if (!p) return;
    pack_cache_forget(this, p, bytes);
    cudaFreeAsync(p, stream);   // reusable by later work on this stream once its readers are done
    mem_used -= bytes;
}

void *Ctx::splitk_scratch(size_t bytes) {
    if (bytes > splitk_bytes) {
        // stream-ordered: launches queued before still read the old buffer before it is reused
        free(splitk_ws, splitk_bytes);
        splitk_ws = nullptr;
        splitk_bytes = 0;
        const size_t grown = std::max(bytes, (size_t)16 << 20);
        splitk_ws = alloc(grown);
        splitk_bytes = grown;
    }
    return splitk_ws;
}

Ctx::Scope::Scope(Ctx *c_, const char *name) : c(c_) {
    c->count_launch();
    nvtxRangePushA(name);   // lets a profiler select launches by name
    if (!c->profiling) return;
    r = &c->prof[name];
    if (!r->pool.empty()) {
        ev = r->pool.back();
        r->pool.pop_back();
    } else {
        JUES_CHECK_CUDA(cudaEventCreate(&ev.first));
        JUES_CHECK_CUDA(cudaEventCreate(&ev.second));
    }
    JUES_CHECK_CUDA(cudaEventRecord(ev.first, c->stream));
}

Ctx::Scope::~Scope() {
    nvtxRangePop();
    if (!r) return;
    cudaEventRecord(ev.second, c->stream);
    r->pending.push_back(ev);
    r->launches += 1;
}

static double wall_ms() {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

Ctx::HostPhase::HostPhase(Ctx *c_, const char *n) : c(c_), name(n) {
    if (!c->profiling) return;
    cudaStreamSynchronize(c->stream);
    t0 = wall_ms();
}

Ctx::HostPhase::~HostPhase() {
    if (!c->profiling) return;
    cudaStreamSynchronize(c->stream);
    ProfRec &r = c->prof[name];
    r.total_ms += wall_ms() - t0;
    r.launches += 1;
}

void Ctx::flush_profile() {
    for (auto &kv : prof) {
        ProfRec &r = kv.second;
        for (auto &e : r.pending) {
            cudaEventSynchronize(e.second);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e.first, e.second);
            r.total_ms += ms;
            r.pool.push_back(e);
        }
        r.pending.clear();
    }
}

void Ctx::check_flags() {
    unsigned h = 0;
    JUES_CHECK_CUDA(cudaMemcpyAsync(&h, d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost, stream));
    JUES_CHECK_CUDA(cudaStreamSynchronize(stream));
    if (h) {
        JUES_CHECK_CUDA(cudaMemsetAsync(d_flags, 0, 4 * sizeof(unsigned), stream));
        if (h & FLAG_TIMEOUT)
            throw Error(JUES_ETIMEOUT, "a bounded device-side wait expired; the kernel returned early");
        if (h & FLAG_NONFINITE) throw Error(JUES_ENONFINITE, "non-finite value detected on the device");
    }
}

}  // namespace jues
