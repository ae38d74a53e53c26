// Page-locked storage for tree coefficients (no reference counterpart: MRCPP's
// trees live in pageable chunk allocators on the host, src/trees/NodeAllocator.cpp).
//
// Whole-tree copies between host and device (the input upload of an apply,
// the result download) run as direct DMA when the host side is page-locked;
// from pageable memory the driver copies through staging buffers at a fraction
// of the link rate.  Tree coefficient vectors (CoefVector) therefore take
// blocks of at least kMinBytes from cudaHostAlloc.  Blocks a vector gives back
// stay in a cache, keyed by size, so the trees an apply creates and drops
// every call (outputs, growing vectors) reuse them instead of pinning pages
// again; beyond kCacheBytes of idle blocks the rest are returned to the driver.
// Where page-locked memory cannot be had (no device, MWH_PAGEABLE=1) every
// request is declined and the C heap serves.
#include <cuda_runtime.h>

#include <cstdlib>
#include <map>
#include <mutex>
#include <unordered_map>

#include "mw_host.h"
#include "mwhost.h"

namespace mwh {
namespace {

constexpr size_t kMinBytes = size_t(4) << 20;
constexpr size_t kCacheBytes = size_t(24) << 30;

struct PinnedBlocks {
    std::mutex mu;
    int state = 0;  // 0 unknown, 1 page-locked memory available, -1 declined
    std::multimap<size_t, void *> idle;
    std::unordered_map<void *, size_t> live;
    size_t idle_bytes = 0, live_bytes = 0;
};

// never destroyed: blocks may be released during static destruction, after
// which the CUDA runtime must not be called
PinnedBlocks &blocks() {
    static PinnedBlocks *b = new PinnedBlocks();
    return *b;
}

}  // namespace

size_t host_block_min() { return kMinBytes; }

void *host_block_alloc(size_t bytes) {
    PinnedBlocks &b = blocks();
    std::lock_guard<std::mutex> lk(b.mu);
    if (b.state == 0) {
        const char *e = std::getenv("MWH_PAGEABLE");
        b.state = (e && e[0] == '1') ? -1 : 1;
    }
    if (b.state < 0) return nullptr;
    // an idle block of the size, or up to a quarter larger
    auto it = b.idle.lower_bound(bytes);
    if (it != b.idle.end() && it->first <= bytes + bytes / 4) {
        void *p = it->second;
        const size_t sz = it->first;
        b.idle.erase(it);
        b.idle_bytes -= sz;
        b.live[p] = sz;
        b.live_bytes += sz;
        return p;
    }
    void *p = nullptr;
    cudaError_t e = cudaHostAlloc(&p, bytes, cudaHostAllocPortable);
    if (e != cudaSuccess && !b.idle.empty()) {
        // out of page-locked memory: give the idle blocks back and try once more
        for (auto &kv : b.idle) cudaFreeHost(kv.second);
        b.idle.clear();
        b.idle_bytes = 0;
        cudaGetLastError();
        e = cudaHostAlloc(&p, bytes, cudaHostAllocPortable);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        // without a device nothing will be page-locked: stop asking
        if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver || e == cudaErrorInitializationError) b.state = -1;
        return nullptr;
    }
    b.live[p] = bytes;
    b.live_bytes += bytes;
    return p;
}

bool host_block_release(void *p, size_t) {
    PinnedBlocks &b = blocks();
    std::lock_guard<std::mutex> lk(b.mu);
    auto it = b.live.find(p);
    if (it == b.live.end()) return false;
    const size_t sz = it->second;
    b.live.erase(it);
    b.live_bytes -= sz;
    if (b.idle_bytes + sz <= kCacheBytes) {
        b.idle.emplace(sz, p);
        b.idle_bytes += sz;
    } else {
        cudaFreeHost(p);
    }
    return true;
}

}  // namespace mwh

extern "C" int mwh_pinned_stats(unsigned long long *live_bytes, unsigned long long *idle_bytes) {
    mwh::PinnedBlocks &b = mwh::blocks();
    std::lock_guard<std::mutex> lk(b.mu);
    if (live_bytes) *live_bytes = b.live_bytes;
    if (idle_bytes) *idle_bytes = b.idle_bytes;
    return b.state;
}
