// Host-side state behind the C-ABI handles (mwgpu_ctx, mwgpu_oper, mwgpu_tree)
// shared by the translation units that implement include/mwgpu.h.
#pragma once

#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../../include/mwgpu.h"
#include "mwgpu_internal.cuh"

using mwgpu::DevMRA;
using mwgpu::DevOper;
using mwgpu::DevTree;
using mwgpu::LevelStats;
using mwgpu::NodeKey;
using mwgpu::WorkItem;

// Device blocks of trees, cached per context.  Freeing a tree hands its blocks
// back here instead of to cudaFree (which waits for the whole device and
// unmaps): they are reused by later trees once the context's stream has
// passed the last work that may read them, so an apply with host trees in
// and out does not pay for allocation.  Sizes are rounded to 4 classes per
// octave (at most 25% over the request).
struct DevPool {
    std::multimap<size_t, void *> free_blocks;  // class size -> block
    std::unordered_map<void *, size_t> bytes_of;  // every block of the pool
    std::vector<void *> pending;                  // freed, stream work may still read them
    size_t cached = 0;                            // bytes of free_blocks + pending
    size_t limit = size_t(8) << 30;               // cached bytes kept (a quarter of the device, set at init)
};

struct mwgpu_ctx {
    int device = 0;
    int precision = MWGPU_PREC_FP64;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr;
    std::string err;
    int *d_err = nullptr;
    LevelStats *d_stats = nullptr;
    int *d_tc_counter = nullptr;  // chunk counter of the tensor-core contraction
    double *d_proj = nullptr;     // projection: Gaussians, value-to-coefficient map, roots
    long long proj_cap = 0;
    int *d_work = nullptr;
    int *d_wtree = nullptr;  // tree of every work entry (batched levels)
    int work_cap = 0;
    // per-tree arrays of a batched level
    DevTree *d_fs = nullptr, *d_gs = nullptr;
    double *d_gthr = nullptr;
    // per work entry thresholds of levels whose precision is scaled per output node
    double *d_gnode = nullptr;
    long long gnode_cap = 0;
    int trees_cap = 0;
    double *d_nstage = nullptr;  // norms of the computed nodes, staged for the host
    long long nstage_cap = 0;
    // pending GenNode set
    NodeKey *d_pkeys = nullptr;
    int *d_pvals = nullptr;
    int phcap = 0;
    NodeKey *d_plist = nullptr;
    int pcap = 0;
    long long ph_total = 0, pl_total = 0;
    int *d_pcount = nullptr;  // one pending count per tree
    int pcount_cap = 0;
    int *d_list = nullptr;  // parent lists for transforms
    int *d_ltree = nullptr;  // tree of every parent (batched transforms)
    int list_cap = 0;
    cudaEvent_t marks[16] = {};
    // work list of the mixed form
    WorkItem *d_items = nullptr;     // work items in term-major order (what the contraction reads)
    WorkItem *d_items_cm = nullptr;  // the builder's cell-major items (same capacity)
    long long items_cap = 0;
    long long *d_pair_off = nullptr, pair_off_cap = 0;
    // mixed-form GenNode families of a level (gen_pass)
    NodeKey *d_fkeys = nullptr, *d_fam_keys = nullptr;
    int *d_fvals = nullptr, *d_famid = nullptr, *d_fam_slots = nullptr, *d_fam_count = nullptr;
    long long fkeys_cap = 0, fvals_cap = 0, famid_cap = 0, fam_keys_cap = 0, fam_slots_cap = 0, fam_count_cap = 0;
    int *d_pcounts = nullptr;
    long long pcounts_cap = 0;
    long long *d_item_off = nullptr, item_off_cap = 0;
    long long *d_scan = nullptr, scan_cap = 0;
    long long *d_goff = nullptr, goff_cap = 0;
    int4 *d_chunks = nullptr;
    int *d_chunk_begin = nullptr;
    int chunks_cap = 0;
    double *d_partial = nullptr;
    size_t partial_cap = 0;  // doubles
    // pencil contraction (k_pencil.cu): units, task order, task sums, per-entry task ranges
    mwgpu::PencilUnit *d_units = nullptr;
    long long units_cap = 0;
    mwgpu::PencilUnit *h_units = nullptr;  // page-locked staging of the units of a per-call level
    size_t h_units_cap = 0;
    int *d_task_unit = nullptr;
    long long task_unit_cap = 0;
    double *d_pen_partial = nullptr;
    size_t pen_partial_cap = 0;  // doubles
    int *d_pen_begin = nullptr;
    long long pen_begin_cap = 0;
    int *d_keep = nullptr;
    long long keep_cap = 0;
    long long *d_keep_off = nullptr;
    long long keep_off_cap = 0;
    int *d_pen_counter = nullptr;
    unsigned long long launches = 0;
    void *d_arena = nullptr;  // scratch of the judged apply, carved per call
    size_t arena_bytes = 0;
    void *d_scrub = nullptr;
    size_t scrub_bytes = 0;
    DevPool pool;
};

struct mwgpu_oper {
    DevMRA mra{};
    double *d_filt = nullptr;
    DevOper op{};
    std::vector<void *> allocs;
    int n_rows = 0;
    std::vector<int> widths;    // [T * n_rows * 5]
    std::vector<int> band_max;  // [n_rows]
    // pencil contraction (order 7), per configuration c (terms of band width
    // <= kPencilCfgW[c] in the pencil kernel): per depth and k = 0..kPencilMaxL
    // the number of terms with band width >= k among those of width <=
    // kPencilCfgW[c], the term row of the first such term (the wider ones come
    // first), and per (depth, group, x slot) the float offset of the stacked
    // form in op.btc_stack (-1: none) and its number of terms
    struct PenCfg {
        std::vector<int> tk;    // [rows][kPencilMaxL + 1]
        std::vector<int> r0;    // [rows]
        std::vector<long long> form;
        std::vector<short> nform;
    };
    PenCfg pen[mwgpu::kPencilCfgs];
    int pen_groups = 0;
};

struct mwgpu_tree {
    DevMRA mra{};
    double *d_filt = nullptr;
    std::vector<double> h_filt;  // host copy of the filters (batch compatibility check)
    int plans = 0;               // plans that hold this tree (its device arrays must not move)
    DevTree t{};
    std::vector<int4> h_idx;
    std::vector<int> h_child0;
    bool is_input = false;
    int gen_prec = -1;  // precision mode whose GenNode arithmetic made the GenNodes held
};

#define MW_CK(call)                                                                                 \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess) {                                                                    \
            ctx->err = std::string(#call) + ": " + cudaGetErrorString(e_);                          \
            return (e_ == cudaErrorMemoryAllocation) ? MWGPU_ERR_OOM : MWGPU_ERR_DEVICE;            \
        }                                                                                           \
    } while (0)

#define MW_ARG(cond, msg)                     \
    do {                                      \
        if (!(cond)) {                        \
            ctx->err = msg;                   \
            return MWGPU_ERR_BAD_ARG;         \
        }                                     \
    } while (0)


// Phase timing of one entry point, on when the environment sets MWGPU_TRACE:
// every mark drains the stream and adds the host time since the previous
// mark; the line goes to stderr when the call returns.  (Tracing serialises
// the host and the device; the figures attribute time, they are not a
// benchmark.)
struct PhaseTrace {
    mwgpu_ctx *ctx;
    const char *fn;
    bool on;
    std::chrono::steady_clock::time_point t0, last;
    std::string line;
    PhaseTrace(mwgpu_ctx *c, const char *f) : ctx(c), fn(f), on(std::getenv("MWGPU_TRACE") != nullptr) {
        if (on) t0 = last = std::chrono::steady_clock::now();
    }
    void mark(const std::string &phase);
    ~PhaseTrace() {
        if (!on) return;
        const double tot = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        std::fprintf(stderr, "[mwgpu] %s%s total=%.3f ms\n", fn, line.c_str(), tot);
    }
};

inline size_t pool_class(size_t b) {
    if (b <= 4096) return 4096;
    const int e = 63 - __builtin_clzll((unsigned long long)b);  // 2^e <= b < 2^(e+1)
    const size_t q = (size_t)1 << (e - 2);
    return (b + q - 1) / q * q;
}

// all cached blocks back to the device (after the stream has drained)
inline void pool_trim(mwgpu_ctx *ctx) {
    DevPool &pl = ctx->pool;
    cudaStreamSynchronize(ctx->stream);
    for (void *q : pl.pending) pl.free_blocks.emplace(pl.bytes_of[q], q);
    pl.pending.clear();
    for (auto &kv : pl.free_blocks) {
        cudaFree(kv.second);
        pl.bytes_of.erase(kv.second);
    }
    pl.free_blocks.clear();
    pl.cached = 0;
}

inline mwgpu_status pool_alloc_bytes(mwgpu_ctx *ctx, void **p, size_t bytes) {
    DevPool &pl = ctx->pool;
    *p = nullptr;
    if (!pl.pending.empty()) {
        MW_CK(cudaStreamSynchronize(ctx->stream));
        for (void *q : pl.pending) pl.free_blocks.emplace(pl.bytes_of[q], q);
        pl.pending.clear();
    }
    const size_t c = pool_class(bytes);
    auto it = pl.free_blocks.find(c);
    if (it != pl.free_blocks.end()) {
        *p = it->second;
        pl.free_blocks.erase(it);
        pl.cached -= c;
        return MWGPU_OK;
    }
    cudaError_t e = cudaMalloc(p, c);
    if (e == cudaErrorMemoryAllocation && pl.cached > 0) {
        cudaGetLastError();
        pool_trim(ctx);
        e = cudaMalloc(p, c);
    }
    MW_CK(e);
    pl.bytes_of[*p] = c;
    return MWGPU_OK;
}

template <class T> inline mwgpu_status pool_alloc(mwgpu_ctx *ctx, T **p, size_t n) {
    void *v = nullptr;
    const mwgpu_status s = pool_alloc_bytes(ctx, &v, sizeof(T) * (n == 0 ? 1 : n));
    *p = (T *)v;
    return s;
}

// a block of the pool goes back to it (reusable after the next stream
// drain); any other pointer is freed
inline void pool_free(mwgpu_ctx *ctx, void *p) {
    if (!p) return;
    DevPool &pl = ctx->pool;
    auto it = pl.bytes_of.find(p);
    if (it == pl.bytes_of.end()) {
        cudaFree(p);
        return;
    }
    pl.pending.push_back(p);
    pl.cached += it->second;
    if (pl.cached > pl.limit) pool_trim(ctx);
}

inline void PhaseTrace::mark(const std::string &phase) {
    if (!on) return;
    cudaStreamSynchronize(ctx->stream);
    const auto now = std::chrono::steady_clock::now();
    char buf[96];
    std::snprintf(buf, sizeof(buf), " %s=%.3f", phase.c_str(), std::chrono::duration<double, std::milli>(now - last).count());
    line += buf;
    last = now;
}

template <class T> inline mwgpu_status dev_alloc(mwgpu_ctx *ctx, T **p, size_t n) {
    *p = nullptr;
    if (n == 0) n = 1;
    MW_CK(cudaMalloc((void **)p, sizeof(T) * n));
    return MWGPU_OK;
}

