// slm.cpp — host side of libslm: the C ABI declared in include/slm.h.
//
// Contexts own a stream and an HBM budget; stores hold device-resident
// descriptors laid out for the kernels; plans turn a list of image pairs into
// work items, scratch buffers and a captured CUDA graph. The single-pair entry
// points (the ratio_match drop-in) run through a pool of workspaces so that
// concurrent host threads (rayon workers in the reference) never share one.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <tuple>
#include <vector>

#include "slm.h"
#include "slm_internal.h"
#include "slm_shortlist.h"

using namespace slm;

namespace {

thread_local std::string g_last_error;

slm_status fail(slm_status s, const std::string &msg) {
    g_last_error = msg;
    return s;
}

#define SLM_CU(call)                                                                                   \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess) {                                                                       \
            if (e_ == cudaErrorMemoryAllocation) return fail(SLM_OOM, std::string(#call) + ": out of memory"); \
            return fail(SLM_CUDA_ERROR, std::string(#call) + ": " + cudaGetErrorString(e_));           \
        }                                                                                              \
    } while (0)

#define SLM_TRY(expr)                \
    do {                             \
        slm_status s_ = (expr);      \
        if (s_ != SLM_OK) return s_; \
    } while (0)

uint64_t pad_rows(uint64_t n) { return (n + kTile - 1) / kTile * kTile; }

// Timing events: under stream capture they must become event-record nodes
// (cudaEventRecordExternal); outside capture the flag is not allowed.
cudaError_t record_event(cudaEvent_t e, cudaStream_t s) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t r = cudaStreamIsCapturing(s, &cs);
    if (r != cudaSuccess) return r;
    return cs == cudaStreamCaptureStatusActive ? cudaEventRecordWithFlags(e, s, cudaEventRecordExternal)
                                               : cudaEventRecord(e, s);
}

}  // namespace

// ------------------------------------------------------------------ context

struct Workspace;
struct Coalescer;
// Coalescing of concurrent single-pair calls (defined with the serving code).
void coalescer_destroy(slm_ctx *c);
slm_status coalesce_call(slm_ctx *c, const float *a, uint32_t na, const float *b, uint32_t nb, float ratio,
                         int mutual, slm_pair *out, uint32_t cap, uint32_t *n_out, slm_stats *st);

struct slm_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int sms = 0;
    // Kernels may read pageable host memory directly (address translation over
    // the CPU-GPU link, as on Grace-based GB300 systems): single-pair inputs are
    // then read by the packing kernels where they lie instead of being copied.
    bool host_direct = false;
    Coalescer *coal = nullptr;  // set by slm_ctx_set_coalescing
    uint64_t budget = 0;
    std::atomic<uint64_t> used{0};
    std::mutex mu;
    std::vector<Workspace *> idle;  // single-pair workspaces not in use
    std::vector<Workspace *> all;
    std::map<uint64_t, slm_tune> tuned;  // autotuned settings by batch shape

    slm_status alloc(void **p, size_t bytes) {
        *p = nullptr;
        if (bytes == 0) return SLM_OK;
        uint64_t now = used.fetch_add(bytes) + bytes;
        if (budget && now > budget) {
            used.fetch_sub(bytes);
            return fail(SLM_OOM, "HBM budget exceeded: need " + std::to_string(now) + " > budget " +
                                     std::to_string(budget) + " bytes");
        }
        cudaError_t e = cudaMalloc(p, bytes);
        if (e != cudaSuccess) {
            used.fetch_sub(bytes);
            cudaGetLastError();
            return fail(SLM_OOM, std::string("cudaMalloc(") + std::to_string(bytes) + "): " + cudaGetErrorString(e));
        }
        return SLM_OK;
    }
    void release(void *p, size_t bytes) {
        if (!p) return;
        cudaFree(p);
        used.fetch_sub(bytes);
    }
    // Stream-ordered allocations from the context's pool, for buffers that one
    // stream uses (a plan's): freeing one orders after that stream's earlier
    // work instead of synchronising the device as cudaFree does, so a plan that
    // grows does not stall the work of other streams (serving slots).
    cudaMemPool_t pool = nullptr;
    slm_status alloc_ordered(void **p, size_t bytes, cudaStream_t s) {
        *p = nullptr;
        if (bytes == 0) return SLM_OK;
        uint64_t now = used.fetch_add(bytes) + bytes;
        if (budget && now > budget) {
            used.fetch_sub(bytes);
            return fail(SLM_OOM, "HBM budget exceeded: need " + std::to_string(now) + " > budget " +
                                     std::to_string(budget) + " bytes");
        }
        cudaError_t e = cudaMallocFromPoolAsync(p, bytes, pool, s);
        if (e != cudaSuccess) {
            used.fetch_sub(bytes);
            cudaGetLastError();
            *p = nullptr;
            return fail(SLM_OOM, std::string("cudaMallocFromPoolAsync(") + std::to_string(bytes) +
                                     "): " + cudaGetErrorString(e));
        }
        return SLM_OK;
    }
    void release_ordered(void *p, size_t bytes, cudaStream_t s) {
        if (!p) return;
        cudaFreeAsync(p, s);
        used.fetch_sub(bytes);
    }
};

// A named range on the calling thread for profilers that read NVTX (nsys,
// ncu's range filters); without such a tool attached the calls return at once.
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// Device buffer owned by a context, grown on demand.
struct DevBuf {
    slm_ctx *ctx = nullptr;
    void *p = nullptr;
    size_t bytes = 0;
    cudaStream_t ord = nullptr;  // set: allocated from the context's pool, ordered on this stream
    bool pooled = false;         // p came from the pool
    // Owners whose buffer one stream uses call this before ensure().
    void order_on(cudaStream_t s) {
        if (s == ord) return;
        if (p && pooled) cudaStreamSynchronize(ord);  // the old stream's work is done before a later free
        ord = s;
    }
    slm_status ensure(slm_ctx *c, size_t need) {
        ctx = c;
        if (need <= bytes) return SLM_OK;
        free_();
        size_t want = need + need / 4;
        if (ord && ctx->pool)
            SLM_TRY(ctx->alloc_ordered(&p, want, ord));
        else
            SLM_TRY(ctx->alloc(&p, want));
        pooled = ord && ctx->pool;
        bytes = want;
        return SLM_OK;
    }
    void free_() {
        if (ctx && p) {
            if (pooled)
                ctx->release_ordered(p, bytes, ord);
            else
                ctx->release(p, bytes);
        }
        p = nullptr;
        bytes = 0;
        pooled = false;
    }
    void reset() { free_(); }
    template <class T>
    T *as() const {
        return static_cast<T *>(p);
    }
    ~DevBuf() { reset(); }
};

extern "C" const char *slm_status_str(slm_status s) {
    switch (s) {
        case SLM_OK: return "SLM_OK";
        case SLM_INVALID_ARG: return "SLM_INVALID_ARG";
        case SLM_CAPACITY: return "SLM_CAPACITY";
        case SLM_OOM: return "SLM_OOM";
        case SLM_CUDA_ERROR: return "SLM_CUDA_ERROR";
        case SLM_TIMEOUT: return "SLM_TIMEOUT";
        case SLM_NO_DEVICE: return "SLM_NO_DEVICE";
        case SLM_INTERNAL: return "SLM_INTERNAL";
        case SLM_CANCELLED: return "SLM_CANCELLED";
    }
    return "SLM_UNKNOWN";
}

extern "C" const char *slm_last_error(void) { return g_last_error.c_str(); }

void slm::set_last_error(const char *msg) { g_last_error = msg ? msg : ""; }

// --------------------------------------------------------------------- store

struct slm_store {
    slm_ctx *ctx = nullptr;
    uint64_t max_rows = 0;  // padded rows
    uint32_t max_views = 0;
    DevBuf raw;             // row-major FP32, padded rows per view
    DevBuf tiled;           // FP32 tiles [slot][row]
    std::vector<uint32_t> row0, n;
    uint64_t rows_used = 0;
    uint64_t version = 0;   // bumps when views are added or cleared
    uint64_t epoch = 0;                      // bumps on clear
    // Low-precision operand images for the shortlist path, [0] BF16 and [1]
    // FP8 (an FP8 plan also reads the BF16 image: pairs the FP8 bound cannot
    // settle are rescued by the BF16 passes). Each is built lazily: only the
    // views appended since its last build, all of them after a clear.
    struct LowpImage {
        uint64_t version = ~0ull, epoch = ~0ull;
        size_t views = 0;                    // views whose images are built
        DevBuf optiles, norms, qscale, vstats;
    } lowp[2];
    uint64_t fp32_epoch = ~0ull;             // FP32 tiles, built lazily the same way
    size_t fp32_views = 0;
    DevBuf tiletab;                          // {row0, n, tile, view} per tile to pack
    DevBuf staging;                          // slm_store_add_views: the host rows, before the scatter
};

// ---------------------------------------------------------------------- plan

struct slm_plan {
    slm_ctx *ctx = nullptr;
    slm_store *st = nullptr;
    uint32_t np = 0;
    float ratio = 0.8f;
    int mutual = 1;
    slm_precision prec = SLM_PREC_FP32;
    slm_tune tune{};
    cudaStream_t stream = nullptr;   // all uploads and launches of this plan
    std::vector<PairMeta> meta;
    std::vector<Item> items;
    std::vector<uint64_t> slot_off;  // np + 1
    uint64_t n_parts = 0, n_cols = 0, n_slots = 0, distances = 0;
    DevBuf d_meta, d_items, d_parts, d_colbest, d_slots, d_counts, d_ctl, d_offsets, d_dense;
    // shortlist path
    std::vector<SlItem> sitems;
    std::vector<SlPair> spairs;
    uint32_t half_recs = kSlHalfRecs;  // records per candidate row and column half
    uint64_t rows_pad = 0, cand_rows_pad = 0, cols_pad = 0, sl_parts = 0, queue_cap = 0, xitem_cap = 0, row_blocks_total = 0;
    uint32_t row_blocks = 1;  // the most row blocks of any pair
    DevBuf d_sitems, d_spairs, d_rowpart, d_rownear, d_colmin, d_rowthr, d_colthr, d_rowcnt, d_rowrec, d_rowrecj, d_colcnt,
        d_rowdec, d_queue, d_rqueue, d_dump, d_xlist, d_xitems, d_xparts, d_blkcnt, d_pairctl;
    bool dump = false;
    uint32_t min_matches = 0;        // pairs with fewer matches report none
    cudaGraphExec_t exec = nullptr;
    cudaGraph_t graph = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;  // bracket the main kernel(s)
    cudaEvent_t evp[3] = {nullptr, nullptr, nullptr};  // shortlist: after pass 1, mid, pass 2
    uint64_t kernels = 0;                      // kernels per launch
    void *graph_optiles[2] = {nullptr, nullptr};  // store buffers the captured graph reads
    void *graph_tiled = nullptr;
    bool launched = false;
    ~slm_plan() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        for (cudaEvent_t &e : evp)
            if (e) cudaEventDestroy(e);
    }
};

// Every device buffer of a plan: all are used on the plan's stream only, and
// allocated ordered on it (DevBuf::order_on).
std::array<DevBuf *, 29> plan_buffers(slm_plan *p) {
    return {&p->d_meta, &p->d_items, &p->d_parts, &p->d_colbest, &p->d_slots, &p->d_counts, &p->d_ctl,
            &p->d_offsets, &p->d_dense, &p->d_sitems, &p->d_spairs, &p->d_rowpart, &p->d_rownear,
            &p->d_colmin, &p->d_rowthr, &p->d_colthr, &p->d_rowcnt, &p->d_rowrec, &p->d_rowrecj,
            &p->d_colcnt, &p->d_rowdec, &p->d_queue, &p->d_rqueue, &p->d_dump, &p->d_xlist, &p->d_xitems,
            &p->d_xparts, &p->d_blkcnt, &p->d_pairctl};
}
// Frees a plan's buffers while its stream still exists (their frees are
// ordered on it): owners call it before destroying that stream.
void plan_release(slm_plan *p) {
    for (DevBuf *b : plan_buffers(p)) b->reset();
}

// Dense compaction of per-pair slots (device) into out + offsets.
namespace slm {
void launch_fill_u32(uint32_t *p, uint64_t n, uint32_t v, cudaStream_t s);
void launch_scatter_rows(const uint4 *tab, uint32_t n, const float *src, float *dst, cudaStream_t s);
// Each view's rows from its own 16-byte-aligned source address: {addr lo, addr hi, store row, rows}.
void launch_gather_rows(const uint4 *tab, uint32_t n, float *dst, cudaStream_t s);
void launch_filter_counts(uint32_t *counts, uint32_t np, uint32_t min_matches, cudaStream_t s);
void launch_scan_counts(const uint32_t *counts, uint32_t np, uint64_t *offsets, cudaStream_t s);
void launch_gather(const uint2 *slots, const uint64_t *slot_off, const uint32_t *counts, const uint64_t *offsets,
                   uint32_t np, uint2 *dense, uint64_t cap, cudaStream_t s);
}  // namespace slm

namespace {

// Plan the exact-path work items: one per (pair, 128-row tile, column chunk).
// Columns are split only when the batch has too few row tiles to fill the GPU.
void plan_items(slm_plan *p) {
    const slm_store *st = p->st;
    uint64_t row_tiles = 0;
    for (uint32_t k = 0; k < p->np; ++k) row_tiles += (p->meta[k].na + kTile - 1) / kTile;
    const uint64_t want = (uint64_t)std::max(1, p->ctx->sms) * (p->tune.items_per_sm ? p->tune.items_per_sm : 4);
    uint32_t split = 1;
    if (row_tiles && row_tiles < want) split = (uint32_t)((want + row_tiles - 1) / row_tiles);
    p->items.clear();
    uint32_t part = 0;
    for (uint32_t k = 0; k < p->np; ++k) {
        PairMeta &m = p->meta[k];
        const uint32_t rt_n = (m.na + kTile - 1) / kTile;
        const uint32_t ct_n = (m.nb + kTile - 1) / kTile;
        uint32_t chunks = std::max(1u, std::min(split, ct_n));
        m.nchunk = chunks;
        m.part_base = part;
        for (uint32_t rt = 0; rt < rt_n; ++rt)
            for (uint32_t c = 0; c < chunks; ++c) {
                Item it{};
                it.pair = k;
                it.rt = rt;
                it.ct0 = (uint32_t)((uint64_t)ct_n * c / chunks);
                it.ct1 = (uint32_t)((uint64_t)ct_n * (c + 1) / chunks);
                it.part = part + rt * chunks + c;
                p->items.push_back(it);
            }
        part += rt_n * chunks;
        (void)st;
    }
    p->n_parts = part;
    // Longest items first (cost ~ rows x columns) for the dynamic queue.
    std::stable_sort(p->items.begin(), p->items.end(), [&](const Item &x, const Item &y) {
        const uint64_t cx = (uint64_t)(x.ct1 - x.ct0), cy = (uint64_t)(y.ct1 - y.ct0);
        return cx > cy;
    });
}

// Shortlist plan: items of up to two 128-row a tiles against a range of
// 128-column b tiles; per-row and per-column arrays padded to 128 entries per
// pair so that every bulk copy starts on a 512-byte boundary.
slm_status plan_build_shortlist(slm_plan *p, const slm_pair *pairs) {
    slm_ctx *c = p->ctx;
    uint64_t supers = 0;
    for (uint32_t k = 0; k < p->np; ++k)
        if (p->meta[k].nb) supers += (p->meta[k].na + 2 * kTile - 1) / (2 * kTile);
    const uint64_t want = (uint64_t)std::max(1, c->sms) * (p->tune.items_per_sm ? p->tune.items_per_sm : 3);
    uint32_t split = 1;
    if (supers && supers < want) split = (uint32_t)((want + supers - 1) / supers);
    p->sitems.clear();
    p->spairs.assign(p->np, SlPair{});
    uint64_t rb = 0, cb = 0, part = 0, row_tiles = 0, blk = 0, crb = 0;
    p->row_blocks = 1;
    for (uint32_t k = 0; k < p->np; ++k) {
        const PairMeta &m = p->meta[k];
        SlPair &sp = p->spairs[k];
        row_tiles += (m.na + kTile - 1) / kTile;
        // row blocks of the per-pair kernels after pass 1
        sp.blk = (uint32_t)blk;
        blk += (m.na + kSlRowBlock - 1) / kSlRowBlock;
        p->row_blocks = std::max(p->row_blocks, (std::max(m.na, m.nb) + kSlRowBlock - 1) / kSlRowBlock);
        sp.rbase = (uint32_t)rb;
        sp.cbase = (uint32_t)cb;
        sp.view_a = pairs[k].i;
        sp.view_b = pairs[k].j;
        const uint32_t rt_n = (m.na + kTile - 1) / kTile, ct_n = (m.nb + kTile - 1) / kTile;
        const uint32_t chunks = std::max(1u, std::min(std::min(split, ct_n), kSlMaxRanges));
        sp.nchunk = chunks;
        sp.part_base = (uint32_t)part;
        sp.crbase = (uint32_t)crb;
        crb += pad_rows(m.na) * chunks;  // one pair of S lists per row and column range
        if (m.na && m.nb) {
            // row_tiles == 1: one 128-row a tile per item (M = 128 per CTA)
            const uint32_t per = p->tune.row_tiles == 1 ? 1u : 2u;
            const uint32_t ns = (rt_n + 1) / 2;
            for (uint32_t s2 = 0; s2 < ns; ++s2)
                for (uint32_t half = 0; half < 2 / per; ++half)
                for (uint32_t ch = 0; ch < chunks; ++ch) {
                    SlItem it{};
                    const uint32_t rt0 = 2 * s2 + half;
                    if (rt0 >= rt_n) continue;
                    it.nat = std::min(per, rt_n - rt0);
                    it.pair[0] = it.pair[1] = k;
                    it.rt[0] = rt0;
                    it.rt[1] = rt0 + 1;
                    it.part[0] = it.part[1] = (uint32_t)(part + s2 * chunks + ch);
                    it.ct0 = (uint32_t)((uint64_t)ct_n * ch / chunks);
                    it.ct1 = (uint32_t)((uint64_t)ct_n * (ch + 1) / chunks);
                    if (it.ct1 > it.ct0) p->sitems.push_back(it);
                }
            part += (uint64_t)ns * chunks;
        }
        rb += pad_rows(m.na);
        cb += pad_rows(m.nb);
    }
    if (rb >= (1ull << 32) || cb >= (1ull << 32) || crb >= (1ull << 31))
        return fail(SLM_CAPACITY, "batch too large for one plan");
    // The last row tile of a pair with an odd tile count makes a one-tile item,
    // which leaves half of the epilogue warps idle. Two such tiles of pairs
    // with the same b view and column range share one item.
    if (p->tune.row_tiles != 1) {
        std::map<std::tuple<uint32_t, uint32_t, uint32_t>, size_t> open;  // (b view, ct0, ct1) -> waiting item
        std::vector<SlItem> merged;
        merged.reserve(p->sitems.size());
        std::vector<bool> gone(p->sitems.size(), false);
        for (size_t x = 0; x < p->sitems.size(); ++x) {
            const SlItem &it = p->sitems[x];
            if (it.nat != 1) continue;
            const auto key = std::make_tuple(p->spairs[it.pair[0]].view_b, it.ct0, it.ct1);
            auto f = open.find(key);
            if (f == open.end()) {
                open.emplace(key, x);
                continue;
            }
            SlItem &w = p->sitems[f->second];  // the waiting tile becomes tile 0
            w.nat = 2;
            w.pair[1] = it.pair[0];
            w.rt[1] = it.rt[0];
            w.part[1] = it.part[0];
            gone[x] = true;
            open.erase(f);
        }
        for (size_t x = 0; x < p->sitems.size(); ++x)
            if (!gone[x]) merged.push_back(p->sitems[x]);
        p->sitems.swap(merged);
    }
    std::stable_sort(p->sitems.begin(), p->sitems.end(), [](const SlItem &x, const SlItem &y) {
        return (uint64_t)(x.ct1 - x.ct0) * x.nat > (uint64_t)(y.ct1 - y.ct0) * y.nat;
    });
    p->rows_pad = rb + 2 * kTile;
    p->cand_rows_pad = crb + 2 * kTile;
    p->cols_pad = cb + kTile;
    p->sl_parts = std::max<uint64_t>(part, 1);
    p->queue_cap = std::max<uint64_t>(p->n_slots, 1) + 64;
    // pairs routed to the exact kernel: at most (row tiles) + (4 x SMs) items
    p->xitem_cap = row_tiles + 4ull * (uint64_t)std::max(1, c->sms);
    if (p->xitem_cap >= (1ull << 32)) return fail(SLM_CAPACITY, "batch too large for one plan");
    SLM_TRY(p->d_sitems.ensure(c, sizeof(SlItem) * std::max<size_t>(1, p->sitems.size())));
    SLM_TRY(p->d_spairs.ensure(c, sizeof(SlPair) * std::max<size_t>(1, p->np)));
    SLM_TRY(p->d_rowpart.ensure(c, sizeof(float2) * 256 * p->sl_parts));
    SLM_TRY(p->d_rownear.ensure(c, sizeof(uint32_t) * 256 * p->sl_parts));
    p->row_blocks_total = blk;
    SLM_TRY(p->d_blkcnt.ensure(c, sizeof(uint32_t) * std::max<uint64_t>(1, blk)));
    SLM_TRY(p->d_pairctl.ensure(c, 4 * sizeof(uint32_t) * std::max<size_t>(1, p->np)));
    SLM_TRY(p->d_xlist.ensure(c, sizeof(uint32_t) * std::max<size_t>(1, p->np)));
    SLM_TRY(p->d_xitems.ensure(c, sizeof(Item) * p->xitem_cap));
    SLM_TRY(p->d_xparts.ensure(c, sizeof(RowPart) * kTile * p->xitem_cap));
    SLM_TRY(p->d_colbest.ensure(c, sizeof(unsigned long long) * std::max<uint64_t>(1, p->n_cols)));
    SLM_TRY(p->d_colmin.ensure(c, sizeof(uint32_t) * p->cols_pad));
    SLM_TRY(p->d_rowthr.ensure(c, sizeof(float) * p->rows_pad));
    SLM_TRY(p->d_colthr.ensure(c, sizeof(float) * p->cols_pad));
    SLM_TRY(p->d_rowcnt.ensure(c, 2 * sizeof(uint32_t) * p->cand_rows_pad));
    p->half_recs = p->tune.shortlist_k ? p->tune.shortlist_k : kSlHalfRecs;
    SLM_TRY(p->d_rowrec.ensure(c, sizeof(float4) * 2 * p->half_recs * p->cand_rows_pad));
    SLM_TRY(p->d_rowrecj.ensure(c, sizeof(uint32_t) * 2 * p->half_recs * p->cand_rows_pad));
    SLM_TRY(p->d_colcnt.ensure(c, sizeof(uint32_t) * p->cols_pad));
    SLM_TRY(p->d_rowdec.ensure(c, sizeof(uint32_t) * p->rows_pad));
    SLM_TRY(p->d_queue.ensure(c, sizeof(SlQueue) * p->queue_cap));
    SLM_TRY(p->d_rqueue.ensure(c, sizeof(SlQueue) * p->queue_cap));
    if (p->dump && p->np) SLM_TRY(p->d_dump.ensure(c, sizeof(float) * std::max<uint64_t>(1, (uint64_t)p->meta[0].na * p->meta[0].nb)));
    SLM_TRY(p->d_meta.ensure(c, sizeof(PairMeta) * std::max<size_t>(1, p->np)));
    SLM_TRY(p->d_slots.ensure(c, sizeof(uint2) * std::max<uint64_t>(1, p->n_slots)));
    SLM_TRY(p->d_counts.ensure(c, sizeof(uint32_t) * std::max<size_t>(1, p->np)));
    SLM_TRY(p->d_ctl.ensure(c, 64));
    SLM_TRY(p->d_offsets.ensure(c, sizeof(uint64_t) * (p->np + 1) * 2));
    SLM_TRY(p->d_dense.ensure(c, sizeof(uint2) * std::max<uint64_t>(1, p->n_slots)));
    cudaStream_t s = p->stream;
    SLM_CU(cudaMemcpyAsync(p->d_meta.p, p->meta.data(), sizeof(PairMeta) * p->np, cudaMemcpyHostToDevice, s));
    SLM_CU(cudaMemcpyAsync(p->d_offsets.as<uint64_t>() + (p->np + 1), p->slot_off.data(),
                           sizeof(uint64_t) * (p->np + 1), cudaMemcpyHostToDevice, s));
    SLM_CU(cudaMemcpyAsync(p->d_spairs.p, p->spairs.data(), sizeof(SlPair) * p->np, cudaMemcpyHostToDevice, s));
    SLM_CU(cudaMemcpyAsync(p->d_sitems.p, p->sitems.data(), sizeof(SlItem) * p->sitems.size(),
                           cudaMemcpyHostToDevice, s));
    return SLM_OK;
}

slm_status plan_build(slm_plan *p, const slm_pair *pairs) {
    slm_store *st = p->st;
    p->meta.resize(p->np);
    p->slot_off.assign(p->np + 1, 0);
    uint64_t col = 0, slot = 0, dist = 0;
    for (uint32_t k = 0; k < p->np; ++k) {
        const uint32_t u = pairs[k].i, v = pairs[k].j;
        if (u >= st->row0.size() || v >= st->row0.size())
            return fail(SLM_INVALID_ARG, "pair " + std::to_string(k) + " names a view not in the store");
        PairMeta &m = p->meta[k];
        m.a_row0 = st->row0[u];
        m.b_row0 = st->row0[v];
        m.na = st->n[u];
        m.nb = st->n[v];
        m.col_base = col;
        m.slot_off = slot;
        p->slot_off[k] = slot;
        col += m.nb;
        slot += m.na;
        dist += (uint64_t)m.na * m.nb;
    }
    p->slot_off[p->np] = slot;
    p->n_cols = col;
    p->n_slots = slot;
    p->distances = dist;
    if (p->prec != SLM_PREC_FP32) return plan_build_shortlist(p, pairs);
    plan_items(p);
    slm_ctx *c = p->ctx;
    SLM_TRY(p->d_meta.ensure(c, sizeof(PairMeta) * std::max<size_t>(1, p->np)));
    SLM_TRY(p->d_colbest.ensure(c, sizeof(unsigned long long) * std::max<uint64_t>(1, col)));
    SLM_TRY(p->d_slots.ensure(c, sizeof(uint2) * std::max<uint64_t>(1, slot)));
    SLM_TRY(p->d_counts.ensure(c, sizeof(uint32_t) * std::max<size_t>(1, p->np)));
    SLM_TRY(p->d_ctl.ensure(c, 64));
    SLM_TRY(p->d_offsets.ensure(c, sizeof(uint64_t) * (p->np + 1) * 2));
    SLM_TRY(p->d_dense.ensure(c, sizeof(uint2) * std::max<uint64_t>(1, slot)));
    cudaStream_t s = p->stream;
    SLM_CU(cudaMemcpyAsync(p->d_meta.p, p->meta.data(), sizeof(PairMeta) * p->np, cudaMemcpyHostToDevice, s));
    // slot offsets live in the second half of d_offsets
    SLM_CU(cudaMemcpyAsync(p->d_offsets.as<uint64_t>() + (p->np + 1), p->slot_off.data(),
                           sizeof(uint64_t) * (p->np + 1), cudaMemcpyHostToDevice, s));
    SLM_TRY(p->d_items.ensure(c, sizeof(Item) * std::max<size_t>(1, p->items.size())));
    SLM_TRY(p->d_parts.ensure(c, sizeof(RowPart) * kTile * std::max<uint64_t>(1, p->n_parts)));
    SLM_CU(cudaMemcpyAsync(p->d_items.p, p->items.data(), sizeof(Item) * p->items.size(), cudaMemcpyHostToDevice, s));
    return SLM_OK;
}

// Enqueue the whole batch on stream s (also used for graph capture).
slm_status plan_enqueue(slm_plan *p, cudaStream_t s) {
    uint32_t *ctl = p->d_ctl.as<uint32_t>();  // [0] work counter, [1] error word, [2..] shortlist counters
    SLM_CU(cudaMemsetAsync(ctl, 0, 64, s));
    if (p->prec != SLM_PREC_FP32) {
        slm_store *st = p->st;
        launch_fill_u32(p->d_colmin.as<uint32_t>(), p->cols_pad, 0xff800000u, s);  // encodes +inf
        SLM_CU(cudaMemsetAsync(p->d_rowcnt.p, 0, 2 * sizeof(uint32_t) * p->cand_rows_pad, s));
        SLM_CU(cudaMemsetAsync(p->d_colcnt.p, 0, sizeof(uint32_t) * p->cols_pad, s));
        SLM_CU(cudaMemsetAsync(p->d_pairctl.p, 0, 4 * sizeof(uint32_t) * p->np, s));
        SLM_CU(cudaMemsetAsync(p->d_counts.p, 0, sizeof(uint32_t) * p->np, s));  // compact adds its blocks
        SlArgs a{};
        const slm_store::LowpImage &im = st->lowp[p->prec == SLM_PREC_FP8 ? 1 : 0];
        a.optiles = im.optiles.as<uint8_t>();
        a.norms = im.norms.as<float>();
        a.raw = st->raw.as<float>();
        a.qscale = p->prec == SLM_PREC_FP8 ? im.qscale.as<float>() : nullptr;
        a.vstats = im.vstats.as<ViewStat>();
        a.pairs = p->d_meta.as<PairMeta>();
        a.spairs = p->d_spairs.as<SlPair>();
        a.npairs = p->np;
        a.items = p->d_sitems.as<SlItem>();
        a.n_items = (uint32_t)p->sitems.size();
        a.rowpart = p->d_rowpart.as<float2>();
        a.rownear = p->d_rownear.as<uint32_t>();
        a.colmin = p->d_colmin.as<uint32_t>();
        a.rowthr = p->d_rowthr.as<float>();
        a.colthr = p->d_colthr.as<float>();
        a.rowcnt = p->d_rowcnt.as<uint32_t>();
        a.rowrec = p->d_rowrec.as<float4>();
        a.half_recs = p->half_recs;
        a.rowrecj = p->d_rowrecj.as<uint32_t>();
        a.colcnt = p->d_colcnt.as<float>();
        a.rowdec = p->d_rowdec.as<uint32_t>();
        a.queue = p->d_queue.as<SlQueue>();
        a.rqueue = p->d_rqueue.as<SlQueue>();
        a.queue_cap = (uint32_t)p->queue_cap;
        a.ctl = ctl;
        a.ratio2 = p->ratio * p->ratio;
        a.mutual = p->mutual;
        a.fp8 = p->prec == SLM_PREC_FP8;
        a.dump = p->dump ? p->d_dump.as<float>() : nullptr;
        a.slots = p->d_slots.as<uint2>();
        a.counts = p->d_counts.as<uint32_t>();
        a.blkcnt = p->d_blkcnt.as<uint32_t>();
        a.pairctl = p->d_pairctl.as<uint32_t>();
        a.row_blocks = p->row_blocks;
        a.tiled = st->tiled.as<float>();
        a.xlist = p->d_xlist.as<uint32_t>();
        a.xitems = p->d_xitems.as<Item>();
        a.xitem_cap = (uint32_t)p->xitem_cap;
        a.xparts = p->d_xparts.as<RowPart>();
        a.colbest = p->d_colbest.as<unsigned long long>();
        a.want_items = 4u * (uint32_t)std::max(1, p->ctx->sms);
        a.rescue = p->prec == SLM_PREC_FP8 ? 1u : 0u;
        a.tier = 0;
        int nk = 1;  // the colmin fill
        SLM_CU(record_event(p->ev0, s));
        nk += launch_shortlist_eps(a, s);
        nk += launch_shortlist_pass(a, 1, p->ctx->sms, s);
        SLM_CU(record_event(p->evp[0], s));
        nk += launch_shortlist_mid(a, s);
        SLM_CU(record_event(p->evp[1], s));
        nk += launch_shortlist_pass(a, 2, p->ctx->sms, s);
        SLM_CU(record_event(p->evp[2], s));
        nk += launch_shortlist_finalize(a, s);
        if (a.rescue) {
            // tier 1: the BF16 passes over the pairs FP8 could not settle (their
            // kernels return at once when no pair was rescued)
            SlArgs b = a;
            const slm_store::LowpImage &bi = st->lowp[0];
            b.optiles = bi.optiles.as<uint8_t>();
            b.norms = bi.norms.as<float>();
            b.qscale = nullptr;
            b.vstats = bi.vstats.as<ViewStat>();
            b.fp8 = 0;
            b.dump = nullptr;
            b.rescue = 0;
            b.tier = 1;
            nk += launch_shortlist_rescue_prep(b, s);
            nk += launch_shortlist_pass(b, 1, p->ctx->sms, s);
            nk += launch_shortlist_mid(b, s);
            nk += launch_shortlist_pass(b, 2, p->ctx->sms, s);
            nk += launch_shortlist_finalize(b, s);
        }
        nk += launch_shortlist_tail(a, p->ctx->sms, s);
        SLM_CU(record_event(p->ev1, s));
        p->kernels = (uint64_t)nk + 2;  // + scan_counts, gather
        if (p->min_matches > 1) {
            launch_filter_counts(p->d_counts.as<uint32_t>(), p->np, p->min_matches, s);
            p->kernels++;
        }
        uint64_t *offsets = p->d_offsets.as<uint64_t>();
        launch_scan_counts(p->d_counts.as<uint32_t>(), p->np, offsets, s);
        launch_gather_blocks(a, offsets + (p->np + 1), offsets, p->d_dense.as<uint2>(), p->n_slots, s);
        SLM_CU(cudaGetLastError());
        return SLM_OK;
    }
    if (p->mutual) launch_fill_u64(p->d_colbest.as<unsigned long long>(), p->n_cols, ~0ull, s);
    const float ratio2 = p->ratio * p->ratio;
    {
        ExactArgs a{};
        a.tiled = p->st->tiled.as<float>();
        a.items = p->d_items.as<Item>();
        a.n_items = (uint32_t)p->items.size();
        a.pairs = p->d_meta.as<PairMeta>();
        a.parts = p->d_parts.as<RowPart>();
        a.colbest = p->d_colbest.as<unsigned long long>();
        a.work = ctl;
        a.err = ctl + 1;
        a.mutual = p->mutual;
        a.x2 = p->tune.variant == 1 ? 0 : 1;  // packed f32x2 arithmetic; 1: all scalar
        // External records so that the events become timing nodes under graph capture.
        SLM_CU(record_event(p->ev0, s));
        if (a.n_items) launch_exact(a, std::min<int>(p->ctx->sms, (int)a.n_items), s);
        SLM_CU(record_event(p->ev1, s));
        p->kernels = (p->mutual ? 1 : 0) + (a.n_items ? 1 : 0) + (p->np ? 1 : 0) + 1 + (p->np ? 1 : 0);
        FinalizeArgs f{};
        f.pairs = p->d_meta.as<PairMeta>();
        f.npairs = p->np;
        f.parts = p->d_parts.as<RowPart>();
        f.colbest = p->d_colbest.as<unsigned long long>();
        f.ratio2 = ratio2;
        f.mutual = p->mutual;
        f.slots = p->d_slots.as<uint2>();
        f.counts = p->d_counts.as<uint32_t>();
        launch_finalize(f, s);
    }
    if (p->min_matches > 1) {
        launch_filter_counts(p->d_counts.as<uint32_t>(), p->np, p->min_matches, s);
        p->kernels++;
    }
    uint64_t *offsets = p->d_offsets.as<uint64_t>();
    launch_scan_counts(p->d_counts.as<uint32_t>(), p->np, offsets, s);
    launch_gather(p->d_slots.as<uint2>(), offsets + (p->np + 1), p->d_counts.as<uint32_t>(), offsets, p->np,
                  p->d_dense.as<uint2>(), p->n_slots, s);
    SLM_CU(cudaGetLastError());
    return SLM_OK;
}

}  // namespace

// ------------------------------------------------------------- workspaces

// Everything one single-pair call needs: its own stream, a two-view store
// and a plan, reused across calls of similar size.
struct Workspace {
    cudaStream_t stream = nullptr;
    slm_store store;
    slm_plan plan;
    DevBuf single;                   // FP32 single-pair calls: inputs and scratch
    DevBuf score;                    // slm_sampson_score: inputs and outputs
    DevBuf feat_in;                  // descriptor producer: the batch's images
    DevBuf feat_up;                  // the images it upsamples 2x, and their upsampling
    DevBuf feat_pyr;                 // its pyramid, gradient tables and candidates
    DevBuf feat_desc[2];             // its descriptors (input-size and upsampled detections) and jobs
    unsigned char *single_host = nullptr;  // their result block: pinned host memory the kernels write
    size_t single_host_bytes = 0;
};

namespace {

slm_status ctx_check_device(slm_ctx *c) {
    SLM_CU(cudaSetDevice(c->device));
    return SLM_OK;
}

slm_status ws_acquire(slm_ctx *c, Workspace **out) {
    {
        std::lock_guard<std::mutex> g(c->mu);
        if (!c->idle.empty()) {
            *out = c->idle.back();
            c->idle.pop_back();
            return SLM_OK;
        }
    }
    Workspace *w = new (std::nothrow) Workspace();
    if (!w) return fail(SLM_OOM, "host allocation failed");
    cudaError_t e = cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete w;
        return fail(SLM_CUDA_ERROR, std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
    }
    w->store.ctx = c;
    w->plan.ctx = c;
    w->plan.st = &w->store;
    {
        std::lock_guard<std::mutex> g(c->mu);
        c->all.push_back(w);
    }
    *out = w;
    return SLM_OK;
}

void ws_release(slm_ctx *c, Workspace *w) {
    std::lock_guard<std::mutex> g(c->mu);
    c->idle.push_back(w);
}

// Reserve room for rows in a store (grows the device buffers if needed).
slm_status store_reserve(slm_store *st, uint64_t rows) {
    slm_ctx *c = st->ctx;
    SLM_TRY(st->raw.ensure(c, rows * kDesc * sizeof(float)));
    SLM_TRY(st->tiled.ensure(c, rows * kDesc * sizeof(float)));
    st->max_rows = std::max<uint64_t>(st->max_rows, st->raw.bytes / (kDesc * sizeof(float)));
    return SLM_OK;
}

// Room for `views` more views of `padded` rows in total.
slm_status store_check_room(const slm_store *st, uint64_t views, uint64_t padded) {
    if (st->max_views && st->row0.size() + views > st->max_views)
        return fail(SLM_CAPACITY, "store view capacity " + std::to_string(st->max_views) + " reached");
    if (st->rows_used + padded > st->max_rows)
        return fail(SLM_CAPACITY, "store descriptor capacity exceeded: " + std::to_string(st->rows_used + padded) +
                                      " > " + std::to_string(st->max_rows) + " padded rows");
    if (st->rows_used + padded >= (1ull << 32)) return fail(SLM_CAPACITY, "store exceeds 2^32 rows");
    return SLM_OK;
}

// Bookkeeping of one appended view of n rows; returns its first store row.
uint64_t store_place(slm_store *st, uint32_t n, uint32_t *id) {
    const uint64_t row0 = st->rows_used;
    if (id) *id = (uint32_t)st->row0.size();
    st->row0.push_back((uint32_t)row0);
    st->n.push_back(n);
    st->rows_used += pad_rows(n);
    st->version++;
    return row0;
}

slm_status store_append(slm_store *st, const float *desc, uint32_t n, bool device_src, cudaStream_t s,
                        uint32_t *id) {
    SLM_TRY(store_check_room(st, 1, pad_rows(n)));
    float *raw = st->raw.as<float>() + st->rows_used * kDesc;
    if (n) {
        SLM_CU(cudaMemcpyAsync(raw, desc, (size_t)n * kDesc * sizeof(float),
                               device_src ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
    }
    store_place(st, n, id);
    return SLM_OK;
}

// Appends `count` views whose rows the device reads where they lie (host
// memory it can read directly, or device memory) with one gather launch.
slm_status store_append_direct(slm_store *st, size_t count, const float *const *src, const uint32_t *n, uint32_t *ids,
                               cudaStream_t s) {
    uint64_t padded = 0;
    for (size_t k = 0; k < count; ++k) padded += pad_rows(n[k]);
    SLM_TRY(store_check_room(st, count, padded));
    std::vector<uint4> tab;
    tab.reserve(count);
    for (size_t k = 0; k < count; ++k) {
        const uint64_t row0 = store_place(st, n[k], ids ? &ids[k] : nullptr);
        const uint64_t adr = reinterpret_cast<uint64_t>(src[k]);
        if (n[k]) tab.push_back(make_uint4((uint32_t)adr, (uint32_t)(adr >> 32), (uint32_t)row0, n[k]));
    }
    launch_gather_rows(tab.data(), (uint32_t)tab.size(), st->raw.as<float>(), s);
    SLM_CU(cudaGetLastError());
    return SLM_OK;
}

// The host status for a plan's error word.
slm_status status_of_word(uint32_t err) {
    if (err == DERR_TIMEOUT_BAR || err == DERR_TIMEOUT_MMA)
        return fail(SLM_TIMEOUT, "device wait gave up (code " + std::to_string(err) + ")");
    if (err) return fail(SLM_INTERNAL, "device invariant failed (code " + std::to_string(err) + ")");
    return SLM_OK;
}

slm_status check_status_word(slm_plan *p) {
    uint32_t err = 0;
    SLM_CU(cudaMemcpy(&err, p->d_ctl.as<uint32_t>() + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    return status_of_word(err);
}

// ctl: a host copy of the plan's 16 control words, or null to read them.
slm_status fill_stats(slm_plan *p, slm_stats *st, uint64_t matches, const uint32_t *ctl = nullptr) {
    if (!st) return SLM_OK;
    std::memset(st, 0, sizeof(*st));
    st->pairs = p->np;
    st->distances = p->distances;
    st->matches = matches;
    st->kernel_launches = p->kernels;
    if (p->prec != SLM_PREC_FP32 && p->launched) {
        uint32_t w[16];
        if (ctl)
            std::memcpy(w, ctl, sizeof(w));
        else
            SLM_CU(cudaMemcpy(w, p->d_ctl.p, sizeof(w), cudaMemcpyDeviceToHost));
        st->rows_rescored = w[kCtlRescored];
        st->rows_recomputed = (uint64_t)w[kCtlQueueRows] + w[kCtlRoutedRows];
        st->cols_recomputed = (uint64_t)w[kCtlQueueCols] + w[kCtlRoutedCols];
        st->pairs_routed = w[kCtlRoutedPairs];
        st->pairs_rescued = w[kCtlRescuedPairs];
        st->rows_rescued = w[kCtlRescuedRows];
        float e;
        std::memcpy(&e, &w[kCtlMaxErr], sizeof(e));
        st->max_abs_err = e;
    }
    if (p->launched && p->ev0 && p->ev1) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, p->ev0, p->ev1) == cudaSuccess) st->kernel_ms = ms;
        if (p->prec != SLM_PREC_FP32) {
            if (cudaEventElapsedTime(&ms, p->ev0, p->evp[0]) == cudaSuccess) st->pass_ms[0] = ms;
            if (cudaEventElapsedTime(&ms, p->evp[1], p->evp[2]) == cudaSuccess) st->pass_ms[1] = ms;
        } else {
            st->pass_ms[0] = st->kernel_ms;
        }
        cudaGetLastError();
    }
    return SLM_OK;
}

bool prec_valid(slm_precision p) {
    return p == SLM_PREC_FP32 || p == SLM_PREC_BF16 || p == SLM_PREC_FP8 || p == SLM_PREC_AUTO;
}

// SLM_PREC_AUTO for a call or batch of `distances` distances.
slm_precision resolve_prec(slm_precision p, uint64_t distances) {
    if (p != SLM_PREC_AUTO) return p;
    return distances >= SLM_AUTO_BF16_DISTANCES ? SLM_PREC_BF16 : SLM_PREC_FP32;
}

uint64_t batch_distances(const slm_store *st, const slm_pair *pairs, uint32_t np) {
    uint64_t d = 0;
    for (uint32_t k = 0; k < np; ++k)
        if (pairs[k].i < st->n.size() && pairs[k].j < st->n.size()) d += (uint64_t)st->n[pairs[k].i] * st->n[pairs[k].j];
    return d;
}

slm_status validate_ratio(float ratio) {
    if (!std::isfinite(ratio)) return fail(SLM_INVALID_ARG, "ratio must be finite");
    return SLM_OK;
}

}  // namespace

extern "C" slm_status slm_ctx_create(const slm_opts *opts, slm_ctx **out) {
    if (!out) return fail(SLM_INVALID_ARG, "out is NULL");
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(SLM_NO_DEVICE, std::string("no CUDA device: ") + cudaGetErrorString(e));
    }
    const int dev = opts ? opts->device : 0;
    if (dev < 0 || dev >= ndev) return fail(SLM_INVALID_ARG, "device ordinal out of range");
    cudaDeviceProp prop{};
    SLM_CU(cudaGetDeviceProperties(&prop, dev));
    if (!(prop.major == 10 && prop.minor == 3))
        return fail(SLM_NO_DEVICE, "libslm is built for sm_103a; device " + std::to_string(dev) + " is sm_" +
                                       std::to_string(prop.major) + std::to_string(prop.minor));
    SLM_CU(cudaSetDevice(dev));
    {
        cudaError_t ke = init_exact_kernels();
        if (ke == cudaSuccess) ke = init_shortlist_kernels();
        if (ke != cudaSuccess) {
            cudaGetLastError();
            return fail(SLM_NO_DEVICE, std::string("kernels do not load on this device: ") + cudaGetErrorString(ke));
        }
    }
    auto *c = new (std::nothrow) slm_ctx();
    if (!c) return fail(SLM_OOM, "host allocation failed");
    c->device = dev;
    c->sms = prop.multiProcessorCount;
    if (opts && opts->stream) {
        c->stream = static_cast<cudaStream_t>(opts->stream);
    } else {
        cudaError_t se = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
        if (se != cudaSuccess) {
            delete c;
            return fail(SLM_CUDA_ERROR, std::string("cudaStreamCreate: ") + cudaGetErrorString(se));
        }
        c->own_stream = true;
    }
    size_t fre = 0, tot = 0;
    cudaMemGetInfo(&fre, &tot);
    c->budget = (opts && opts->hbm_budget) ? opts->hbm_budget : (uint64_t)fre;
    int pageable = 0;
    if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, c->device) != cudaSuccess) {
        cudaGetLastError();
        pageable = 0;
    }
    const char *no_direct = std::getenv("SLM_NO_HOST_DIRECT");
    c->host_direct = pageable == 1 && !(no_direct && no_direct[0] == '1');
    {
        // the pool keeps up to 1 GiB of freed plan buffers for reuse
        cudaMemPoolProps pp{};
        pp.allocType = cudaMemAllocationTypePinned;
        pp.location.type = cudaMemLocationTypeDevice;
        pp.location.id = dev;
        uint64_t keep = 1ull << 30;
        if (cudaMemPoolCreate(&c->pool, &pp) != cudaSuccess ||
            cudaMemPoolSetAttribute(c->pool, cudaMemPoolAttrReleaseThreshold, &keep) != cudaSuccess) {
            cudaGetLastError();
            if (c->pool) cudaMemPoolDestroy(c->pool);
            c->pool = nullptr;  // plans then allocate with cudaMalloc
        }
    }
    *out = c;
    return SLM_OK;
}

extern "C" slm_status slm_ctx_destroy(slm_ctx *c) {
    if (!c) return SLM_OK;
    cudaSetDevice(c->device);
    coalescer_destroy(c);
    cudaDeviceSynchronize();
    for (Workspace *w : c->all) {
        plan_release(&w->plan);
        if (w->stream) cudaStreamDestroy(w->stream);
        if (w->single_host) cudaFreeHost(w->single_host);
        delete w;
    }
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    if (c->pool) cudaMemPoolDestroy(c->pool);
    delete c;
    return SLM_OK;
}

extern "C" void *slm_ctx_stream(slm_ctx *c) { return c ? static_cast<void *>(c->stream) : nullptr; }

extern "C" uint64_t slm_ctx_bytes_in_use(slm_ctx *c) { return c ? c->used.load() : 0; }

extern "C" slm_status slm_selftest_wait_timeout(slm_ctx *c, uint32_t polls) {
    if (!c) return fail(SLM_INVALID_ARG, "NULL context");
    if (polls < 1 || polls > 65536) return fail(SLM_INVALID_ARG, "polls must be in 1..65536");
    SLM_TRY(ctx_check_device(c));
    DevBuf word;
    SLM_TRY(word.ensure(c, sizeof(uint32_t)));
    SLM_CU(cudaMemsetAsync(word.p, 0, sizeof(uint32_t), c->stream));
    launch_wait_selftest(polls, word.as<uint32_t>(), c->stream);
    SLM_CU(cudaGetLastError());
    uint32_t err = 0;
    SLM_CU(cudaMemcpyAsync(&err, word.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream));
    SLM_CU(cudaStreamSynchronize(c->stream));
    if (err == DERR_TIMEOUT_BAR) return fail(SLM_TIMEOUT, "device wait gave up (self-test, as expected)");
    return fail(SLM_INTERNAL, "wait self-test: the wait did not give up (error word " + std::to_string(err) + ")");
}

// ------------------------------------------------------------------ stores

extern "C" slm_status slm_store_create(slm_ctx *c, uint64_t max_descs, uint32_t max_views, slm_store **out) {
    if (!c || !out) return fail(SLM_INVALID_ARG, "NULL argument");
    *out = nullptr;
    SLM_TRY(ctx_check_device(c));
    auto *st = new (std::nothrow) slm_store();
    if (!st) return fail(SLM_OOM, "host allocation failed");
    st->ctx = c;
    st->max_views = max_views;
    // every view may waste up to 127 padding rows
    const uint64_t rows = pad_rows(max_descs) + (uint64_t)max_views * kTile;
    slm_status s = store_reserve(st, rows);
    if (s != SLM_OK) {
        delete st;
        return s;
    }
    st->max_rows = rows;
    // the packing kernels' tile table, at its largest size once (a buffer that
    // grew later would be freed with a device-wide synchronisation)
    s = st->tiletab.ensure(c, std::max<uint64_t>(rows / kTile, 1) * sizeof(uint4));
    if (s != SLM_OK) {
        delete st;
        return s;
    }
    *out = st;
    return SLM_OK;
}

extern "C" slm_status slm_store_destroy(slm_store *st) {
    if (!st) return SLM_OK;
    cudaSetDevice(st->ctx->device);
    cudaStreamSynchronize(st->ctx->stream);
    delete st;
    return SLM_OK;
}

extern "C" slm_status slm_store_add_view(slm_store *st, const float *desc, uint32_t n, uint32_t *view_id) {
    NvtxRange range_("slm_store_add_view");
    if (!st || (!desc && n)) return fail(SLM_INVALID_ARG, "NULL argument");
    SLM_TRY(ctx_check_device(st->ctx));
    return store_append(st, desc, n, false, st->ctx->stream, view_id);
}

// Many views from one host buffer: one host-to-device copy of the rows they
// span into a staging buffer, then one kernel launch per 1024 views scatters
// them into their padded store rows (instead of one copy per view, each with
// its own call overhead). All views are checked for room before any is added.
// Views per slm_store_add_views call copied one by one (pinned or device
// sources); above this, a staging copy and a scatter kernel.
constexpr uint32_t kDirectViewCopies = 4096;

extern "C" slm_status slm_store_add_views(slm_store *st, const float *desc, const uint64_t *offsets,
                                          const uint32_t *counts, uint32_t nviews, uint32_t *ids) {
    NvtxRange range_("slm_store_add_views");
    if (!st || (!desc && nviews) || (nviews && (!offsets || !counts))) return fail(SLM_INVALID_ARG, "NULL argument");
    SLM_TRY(ctx_check_device(st->ctx));
    uint64_t lo = ~0ull, hi = 0, padded = 0;
    for (uint32_t v = 0; v < nviews; ++v) {
        padded += pad_rows(counts[v]);
        if (!counts[v]) continue;
        lo = std::min<uint64_t>(lo, offsets[v]);
        hi = std::max<uint64_t>(hi, offsets[v] + counts[v]);
    }
    SLM_TRY(store_check_room(st, nviews, padded));
    cudaStream_t s = st->ctx->stream;
    // Pinned or device sources: one copy per view straight into its padded
    // store rows. From pinned host memory these run on the copy engines; a
    // staging copy followed by a scatter kernel or by device-to-device copies
    // would need SMs, which a batch running on another stream may hold.
    cudaPointerAttributes pa{};
    const bool direct_copies = nviews <= kDirectViewCopies && cudaPointerGetAttributes(&pa, desc) == cudaSuccess &&
                               (pa.type == cudaMemoryTypeHost || pa.type == cudaMemoryTypeDevice);
    cudaGetLastError();
    if (direct_copies) {
        const cudaMemcpyKind kind = pa.type == cudaMemoryTypeDevice ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
        for (uint32_t v = 0; v < nviews; ++v) {
            uint32_t id = 0;
            const uint64_t row0 = store_place(st, counts[v], &id);
            if (ids) ids[v] = id;
            if (counts[v])
                SLM_CU(cudaMemcpyAsync(st->raw.as<float>() + row0 * kDesc, desc + offsets[v] * kDesc,
                                       (size_t)counts[v] * kDesc * sizeof(float), kind, s));
        }
        return SLM_OK;
    }
    if (hi > lo) {
        SLM_TRY(st->staging.ensure(st->ctx, (size_t)(hi - lo) * kDesc * sizeof(float)));
        SLM_CU(cudaMemcpyAsync(st->staging.p, desc + lo * kDesc, (size_t)(hi - lo) * kDesc * sizeof(float),
                               cudaMemcpyDefault, s));  // host or device source (unified addressing)
    }
    std::vector<uint4> tab;  // {first staging row, first store row, rows, 0}
    tab.reserve(nviews);
    for (uint32_t v = 0; v < nviews; ++v) {
        uint32_t id = 0;
        const uint64_t row0 = store_place(st, counts[v], &id);
        if (ids) ids[v] = id;
        if (counts[v]) tab.push_back(make_uint4((uint32_t)(offsets[v] - lo), (uint32_t)row0, counts[v], 0u));
    }
    if (!tab.empty()) {
        launch_scatter_rows(tab.data(), (uint32_t)tab.size(), st->staging.as<float>(), st->raw.as<float>(), s);
        SLM_CU(cudaGetLastError());
    }
    return SLM_OK;
}

extern "C" slm_status slm_store_clear(slm_store *st) {
    if (!st) return fail(SLM_INVALID_ARG, "NULL store");
    st->row0.clear();
    st->n.clear();
    st->rows_used = 0;
    st->version++;
    st->epoch++;
    return SLM_OK;
}

extern "C" uint32_t slm_store_num_views(slm_store *st) { return st ? (uint32_t)st->row0.size() : 0; }

// ------------------------------------------------------------------- plans

namespace {

// Upload the tile table of views [first, end) and return its tile count.
slm_status upload_tiletab(slm_store *st, size_t first, size_t end, cudaStream_t s, uint32_t *ntiles) {
    std::vector<uint4> tab;
    for (size_t v = first; v < end; ++v)
        for (uint32_t t = 0; t < (st->n[v] + kTile - 1) / kTile; ++t)
            tab.push_back(make_uint4(st->row0[v], st->n[v], t, (uint32_t)v));
    *ntiles = (uint32_t)tab.size();
    if (tab.empty()) return SLM_OK;
    SLM_TRY(st->tiletab.ensure(st->ctx, tab.size() * sizeof(uint4)));
    SLM_CU(cudaMemcpyAsync(st->tiletab.p, tab.data(), tab.size() * sizeof(uint4), cudaMemcpyHostToDevice, s));
    return SLM_OK;
}

// FP32 tiles of the views appended since the last build (one launch).
slm_status store_sync_fp32(slm_store *st, cudaStream_t s) {
    const size_t first = st->fp32_epoch == st->epoch ? st->fp32_views : 0;
    if (first >= st->row0.size() && st->fp32_epoch == st->epoch) return SLM_OK;
    uint32_t nt = 0;
    SLM_TRY(upload_tiletab(st, first, st->row0.size(), s, &nt));
    launch_pack_fp32_tiles(st->tiletab.as<uint4>(), nt, st->raw.as<float>(), st->tiled.as<float>(), s);
    SLM_CU(cudaGetLastError());
    st->fp32_epoch = st->epoch;
    st->fp32_views = st->row0.size();
    return SLM_OK;
}

// Build one of the store's low-precision operand images: only the views
// appended since its last build, unless the store was cleared.
slm_status store_sync_lowp(slm_store *st, bool fp8, cudaStream_t s) {
    slm_store::LowpImage &im = st->lowp[fp8 ? 1 : 0];
    if (im.version == st->version) return SLM_OK;
    slm_ctx *c = st->ctx;
    const uint64_t tiles = std::max<uint64_t>(st->max_rows / kTile, 1);
    const size_t tb = fp8 ? kFp8TileBytes : kBf16TileStride;
    size_t first = im.epoch != st->epoch ? 0 : im.views;
    SLM_TRY(im.optiles.ensure(c, tiles * tb));
    SLM_TRY(im.norms.ensure(c, tiles * kTile * sizeof(float)));
    if (fp8) SLM_TRY(im.qscale.ensure(c, tiles * kTile * sizeof(float)));
    const size_t nv = std::max<size_t>({st->row0.size(), (size_t)st->max_views, 1});
    if (im.vstats.bytes < nv * sizeof(ViewStat)) first = 0;  // grows: statistics are rebuilt
    SLM_TRY(im.vstats.ensure(c, nv * sizeof(ViewStat)));
    if (first < st->row0.size())
        SLM_CU(cudaMemsetAsync(im.vstats.as<ViewStat>() + first, 0, (st->row0.size() - first) * sizeof(ViewStat), s));
    uint32_t nt = 0;
    SLM_TRY(upload_tiletab(st, first, st->row0.size(), s, &nt));
    launch_pack_lowp(st->tiletab.as<uint4>(), nt, st->raw.as<float>(), fp8 ? 1 : 0, im.optiles.as<uint8_t>(),
                     im.norms.as<float>(), im.qscale.as<float>(), im.vstats.as<ViewStat>(), s);
    SLM_CU(cudaGetLastError());
    im.version = st->version;
    im.epoch = st->epoch;
    im.views = st->row0.size();
    return SLM_OK;
}

// The images a plan of this precision reads: BF16 for BF16 plans, both for
// FP8 plans (the BF16 passes rescue the pairs the FP8 bound cannot settle).
slm_status store_sync_plan_images(slm_store *st, slm_precision prec, cudaStream_t s) {
    if (prec == SLM_PREC_BF16 || prec == SLM_PREC_FP8) SLM_TRY(store_sync_lowp(st, false, s));
    if (prec == SLM_PREC_FP8) SLM_TRY(store_sync_lowp(st, true, s));
    return SLM_OK;
}

slm_status plan_init(slm_plan *p, slm_ctx *c, slm_store *st, const slm_pair *pairs, uint32_t np, float ratio,
                     int mutual, slm_precision prec, const slm_tune *tune, cudaStream_t stream) {
    p->ctx = c;
    p->stream = stream;
    for (DevBuf *b : plan_buffers(p)) b->order_on(stream);
    p->st = st;
    p->np = np;
    p->ratio = ratio;
    p->mutual = mutual ? 1 : 0;
    prec = resolve_prec(prec, prec == SLM_PREC_AUTO ? batch_distances(st, pairs, np) : 0);
    p->prec = prec;
    p->tune = tune ? *tune : slm_tune{};
    if (!p->tune.use_graph) p->tune.use_graph = 1;
    if (p->exec) {
        cudaGraphExecDestroy(p->exec);
        p->exec = nullptr;
    }
    if (p->graph) {
        cudaGraphDestroy(p->graph);
        p->graph = nullptr;
    }
    p->launched = false;
    p->dump = p->tune.variant == 2 && prec != SLM_PREC_FP32;
    // FP32 tiles: the whole store for FP32 and FP8 plans (FP8 routes most
    // pairs of unit descriptors to the exact kernel); a BF16 batch packs the
    // tiles of its few routed pairs' views itself, on the device
    if (prec != SLM_PREC_BF16) SLM_TRY(store_sync_fp32(st, stream));
    SLM_TRY(store_sync_plan_images(st, prec, stream));
    return plan_build(p, pairs);
}

slm_status plan_launch_on(slm_plan *p, cudaStream_t s, bool use_graph) {
    if (p->prec != SLM_PREC_BF16) SLM_TRY(store_sync_fp32(p->st, s));
    SLM_TRY(store_sync_plan_images(p->st, p->prec, s));
    // a store buffer the captured graph reads may have moved: capture again
    if (p->exec && (p->st->tiled.p != p->graph_tiled || p->st->lowp[0].optiles.p != p->graph_optiles[0] ||
                    p->st->lowp[1].optiles.p != p->graph_optiles[1])) {
        cudaGraphExecDestroy(p->exec);
        p->exec = nullptr;
    }
    p->graph_tiled = p->st->tiled.p;
    p->graph_optiles[0] = p->st->lowp[0].optiles.p;
    p->graph_optiles[1] = p->st->lowp[1].optiles.p;
    if (!p->ev0) SLM_CU(cudaEventCreate(&p->ev0));
    if (!p->ev1) SLM_CU(cudaEventCreate(&p->ev1));
    for (cudaEvent_t &e : p->evp)
        if (!e) SLM_CU(cudaEventCreate(&e));
    if (use_graph) {
        if (!p->exec) {
            SLM_CU(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            slm_status es = plan_enqueue(p, s);
            cudaGraph_t g = nullptr;
            cudaError_t ce = cudaStreamEndCapture(s, &g);
            if (es != SLM_OK) {
                if (g) cudaGraphDestroy(g);
                return es;
            }
            if (ce != cudaSuccess) return fail(SLM_CUDA_ERROR, std::string("graph capture: ") + cudaGetErrorString(ce));
            p->graph = g;
            SLM_CU(cudaGraphInstantiate(&p->exec, g, 0));
        }
        SLM_CU(cudaGraphLaunch(p->exec, s));
    } else {
        SLM_TRY(plan_enqueue(p, s));
    }
    p->launched = true;
    return SLM_OK;
}

}  // namespace

namespace {

uint64_t tune_key(const slm_store *st, const slm_pair *pairs, uint32_t np, int mutual, slm_precision prec) {
    uint64_t rows = 0;
    for (uint32_t k = 0; k < np; ++k) rows += pairs[k].i < st->n.size() ? st->n[pairs[k].i] : 0;
    auto lg = [](uint64_t x) {
        uint64_t b = 0;
        while (x > 1) x >>= 1, ++b;
        return b;
    };
    return ((uint64_t)prec << 16) | ((uint64_t)(mutual ? 1 : 0) << 15) | (lg(np ? rows / np : 0) << 8) | lg(np);
}

}  // namespace

extern "C" slm_status slm_autotune(slm_ctx *c, slm_store *st, const slm_pair *pairs, uint32_t np, float ratio,
                                   int mutual, slm_precision prec, slm_tune *best, float *best_ms) {
    NvtxRange range_("slm_autotune");
    if (!c || !st || (np && !pairs)) return fail(SLM_INVALID_ARG, "NULL argument");
    if (!prec_valid(prec)) return fail(SLM_INVALID_ARG, "unknown precision");
    SLM_TRY(validate_ratio(ratio));
    SLM_TRY(ctx_check_device(c));
    prec = resolve_prec(prec, prec == SLM_PREC_AUTO ? batch_distances(st, pairs, np) : 0);
    // FP32: items per SM x arithmetic variant; BF16/FP8: items per SM x the
    // M tile shape (128-row a tiles per CTA work item, M = 128 or 256) x the
    // shortlist capacity (records of 4-column hit groups per row and column half)
    std::vector<slm_tune> grid;
    const uint32_t ips[3] = {2, 4, 8};
    const uint32_t ks[3] = {8, 12, 16};
    for (uint32_t a = 0; a < 2; ++a)
        for (uint32_t ki = 0; ki < (prec == SLM_PREC_FP32 ? 1u : 3u); ++ki)
            for (uint32_t ipsm : ips) {
                slm_tune t{};
                t.use_graph = 2;
                t.items_per_sm = ipsm;
                if (prec == SLM_PREC_FP32) {
                    t.variant = a;  // 0 packed f32x2 sub/add, 1 scalar
                } else {
                    t.row_tiles = a + 1;
                    t.shortlist_k = ks[ki];
                }
                grid.push_back(t);
            }
    std::unique_ptr<slm_plan> p(new (std::nothrow) slm_plan());
    if (!p) return fail(SLM_OOM, "host allocation failed");
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    SLM_CU(cudaEventCreate(&e0));
    SLM_CU(cudaEventCreate(&e1));
    float best_t = 3.4e38f;
    slm_tune best_tune = grid[0];
    slm_status status = SLM_OK;
    for (const slm_tune &t : grid) {
        status = plan_init(p.get(), c, st, pairs, np, ratio, mutual, prec, &t, c->stream);
        if (status != SLM_OK) break;
        status = plan_launch_on(p.get(), c->stream, false);  // warm-up
        float tmin = 3.4e38f;
        for (int rep = 0; rep < 3 && status == SLM_OK; ++rep) {
            cudaEventRecord(e0, c->stream);
            status = plan_launch_on(p.get(), c->stream, false);
            cudaEventRecord(e1, c->stream);
            if (cudaEventSynchronize(e1) != cudaSuccess) status = fail(SLM_CUDA_ERROR, "autotune timing");
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            tmin = std::min(tmin, ms);
        }
        if (status != SLM_OK) break;
        SLM_TRY(check_status_word(p.get()));
        if (tmin < best_t) best_t = tmin, best_tune = t;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (status != SLM_OK) return status;
    best_tune.use_graph = 1;
    {
        std::lock_guard<std::mutex> g(c->mu);
        c->tuned[tune_key(st, pairs, np, mutual, prec)] = best_tune;
    }
    if (best) *best = best_tune;
    if (best_ms) *best_ms = best_t;
    return SLM_OK;
}

extern "C" slm_status slm_plan_create(slm_ctx *c, slm_store *st, const slm_pair *pairs, uint32_t np, float ratio,
                                      int mutual, slm_precision prec, const slm_tune *tune, slm_plan **out) {
    if (!c || !st || !out || (np && !pairs)) return fail(SLM_INVALID_ARG, "NULL argument");
    if (!prec_valid(prec)) return fail(SLM_INVALID_ARG, "unknown precision");
    SLM_TRY(validate_ratio(ratio));
    *out = nullptr;
    SLM_TRY(ctx_check_device(c));
    prec = resolve_prec(prec, prec == SLM_PREC_AUTO ? batch_distances(st, pairs, np) : 0);
    slm_tune t = tune ? *tune : slm_tune{};
    if (t.autotune) {
        const uint64_t key = tune_key(st, pairs, np, mutual, prec);
        bool have = false;
        {
            std::lock_guard<std::mutex> g(c->mu);
            auto it = c->tuned.find(key);
            if (it != c->tuned.end()) have = true, t = it->second;
        }
        if (!have) SLM_TRY(slm_autotune(c, st, pairs, np, ratio, mutual, prec, &t, nullptr));
        if (tune && tune->use_graph) t.use_graph = tune->use_graph;
        t.autotune = 0;
    }
    if (t.shortlist_k > kSlHalfRecsMax)
        return fail(SLM_INVALID_ARG, "shortlist_k must be at most " + std::to_string(kSlHalfRecsMax));
    auto *p = new (std::nothrow) slm_plan();
    if (!p) return fail(SLM_OOM, "host allocation failed");
    slm_status s = plan_init(p, c, st, pairs, np, ratio, mutual, prec, &t, c->stream);
    if (s != SLM_OK) {
        std::string keep = g_last_error;
        delete p;
        g_last_error = keep;
        return s;
    }
    *out = p;
    return SLM_OK;
}

extern "C" slm_status slm_plan_destroy(slm_plan *p) {
    if (!p) return SLM_OK;
    cudaSetDevice(p->ctx->device);
    cudaStreamSynchronize(p->stream);
    delete p;
    return SLM_OK;
}

extern "C" slm_status slm_plan_launch(slm_plan *p) {
    NvtxRange range_("slm_plan_launch");
    if (!p) return fail(SLM_INVALID_ARG, "NULL plan");
    SLM_TRY(ctx_check_device(p->ctx));
    return plan_launch_on(p, p->stream, p->tune.use_graph != 2);
}

extern "C" slm_status slm_plan_results(slm_plan *p, slm_pair *out, uint64_t cap, uint64_t *offsets, slm_stats *st) {
    NvtxRange range_("slm_plan_results");
    if (!p || !offsets || (cap && !out)) return fail(SLM_INVALID_ARG, "NULL argument");
    if (!p->launched) return fail(SLM_INVALID_ARG, "plan was not launched");
    SLM_TRY(ctx_check_device(p->ctx));
    SLM_CU(cudaStreamSynchronize(p->stream));
    SLM_TRY(check_status_word(p));
    SLM_CU(cudaMemcpy(offsets, p->d_offsets.p, sizeof(uint64_t) * (p->np + 1), cudaMemcpyDeviceToHost));
    const uint64_t total = offsets[p->np];
    SLM_TRY(fill_stats(p, st, total));
    if (total > cap) return fail(SLM_CAPACITY, "need " + std::to_string(total) + " pairs, have " + std::to_string(cap));
    if (total) SLM_CU(cudaMemcpy(out, p->d_dense.p, sizeof(slm_pair) * total, cudaMemcpyDeviceToHost));
    return SLM_OK;
}

extern "C" slm_status slm_plan_device_results(slm_plan *p, const uint32_t **d_counts, const slm_pair **d_slots,
                                              const uint64_t **h_slot_offsets) {
    if (!p) return fail(SLM_INVALID_ARG, "NULL plan");
    if (d_counts) *d_counts = p->d_counts.as<uint32_t>();
    if (d_slots) *d_slots = p->d_slots.as<slm_pair>();
    if (h_slot_offsets) *h_slot_offsets = p->slot_off.data();
    return SLM_OK;
}

extern "C" uint64_t slm_plan_bytes(slm_plan *p) {
    if (!p) return 0;
    return p->d_meta.bytes + p->d_items.bytes + p->d_parts.bytes + p->d_colbest.bytes + p->d_slots.bytes +
           p->d_counts.bytes + p->d_ctl.bytes + p->d_offsets.bytes + p->d_dense.bytes;
}

extern "C" slm_status slm_match_batch(slm_ctx *c, slm_store *st, const slm_pair *pairs, uint32_t np, float ratio,
                                      int mutual, slm_precision prec, slm_pair *out, uint64_t cap, uint64_t *offsets,
                                      slm_stats *stats) {
    slm_plan *p = nullptr;
    SLM_TRY(slm_plan_create(c, st, pairs, np, ratio, mutual, prec, nullptr, &p));
    slm_status s = slm_plan_launch(p);
    if (s == SLM_OK) s = slm_plan_results(p, out, cap, offsets, stats);
    std::string keep = g_last_error;
    slm_plan_destroy(p);
    g_last_error = keep;
    return s;
}

extern "C" slm_status slm_plan_set_min_matches(slm_plan *p, uint32_t min_matches) {
    if (!p) return fail(SLM_INVALID_ARG, "NULL plan");
    if (p->min_matches != min_matches && p->exec) {  // the captured graph has the old filter
        cudaGraphExecDestroy(p->exec);
        p->exec = nullptr;
    }
    p->min_matches = min_matches;
    return SLM_OK;
}

extern "C" slm_status slm_match_pairs(slm_ctx *c, slm_store *st, const uint64_t *views, uint32_t nv,
                                      const slm_pair_schedule *sch, float ratio, int mutual, slm_precision prec,
                                      uint32_t min_matches, slm_pair *pairs_out, uint64_t pairs_cap,
                                      uint64_t *n_pairs, slm_pair *out, uint64_t cap, uint64_t *offsets,
                                      slm_stats *stats) {
    NvtxRange range_("slm_match_pairs");
    if (!c || !st || (nv && !views) || !n_pairs || (pairs_cap && (!pairs_out || !offsets)))
        return fail(SLM_INVALID_ARG, "NULL argument");
    if (nv > st->row0.size())
        return fail(SLM_INVALID_ARG, "views names " + std::to_string(nv) + " views, the store holds " +
                                         std::to_string(st->row0.size()));
    *n_pairs = 0;
    const slm_pair_schedule def = slm_pair_schedule_default();
    uint64_t total = 0;
    slm_status s = slm_scheduled_pairs(views, nv, sch ? sch : &def, nullptr, 0, &total);
    if (s != SLM_OK && s != SLM_CAPACITY) return s;
    if (total >= (1ull << 32)) return fail(SLM_CAPACITY, "too many scheduled pairs for one batch");
    std::vector<slm_pair> pairs(std::max<uint64_t>(total, 1));
    SLM_TRY(slm_scheduled_pairs(views, nv, sch ? sch : &def, pairs.data(), total, &total));
    const uint32_t np = (uint32_t)total;
    slm_plan *p = nullptr;
    SLM_TRY(slm_plan_create(c, st, pairs.data(), np, ratio, mutual, prec, nullptr, &p));
    p->min_matches = min_matches;
    std::vector<uint64_t> off(np + 1, 0);
    s = slm_plan_launch(p);
    if (s == SLM_OK) s = slm_plan_results(p, out, cap, off.data(), stats);
    const std::string keep_err = g_last_error;
    slm_plan_destroy(p);
    g_last_error = keep_err;
    if (s != SLM_OK && s != SLM_CAPACITY) return s;
    // pairs that passed the filter, in schedule order (pipeline.rs:487-496 keeps
    // the order of the pair list)
    uint64_t kept = 0;
    for (uint32_t k = 0; k < np; ++k) {
        const uint64_t m = off[k + 1] - off[k];
        if (m < min_matches) continue;  // filtered on the device: m == 0 here
        if (kept < pairs_cap) {
            pairs_out[kept] = pairs[k];
            offsets[kept] = off[k];
        }
        ++kept;
    }
    *n_pairs = kept;
    if (kept > pairs_cap)
        return fail(SLM_CAPACITY, "pairs_cap " + std::to_string(pairs_cap) + " < " + std::to_string(kept) +
                                      " pairs kept");
    if (pairs_cap) offsets[kept] = off[np];
    return s;  // SLM_CAPACITY here: out holds fewer than offsets[kept] matches
}

// -------------------------------------------------------------- single pair

namespace {

// Run one pair through a workspace: load a and b into its two-view store,
// plan and enqueue on its stream. The caller synchronises.
slm_status single_pair_enqueue(slm_ctx *c, Workspace *w, const float *a, uint32_t na, const float *b, uint32_t nb,
                               float ratio, int mutual, slm_precision prec, bool device_src) {
    slm_store *st = &w->store;
    const uint64_t rows = pad_rows(na) + pad_rows(nb);
    SLM_TRY(store_reserve(st, std::max<uint64_t>(rows, kTile)));
    slm_store_clear(st);
    const bool aligned = ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b)) & 15) == 0;
    if ((device_src || c->host_direct) && aligned) {  // one gather launch reads both where they lie
        const float *src[2] = {a, b};
        const uint32_t n[2] = {na, nb};
        SLM_TRY(store_append_direct(st, 2, src, n, nullptr, w->stream));
    } else {
        SLM_TRY(store_append(st, a, na, false, w->stream, nullptr));
        SLM_TRY(store_append(st, b, nb, false, w->stream, nullptr));
    }
    const slm_pair pr{0, 1};
    slm_tune t{};
    t.use_graph = 2;  // one-off shapes: plain launches, no graph
    SLM_TRY(plan_init(&w->plan, c, st, &pr, 1, ratio, mutual, prec, &t, w->stream));
    return plan_launch_on(&w->plan, w->stream, false);
}

struct WsGuard {
    slm_ctx *c;
    Workspace *w;
    ~WsGuard() {
        if (w) ws_release(c, w);
    }
};

slm_status check_pair_args(slm_ctx *c, const float *a, uint32_t na, const float *b, uint32_t nb, float ratio,
                           slm_precision prec) {
    if (!c) return fail(SLM_INVALID_ARG, "NULL context");
    if ((na && !a) || (nb && !b)) return fail(SLM_INVALID_ARG, "NULL descriptor array");
    if (!prec_valid(prec)) return fail(SLM_INVALID_ARG, "unknown precision");
    return validate_ratio(ratio);
}

}  // namespace

namespace {

// The workspace's pinned, mapped host block of at least `bytes` (grown with
// slack). The old block is freed only once the workspace's stream is idle: a
// call that failed after enqueuing work may have left a copy into it pending.
slm_status ws_host_block(Workspace *w, size_t bytes) {
    if (w->single_host_bytes >= bytes) return SLM_OK;
    if (w->single_host) {
        cudaStreamSynchronize(w->stream);
        cudaFreeHost(w->single_host);
    }
    w->single_host = nullptr;
    w->single_host_bytes = 0;
    const size_t want = bytes + bytes / 4 + 4096;
    SLM_CU(cudaHostAlloc(reinterpret_cast<void **>(&w->single_host), want, cudaHostAllocMapped));
    w->single_host_bytes = want;
    return SLM_OK;
}

// An FP32 single-pair call without a store or a plan: the packing reads the
// inputs where they lie (or from the workspace's scratch block after two
// uploads), the metadata is made on the device, and the finalize kernel writes
// the pairs and their count into pinned host memory (3 kernels, no read-back).
slm_status single_pair_fp32(slm_ctx *c, Workspace *w, const float *a, uint32_t na, const float *b, uint32_t nb,
                            float ratio, int mutual, slm_pair *out, uint32_t cap, uint32_t *n_out, slm_stats *st) {
    const SingleLayout L = single_layout(na, nb, c->sms, true);
    SLM_TRY(w->single.ensure(c, L.bytes));
    unsigned char *sc = w->single.as<unsigned char>();
    cudaStream_t s = w->stream;
    const float *src_a = a, *src_b = b;
    // the packing kernels read rows as float4: direct reads need 16-byte alignment
    const bool direct = c->host_direct && ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b)) & 15) == 0;
    if (!direct) {
        SLM_CU(cudaMemcpyAsync(sc + L.raw_a, a, (size_t)na * kDesc * sizeof(float), cudaMemcpyHostToDevice, s));
        SLM_CU(cudaMemcpyAsync(sc + L.raw_b, b, (size_t)nb * kDesc * sizeof(float), cudaMemcpyHostToDevice, s));
        src_a = reinterpret_cast<const float *>(sc + L.raw_a);
        src_b = reinterpret_cast<const float *>(sc + L.raw_b);
    }
    // finalize writes the count and the pairs straight into pinned host memory
    // (no separate read-back)
    SLM_TRY(ws_host_block(w, 8 + sizeof(slm_pair) * (size_t)na));
    unsigned char *res = nullptr;
    SLM_CU(cudaHostGetDevicePointer(reinterpret_cast<void **>(&res), w->single_host, 0));
    SLM_CU(single_exact_enqueue(sc, L, src_a, na, src_b, nb, ratio, mutual, reinterpret_cast<slm_pair *>(res + 8), na,
                                reinterpret_cast<uint32_t *>(res), c->sms, s));
    SLM_CU(cudaStreamSynchronize(s));
    uint32_t n = 0;
    std::memcpy(&n, w->single_host, sizeof(n));
    if (n == 0xffffffffu) return fail(SLM_TIMEOUT, "device wait gave up");
    *n_out = n;
    if (st) {
        st->pairs = 1;
        st->distances = (uint64_t)na * nb;
        st->matches = n;
        st->kernel_launches = 3;
    }
    if (n > cap) return fail(SLM_CAPACITY, "need " + std::to_string(n) + " pairs, have " + std::to_string(cap));
    if (n) std::memcpy(out, w->single_host + 8, sizeof(slm_pair) * (size_t)n);
    return SLM_OK;
}

}  // namespace

extern "C" slm_status slm_ratio_match(slm_ctx *c, const float *a, uint32_t na, const float *b, uint32_t nb,
                                      float ratio, int mutual, slm_precision prec, slm_pair *out, uint32_t cap,
                                      uint32_t *n_out, slm_stats *st) {
    NvtxRange range_("slm_ratio_match");
    SLM_TRY(check_pair_args(c, a, na, b, nb, ratio, prec));
    const bool coalesce = prec == SLM_PREC_AUTO && c->coal;
    prec = resolve_prec(prec, (uint64_t)na * nb);
    if (!n_out || (cap && !out)) return fail(SLM_INVALID_ARG, "NULL output");
    *n_out = 0;
    if (st) std::memset(st, 0, sizeof(*st));
    // matching.rs:160-166: no second neighbour (or nothing to match) -> no pairs.
    if (na == 0 || nb < 2) {
        if (st) st->pairs = 1, st->distances = (uint64_t)na * nb;
        return SLM_OK;
    }
    SLM_TRY(ctx_check_device(c));
    if (coalesce) return coalesce_call(c, a, na, b, nb, ratio, mutual, out, cap, n_out, st);
    Workspace *w = nullptr;
    SLM_TRY(ws_acquire(c, &w));
    WsGuard guard{c, w};
    if (prec == SLM_PREC_FP32) return single_pair_fp32(c, w, a, na, b, nb, ratio, mutual, out, cap, n_out, st);
    SLM_TRY(single_pair_enqueue(c, w, a, na, b, nb, ratio, mutual, prec, false));
    slm_plan *p = &w->plan;
    // the control words, the offsets and every slot the pairs may fill come
    // back with the launch into pinned memory: one synchronisation per call
    const size_t pair_bytes = sizeof(slm_pair) * p->n_slots;
    SLM_TRY(ws_host_block(w, 80 + pair_bytes));
    unsigned char *h = w->single_host;
    SLM_CU(cudaMemcpyAsync(h, p->d_ctl.p, 64, cudaMemcpyDeviceToHost, w->stream));
    SLM_CU(cudaMemcpyAsync(h + 64, p->d_offsets.p, 16, cudaMemcpyDeviceToHost, w->stream));
    if (pair_bytes) SLM_CU(cudaMemcpyAsync(h + 80, p->d_dense.p, pair_bytes, cudaMemcpyDeviceToHost, w->stream));
    SLM_CU(cudaStreamSynchronize(w->stream));
    uint32_t ctl[16];
    std::memcpy(ctl, h, sizeof(ctl));
    SLM_TRY(status_of_word(ctl[1]));
    uint64_t off[2];
    std::memcpy(off, h + 64, sizeof(off));
    const uint64_t total = off[1];
    *n_out = (uint32_t)total;
    SLM_TRY(fill_stats(p, st, total, ctl));
    if (total > cap) return fail(SLM_CAPACITY, "need " + std::to_string(total) + " pairs, have " + std::to_string(cap));
    if (total) std::memcpy(out, h + 80, sizeof(slm_pair) * total);
    return SLM_OK;
}

namespace slm {
void launch_copy_pairs(const uint2 *src, const uint64_t *total, slm_pair *dst, uint32_t cap, uint32_t *d_count,
                       cudaStream_t s);
}

extern "C" slm_status slm_ratio_match_device(slm_ctx *c, const float *d_a, uint32_t na, const float *d_b, uint32_t nb,
                                             float ratio, int mutual, slm_precision prec, slm_pair *d_out,
                                             uint32_t cap, uint32_t *d_count) {
    NvtxRange range_("slm_ratio_match_device");
    SLM_TRY(check_pair_args(c, d_a, na, d_b, nb, ratio, prec));
    prec = resolve_prec(prec, (uint64_t)na * nb);
    if (!d_count || (cap && !d_out)) return fail(SLM_INVALID_ARG, "NULL output");
    SLM_TRY(ctx_check_device(c));
    if (na == 0 || nb < 2) {
        SLM_CU(cudaMemsetAsync(d_count, 0, sizeof(uint32_t), c->stream));
        return SLM_OK;
    }
    Workspace *w = nullptr;
    SLM_TRY(ws_acquire(c, &w));
    WsGuard guard{c, w};
    // Order the workspace stream after prior work on the context stream and
    // the context stream after this call, so the call behaves as if it ran on
    // the context stream.
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    SLM_CU(cudaEventCreateWithFlags(&e0, cudaEventDisableTiming));
    SLM_CU(cudaEventCreateWithFlags(&e1, cudaEventDisableTiming));
    SLM_CU(cudaEventRecord(e0, c->stream));
    SLM_CU(cudaStreamWaitEvent(w->stream, e0, 0));
    slm_status s = single_pair_enqueue(c, w, d_a, na, d_b, nb, ratio, mutual, prec, true);
    if (s == SLM_OK) {
        slm_plan *p = &w->plan;
        launch_copy_pairs(p->d_dense.as<uint2>(), p->d_offsets.as<uint64_t>() + 1, d_out, cap, d_count, w->stream);
        cudaError_t le = cudaGetLastError();
        if (le != cudaSuccess) s = fail(SLM_CUDA_ERROR, std::string("copy kernel: ") + cudaGetErrorString(le));
    }
    cudaEventRecord(e1, w->stream);
    cudaStreamWaitEvent(c->stream, e1, 0);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return s;
}

// ---------------------------------------------------------- pair generators

namespace {

uint64_t absdiff(uint64_t x, uint64_t y) { return x > y ? x - y : y - x; }
bool is_pow2(uint64_t d) { return d && !(d & (d - 1)); }

slm_status emit_pairs(const std::vector<slm_pair> &v, slm_pair *out, uint64_t cap, uint64_t *n_out) {
    *n_out = v.size();
    const uint64_t n = std::min<uint64_t>(cap, v.size());
    if (n) std::memcpy(out, v.data(), n * sizeof(slm_pair));
    if (v.size() > cap) return fail(SLM_CAPACITY, "need " + std::to_string(v.size()) + " pairs");
    return SLM_OK;
}

}  // namespace

// matching.rs:18-40: same camera with position gap 1..=temporal or a power of
// two <= pow2_max; different cameras with gap <= cross. i < j, sorted, unique.
extern "C" slm_status slm_candidate_pairs(const uint64_t *views, uint32_t nv, uint64_t temporal, uint64_t cross,
                                          uint64_t pow2_max, slm_pair *out, uint64_t cap, uint64_t *n_out) {
    if ((!views && nv) || !n_out || (cap && !out)) return fail(SLM_INVALID_ARG, "NULL argument");
    std::vector<slm_pair> v;
    for (uint32_t i = 0; i < nv; ++i)
        for (uint32_t j = i + 1; j < nv; ++j) {
            const uint64_t ca = views[2 * i], pa = views[2 * i + 1], cb = views[2 * j], pb = views[2 * j + 1];
            const uint64_t d = absdiff(pa, pb);
            const bool ok = ca == cb ? (d >= 1 && (d <= temporal || (is_pow2(d) && d <= pow2_max))) : d <= cross;
            if (ok) v.push_back(slm_pair{i, j});
        }
    return emit_pairs(v, out, cap, n_out);
}

extern "C" slm_pair_schedule slm_pair_schedule_default(void) {
    slm_pair_schedule s{};
    s.temporal = 5;
    s.pow2_max = 16;
    s.spec = 0;
    s.range = 4;
    s.right_min = 20;
    s.left_min = 20;
    s.max = 40;
    s.step = 4;
    return s;
}

extern "C" slm_pair_schedule slm_pair_schedule_spec(void) {
    slm_pair_schedule s = slm_pair_schedule_default();
    s.spec = 1;
    s.range = 4;
    return s;
}

// matching.rs:103-142. Cameras: front 0, right 1, left 2 (matching.rs:42-45).
extern "C" slm_status slm_scheduled_pairs(const uint64_t *views, uint32_t nv, const slm_pair_schedule *sch,
                                          slm_pair *out, uint64_t cap, uint64_t *n_out) {
    if ((!views && nv) || !sch || !n_out || (cap && !out)) return fail(SLM_INVALID_ARG, "NULL argument");
    std::vector<slm_pair> v;
    for (uint32_t i = 0; i < nv; ++i)
        for (uint32_t j = 0; j < nv; ++j) {
            if (i == j) continue;
            const uint64_t ca = views[2 * i], pa = views[2 * i + 1], cb = views[2 * j], pb = views[2 * j + 1];
            const uint64_t d = absdiff(pa, pb);
            bool ok;
            if (ca == cb) {
                ok = j > i && d >= 1 && (d <= sch->temporal || (is_pow2(d) && d <= sch->pow2_max));
            } else if (sch->spec) {
                ok = j > i && d <= sch->range;
            } else {
                bool has = false;
                uint64_t lo = 0;
                if (ca == 0 && cb == 1) has = true, lo = sch->right_min;
                if (ca == 0 && cb == 2) has = true, lo = sch->left_min;
                const uint64_t step = std::max<uint64_t>(sch->step, 1);
                ok = has && pb >= pa + lo && pb <= pa + sch->max && (pb - pa - lo) % step == 0;
            }
            if (ok) v.push_back(slm_pair{std::min(i, j), std::max(i, j)});
        }
    std::sort(v.begin(), v.end(), [](const slm_pair &x, const slm_pair &y) {
        return x.i != y.i ? x.i < y.i : x.j < y.j;
    });
    v.erase(std::unique(v.begin(), v.end(), [](const slm_pair &x, const slm_pair &y) {
                return x.i == y.i && x.j == y.j;
            }),
            v.end());
    return emit_pairs(v, out, cap, n_out);
}

extern "C" slm_status slm_plan_debug_dump(slm_plan *p, float *out, uint64_t cap) {
    if (!p || (cap && !out)) return fail(SLM_INVALID_ARG, "NULL argument");
    if (!p->dump || !p->np) return fail(SLM_INVALID_ARG, "plan was not created with the dump variant");
    const uint64_t n = (uint64_t)p->meta[0].na * p->meta[0].nb;
    if (n > cap) return fail(SLM_CAPACITY, "need " + std::to_string(n) + " floats");
    SLM_CU(cudaStreamSynchronize(p->stream));
    if (n) SLM_CU(cudaMemcpy(out, p->d_dump.p, n * sizeof(float), cudaMemcpyDeviceToHost));
    return SLM_OK;
}

// ----------------------------------------------------------------- serving

#include <chrono>
#include <condition_variable>
#include <deque>
#include <thread>
#include <unordered_map>

namespace {

using Clock = std::chrono::steady_clock;

struct ServeRequest {
    uint64_t ticket = 0;
    uint32_t view = 0;
    std::vector<float> desc;         // host copy (slm_server_submit), kept until the batch is done
    const float *src = nullptr;      // the view's rows: desc.data(), or the caller's (slm_server_submit_ptr)
    uint32_t n = 0;                  // rows of the view
    bool dropped = false;            // cancelled while queued: uploaded (later requests may name it), no pairs
    std::vector<slm_pair> pairs;     // SLM_SELF resolved to `view`
    std::vector<slm_pair> matches;   // results, pair order
    std::vector<uint64_t> offsets;   // np + 1
    Clock::time_point t_submit, t_done;
    bool uploaded = false, done = false;
    bool cancelled = false;          // slm_server_cancel: results are not kept
    slm_status status = SLM_OK;
    std::string error;
};

struct ServeSlot {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    slm_plan plan;
    std::vector<ServeRequest *> reqs;
    uint32_t np = 0;                 // pairs of the running batch (0: uploads of dropped requests only)
    bool busy = false;
    slm_pair *pin = nullptr;         // pinned staging of a finished batch's matches (grows)
    uint64_t pin_cap = 0;
    uint64_t *pin_off = nullptr;     // pinned staging of its per-pair offsets (grows)
    uint64_t pin_off_cap = 0;
    // Outgrown staging blocks, freed with the slot: cudaFreeHost waits for
    // the whole device, which would stall the worker behind the other slots.
    std::vector<void *> retired;
    ~ServeSlot() {
        if (pin) cudaFreeHost(pin);
        if (pin_off) cudaFreeHost(pin_off);
        for (void *q : retired) cudaFreeHost(q);
    }
    // Grows a pinned block to hold `need` elements (half as much again).
    template <class T>
    slm_status grow(T *&buf, uint64_t &cap, uint64_t need) {
        if (need <= cap) return SLM_OK;
        if (buf) retired.push_back(buf);
        buf = nullptr;
        cap = 0;
        const uint64_t want = need + need / 2;
        SLM_CU(cudaMallocHost(reinterpret_cast<void **>(&buf), sizeof(T) * want));
        cap = want;
        return SLM_OK;
    }
};

// A finished batch's matches and per-pair offsets into the slot's pinned
// staging: only the matches the batch found cross the link, in one copy.
slm_status serve_read_results(ServeSlot *s, std::vector<uint64_t> &off) {
    slm_plan *p = &s->plan;
    SLM_CU(cudaStreamSynchronize(p->stream));
    SLM_TRY(check_status_word(p));
    SLM_TRY(s->grow(s->pin_off, s->pin_off_cap, p->np + 1));
    SLM_CU(cudaMemcpyAsync(s->pin_off, p->d_offsets.p, sizeof(uint64_t) * (p->np + 1), cudaMemcpyDeviceToHost,
                           p->stream));
    SLM_CU(cudaStreamSynchronize(p->stream));
    off.assign(s->pin_off, s->pin_off + p->np + 1);
    const uint64_t total = off[p->np];
    SLM_TRY(s->grow(s->pin, s->pin_cap, total));
    if (total) {
        SLM_CU(cudaMemcpyAsync(s->pin, p->d_dense.p, sizeof(slm_pair) * total, cudaMemcpyDeviceToHost, p->stream));
        SLM_CU(cudaStreamSynchronize(p->stream));
    }
    return SLM_OK;
}

}  // namespace

struct slm_server {
    slm_ctx *ctx = nullptr;
    slm_store *store = nullptr;
    slm_server_opts opts{};
    std::vector<ServeSlot *> slots;
    cudaEvent_t upload_done = nullptr;  // last store upload
    std::thread worker;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<ServeRequest *> pending;
    std::unordered_map<uint64_t, ServeRequest *> reqs;
    uint64_t next_ticket = 1;
    uint32_t next_view = 0;
    uint64_t slot_budget = 0;
    std::vector<uint32_t> view_n;       // rows of every submitted view, by view id (admission)
    bool stop = false;
    slm_server_stats stats{};
};

namespace {

// Scratch a batch needs (matches plan_build_shortlist's and plan_build's
// allocations; used for admission).
uint64_t batch_bytes(const slm_store *st, const std::vector<uint32_t> &vn, const std::vector<slm_pair> &pairs,
                     slm_precision prec) {
    uint64_t rows = 0, cols = 0, na = 0, items = 0, supers = 0, cand_rows = 0;
    for (const slm_pair &p : pairs) {
        const uint64_t a = p.i < vn.size() ? vn[p.i] : 0, b = p.j < vn.size() ? vn[p.j] : 0;
        if (b) supers += (a + 2 * kTile - 1) / (2 * kTile);
    }
    // column ranges per pair as plan_build_shortlist splits them (default items per SM)
    const uint64_t want = (uint64_t)std::max(1, st->ctx->sms) * 3;
    const uint64_t split = supers && supers < want ? (want + supers - 1) / supers : 1;
    for (const slm_pair &p : pairs) {
        const uint64_t a = p.i < vn.size() ? vn[p.i] : 0, b = p.j < vn.size() ? vn[p.j] : 0;
        rows += pad_rows(a);
        cols += pad_rows(b);
        na += a;
        items += (pad_rows(a) / kTile + 1) * 4;
        cand_rows += pad_rows(a) *
                     std::max<uint64_t>(1, std::min<uint64_t>(std::min<uint64_t>(split, pad_rows(b) / kTile), kSlMaxRanges));
    }
    uint64_t bytes = 64 + pairs.size() * (sizeof(PairMeta) + 16 + 8) + na * 16 + cols * 8;
    if (prec == SLM_PREC_FP32)
        bytes += items * (sizeof(Item) + sizeof(RowPart) * kTile);
    else
        bytes += rows * 3 * 4 + cand_rows * (2 * 4 + 2 * kSlHalfRecs * 20) + cols * 12 + na * 2 * sizeof(SlQueue) +
                 items * 256 * 12 +
                 pairs.size() * (4 + 16) + (rows / kSlRowBlock + pairs.size()) * 4 +
                 (rows / kTile + 4ull * (uint64_t)std::max(1, st->ctx->sms)) * (sizeof(Item) + sizeof(RowPart) * kTile);
    return bytes + bytes / 4;  // DevBuf growth slack
}

void serve_fail_request(ServeRequest *r, slm_status s, const std::string &error) {
    r->status = s;
    r->error = error;
    r->done = true;
    r->t_done = Clock::now();
    std::vector<slm_pair>().swap(r->matches);
    std::vector<uint64_t>().swap(r->offsets);
}

// The views of a batch's requests, in submission order (their ids were given
// at submit): one gather launch that reads every view where it lies when the
// device can read host memory directly and the rows are 16-byte aligned, else
// one copy per view. On the store's stream.
slm_status serve_upload(slm_server *srv, const std::vector<ServeRequest *> &take) {
    slm_store *st = srv->store;
    bool direct = srv->ctx->host_direct;
    for (const ServeRequest *r : take) direct &= (reinterpret_cast<uintptr_t>(r->src) & 15u) == 0;
    std::vector<uint32_t> ids(take.size());
    if (direct) {
        std::vector<const float *> src(take.size());
        std::vector<uint32_t> n(take.size());
        for (size_t k = 0; k < take.size(); ++k) src[k] = take[k]->src, n[k] = take[k]->n;
        SLM_TRY(store_append_direct(st, take.size(), src.data(), n.data(), ids.data(), srv->ctx->stream));
    } else {
        for (size_t k = 0; k < take.size(); ++k)
            SLM_TRY(store_append(st, take[k]->src, take[k]->n, false, srv->ctx->stream, &ids[k]));
    }
    for (size_t k = 0; k < take.size(); ++k)
        if (ids[k] != take[k]->view) return fail(SLM_INTERNAL, "serving: view ids out of order");
    return SLM_OK;
}

// Worker: collect finished batches, then admit pending requests into free
// slots. The lock is held only to move requests between the queue and the
// slots and to publish results: uploads, planning, launches and result copies
// run without it, so clients submit and wait meanwhile, and the requests that
// arrive while the worker is busy make the next batch larger.
void serve_loop(slm_server *srv) {
    cudaSetDevice(srv->ctx->device);
    std::unique_lock<std::mutex> lk(srv->mu);
    while (true) {
        // Sleep one tick (completions are polled every tick) unless a new
        // request can start right away.
        srv->cv_work.wait_for(lk, std::chrono::microseconds(srv->opts.tick_us), [&] {
            if (srv->stop) return true;
            if (srv->pending.empty()) return false;
            for (ServeSlot *s : srv->slots)
                if (!s->busy) return true;
            return false;
        });
        if (srv->stop) {
            bool busy = false;
            for (ServeSlot *s : srv->slots) busy |= s->busy;
            if (!busy && srv->pending.empty()) break;
        }
        // 1. completions: results copied out without the lock, published with it
        std::vector<ServeSlot *> fin;
        for (ServeSlot *s : srv->slots) {
            if (!s->busy) continue;
            if (cudaEventQuery(s->done) == cudaSuccess) fin.push_back(s);
            cudaGetLastError();  // cudaErrorNotReady
        }
        if (!fin.empty()) {
            lk.unlock();
            std::vector<slm_status> rs(fin.size(), SLM_OK);
            std::vector<std::string> err(fin.size());
            for (size_t f = 0; f < fin.size(); ++f) {
                ServeSlot *s = fin[f];
                if (!s->np) {  // requests without pairs (the first views of a zone)
                    for (ServeRequest *r : s->reqs) r->offsets.assign(1, 0), r->matches.clear();
                    continue;
                }
                std::vector<uint64_t> off;
                rs[f] = serve_read_results(s, off);
                if (rs[f] != SLM_OK) {
                    err[f] = g_last_error;
                    continue;
                }
                uint32_t k = 0;
                for (ServeRequest *r : s->reqs) {
                    if (r->dropped) continue;
                    const uint64_t b0 = off[k];
                    r->matches.assign(s->pin + b0, s->pin + off[k + r->pairs.size()]);
                    r->offsets.resize(r->pairs.size() + 1);
                    for (size_t q = 0; q <= r->pairs.size(); ++q) r->offsets[q] = off[k + q] - b0;
                    k += (uint32_t)r->pairs.size();
                }
            }
            lk.lock();
            for (size_t f = 0; f < fin.size(); ++f) {
                ServeSlot *s = fin[f];
                for (ServeRequest *r : s->reqs) {
                    std::vector<float>().swap(r->desc);  // the upload has read it
                    if (r->cancelled || r->dropped)
                        serve_fail_request(r, SLM_CANCELLED, "request cancelled");
                    else if (rs[f] != SLM_OK)
                        serve_fail_request(r, rs[f], err[f]);
                    else {
                        r->done = true;
                        r->t_done = Clock::now();
                        srv->stats.completed++;
                        srv->stats.matches += r->matches.size();
                    }
                }
                s->reqs.clear();
                s->busy = false;
            }
            srv->cv_done.notify_all();
        }
        // 2. admission: FIFO into each free slot while the batch fits
        for (ServeSlot *s : srv->slots) {
            if (s->busy || srv->pending.empty()) continue;
            std::vector<ServeRequest *> take;
            std::vector<slm_pair> pairs;
            while (!srv->pending.empty()) {
                ServeRequest *r = srv->pending.front();
                if (r->cancelled) {
                    r->dropped = true;  // its view is still added to the store (later requests may name it)
                } else {
                    if (!pairs.empty() && pairs.size() + r->pairs.size() > srv->opts.max_batch_pairs) break;
                    std::vector<slm_pair> trial = pairs;
                    trial.insert(trial.end(), r->pairs.begin(), r->pairs.end());
                    if (!pairs.empty() && batch_bytes(srv->store, srv->view_n, trial, srv->opts.prec) > srv->slot_budget)
                        break;
                    pairs.swap(trial);
                }
                take.push_back(r);
                srv->pending.pop_front();
            }
            if (take.empty()) continue;
            lk.unlock();
            // the new views, their FP32 tiles and low-precision images on the
            // store's stream, so every slot that waits for the upload sees them
            slm_status ps = serve_upload(srv, take);
            if (ps == SLM_OK && srv->opts.prec != SLM_PREC_BF16) ps = store_sync_fp32(srv->store, srv->ctx->stream);
            if (ps == SLM_OK) ps = store_sync_plan_images(srv->store, srv->opts.prec, srv->ctx->stream);
            if (ps == SLM_OK && cudaEventRecord(srv->upload_done, srv->ctx->stream) != cudaSuccess)
                ps = fail(SLM_CUDA_ERROR, "cudaEventRecord");
            if (ps == SLM_OK && cudaStreamWaitEvent(s->stream, srv->upload_done, 0) != cudaSuccess)
                ps = fail(SLM_CUDA_ERROR, "cudaStreamWaitEvent");
            if (ps == SLM_OK && !pairs.empty()) {
                slm_tune t{};
                t.use_graph = 2;
                ps = plan_init(&s->plan, srv->ctx, srv->store, pairs.data(), (uint32_t)pairs.size(), srv->opts.ratio,
                               srv->opts.mutual, srv->opts.prec, &t, s->stream);
                if (ps == SLM_OK) ps = plan_launch_on(&s->plan, s->stream, false);
            }
            if (ps == SLM_OK && cudaEventRecord(s->done, s->stream) != cudaSuccess)
                ps = fail(SLM_CUDA_ERROR, "cudaEventRecord");
            const std::string err = ps == SLM_OK ? std::string() : g_last_error;
            if (ps != SLM_OK) cudaStreamSynchronize(srv->ctx->stream);  // no upload still reads a request's rows
            lk.lock();
            if (ps != SLM_OK) {
                for (ServeRequest *r : take) serve_fail_request(r, ps, err);
                srv->cv_done.notify_all();
                continue;
            }
            s->reqs = take;
            s->np = (uint32_t)pairs.size();
            s->busy = true;
            srv->stats.batches++;
            srv->stats.pairs += pairs.size();
            srv->stats.max_batch_requests = std::max<uint64_t>(srv->stats.max_batch_requests, take.size());
            uint64_t inflight = 0;
            for (ServeSlot *q : srv->slots) inflight += q->busy;
            srv->stats.max_inflight = std::max(srv->stats.max_inflight, inflight);
        }
    }
}

}  // namespace

extern "C" slm_status slm_server_create(const slm_server_opts *opts, slm_server **out) {
    if (!opts || !out) return fail(SLM_INVALID_ARG, "NULL argument");
    *out = nullptr;
    if (!prec_valid(opts->prec)) return fail(SLM_INVALID_ARG, "unknown precision");
    SLM_TRY(validate_ratio(opts->ratio));
    auto *srv = new (std::nothrow) slm_server();
    if (!srv) return fail(SLM_OOM, "host allocation failed");
    srv->opts = *opts;
    if (!srv->opts.slots) srv->opts.slots = 3;
    if (!srv->opts.max_batch_pairs) srv->opts.max_batch_pairs = 256;
    if (!srv->opts.tick_us) srv->opts.tick_us = 200;
    slm_opts co{};
    co.device = opts->device;
    co.hbm_budget = opts->hbm_budget;
    slm_status s = slm_ctx_create(&co, &srv->ctx);
    if (s == SLM_OK && !opts->hbm_budget) srv->ctx->budget = srv->ctx->budget / 5 * 4;
    if (s == SLM_OK) s = slm_store_create(srv->ctx, opts->max_descs, opts->max_views, &srv->store);
    if (s == SLM_OK && cudaEventCreateWithFlags(&srv->upload_done, cudaEventDisableTiming) != cudaSuccess)
        s = fail(SLM_CUDA_ERROR, "cudaEventCreate");
    for (uint32_t k = 0; s == SLM_OK && k < srv->opts.slots; ++k) {
        auto *sl = new ServeSlot();
        srv->slots.push_back(sl);
        if (cudaStreamCreateWithFlags(&sl->stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&sl->done, cudaEventDisableTiming) != cudaSuccess)
            s = fail(SLM_CUDA_ERROR, "stream/event creation failed");
        sl->plan.ctx = srv->ctx;
        // staging for a full batch of typical pairs (up to 2048 matches each),
        // so a burst does not grow pinned memory while other slots run
        if (s == SLM_OK) s = sl->grow(sl->pin, sl->pin_cap, uint64_t(srv->opts.max_batch_pairs) * 1366);
        if (s == SLM_OK) s = sl->grow(sl->pin_off, sl->pin_off_cap, uint64_t(srv->opts.max_batch_pairs) + 1);
    }
    if (s != SLM_OK) {
        std::string keep = g_last_error;
        slm_server_destroy(srv);
        g_last_error = keep;
        return s;
    }
    // the store's operand images for its whole capacity now, not in the first
    // batch (with no views yet this allocates and packs nothing else)
    if (s == SLM_OK) s = store_sync_plan_images(srv->store, srv->opts.prec, srv->ctx->stream);
    if (s == SLM_OK && cudaStreamSynchronize(srv->ctx->stream) != cudaSuccess)
        s = fail(SLM_CUDA_ERROR, "cudaStreamSynchronize");
    if (s != SLM_OK) {
        std::string keep = g_last_error;
        slm_server_destroy(srv);
        g_last_error = keep;
        return s;
    }
    const uint64_t used = srv->ctx->used.load();
    const uint64_t left = srv->ctx->budget > used ? srv->ctx->budget - used : 0;
    srv->slot_budget = left / srv->opts.slots;
    // Map the slots' scratch into the context's pool now (up to the 1 GiB it
    // keeps): the first batches then take their buffers from memory already
    // mapped instead of growing the pool while other slots run.
    if (srv->ctx->pool) {
        void *warm = nullptr;
        const uint64_t want = std::min<uint64_t>(left, 1ull << 30);
        if (want && srv->ctx->alloc_ordered(&warm, want, srv->ctx->stream) == SLM_OK) {
            srv->ctx->release_ordered(warm, want, srv->ctx->stream);
            cudaStreamSynchronize(srv->ctx->stream);
        }
        g_last_error.clear();
        cudaGetLastError();
    }
    srv->worker = std::thread(serve_loop, srv);
    *out = srv;
    return SLM_OK;
}

extern "C" slm_status slm_server_destroy(slm_server *srv) {
    if (!srv) return SLM_OK;
    if (srv->worker.joinable()) {
        {
            std::lock_guard<std::mutex> g(srv->mu);
            srv->stop = true;
        }
        srv->cv_work.notify_all();
        srv->worker.join();
    }
    if (srv->ctx) cudaSetDevice(srv->ctx->device);
    for (ServeSlot *s : srv->slots) {
        if (s->stream) cudaStreamSynchronize(s->stream);
        if (s->plan.ev0) {
            cudaEventDestroy(s->plan.ev0);
            s->plan.ev0 = nullptr;
        }
        if (s->plan.ev1) {
            cudaEventDestroy(s->plan.ev1);
            s->plan.ev1 = nullptr;
        }
        if (s->done) cudaEventDestroy(s->done);
        plan_release(&s->plan);
        if (s->stream) cudaStreamDestroy(s->stream);
        delete s;
    }
    for (auto &kv : srv->reqs) delete kv.second;
    if (srv->upload_done) cudaEventDestroy(srv->upload_done);
    if (srv->store) slm_store_destroy(srv->store);
    if (srv->ctx) slm_ctx_destroy(srv->ctx);
    delete srv;
    return SLM_OK;
}

namespace {
slm_status server_submit(slm_server *srv, const float *desc, uint32_t n, bool copy, const slm_pair *pairs,
                         uint32_t np, uint32_t *view_id, uint64_t *ticket) {
    if (!srv || (n && !desc) || (np && !pairs) || !ticket) return fail(SLM_INVALID_ARG, "NULL argument");
    auto *r = new (std::nothrow) ServeRequest();
    if (!r) return fail(SLM_OOM, "host allocation failed");
    if (copy) {
        r->desc.assign(desc, desc + (size_t)n * kDesc);
        r->src = r->desc.data();
    } else {
        r->src = desc;
    }
    r->n = n;
    r->t_submit = Clock::now();
    std::lock_guard<std::mutex> g(srv->mu);
    if (srv->next_view >= srv->opts.max_views) {
        delete r;
        return fail(SLM_CAPACITY, "server store is full (max_views)");
    }
    r->view = srv->next_view;
    for (uint32_t k = 0; k < np; ++k) {
        slm_pair p = pairs[k];
        if (p.i == SLM_SELF) p.i = r->view;
        if (p.j == SLM_SELF) p.j = r->view;
        if (p.i > r->view || p.j > r->view) {
            delete r;
            return fail(SLM_INVALID_ARG, "pair names a view not yet submitted");
        }
        r->pairs.push_back(p);
    }
    srv->view_n.push_back(n);
    srv->next_view++;
    r->ticket = srv->next_ticket++;
    srv->reqs[r->ticket] = r;
    srv->pending.push_back(r);
    srv->stats.submitted++;
    if (view_id) *view_id = r->view;
    *ticket = r->ticket;
    srv->cv_work.notify_all();
    return SLM_OK;
}
}  // namespace

extern "C" slm_status slm_server_submit(slm_server *srv, const float *desc, uint32_t n, const slm_pair *pairs,
                                        uint32_t np, uint32_t *view_id, uint64_t *ticket) {
    return server_submit(srv, desc, n, true, pairs, np, view_id, ticket);
}

extern "C" slm_status slm_server_submit_ptr(slm_server *srv, const float *desc, uint32_t n, const slm_pair *pairs,
                                            uint32_t np, uint32_t *view_id, uint64_t *ticket) {
    return server_submit(srv, desc, n, false, pairs, np, view_id, ticket);
}

extern "C" slm_status slm_server_wait(slm_server *srv, uint64_t ticket, uint32_t timeout_ms, slm_pair *out,
                                      uint64_t cap, uint64_t *offsets, double *latency_ms) {
    if (!srv || (cap && !out) || !offsets) return fail(SLM_INVALID_ARG, "NULL argument");
    std::unique_lock<std::mutex> lk(srv->mu);
    auto it = srv->reqs.find(ticket);
    if (it == srv->reqs.end()) return fail(SLM_INVALID_ARG, "unknown ticket");
    ServeRequest *r = it->second;
    if (!srv->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return r->done; }))
        return fail(SLM_TIMEOUT, "request not finished");
    if (r->status != SLM_OK) {
        const slm_status s = r->status;
        g_last_error = r->error;
        srv->reqs.erase(it);
        delete r;
        return s;
    }
    if (r->matches.size() > cap) return fail(SLM_CAPACITY, "need " + std::to_string(r->matches.size()) + " pairs");
    std::copy(r->offsets.begin(), r->offsets.end(), offsets);
    std::copy(r->matches.begin(), r->matches.end(), out);
    if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
    srv->reqs.erase(it);
    delete r;
    return SLM_OK;
}

extern "C" slm_status slm_server_cancel(slm_server *srv, uint64_t ticket) {
    if (!srv) return fail(SLM_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> g(srv->mu);
    auto it = srv->reqs.find(ticket);
    if (it == srv->reqs.end()) return fail(SLM_INVALID_ARG, "unknown ticket");
    ServeRequest *r = it->second;
    r->cancelled = true;
    if (r->done && r->status == SLM_OK) {  // finished: drop the results
        r->status = SLM_CANCELLED;
        r->error = "request cancelled";
        std::vector<slm_pair>().swap(r->matches);
        std::vector<uint64_t>().swap(r->offsets);
    }
    srv->cv_work.notify_all();
    return SLM_OK;
}

extern "C" slm_status slm_server_stats_get(slm_server *srv, slm_server_stats *st) {
    if (!srv || !st) return fail(SLM_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> g(srv->mu);
    *st = srv->stats;
    st->bytes_in_use = srv->ctx->used.load();
    return SLM_OK;
}

// --------------------------------------------------------- Sampson scoring

extern "C" slm_status slm_sampson_score(slm_ctx *c, const double *pts, const uint64_t *pair_off, uint32_t np,
                                        const double *thresh, const double *E, const uint32_t *hyp_pair, uint32_t nh,
                                        uint32_t *counts, const uint64_t *mask_off, uint32_t *masks,
                                        uint64_t mask_words) {
    NvtxRange range_("slm_sampson_score");
    if (!c || (np && !thresh) || !pair_off || (nh && (!E || !hyp_pair || !counts)) ||
        (mask_off && mask_words && !masks))
        return fail(SLM_INVALID_ARG, "NULL argument");
    for (uint32_t q = 0; q < np; ++q)
        if (pair_off[q + 1] < pair_off[q]) return fail(SLM_INVALID_ARG, "pair_off must not decrease");
    const uint64_t m = pair_off[np];
    if (pair_off[0] != 0) return fail(SLM_INVALID_ARG, "pair_off[0] must be 0");
    if (m && !pts) return fail(SLM_INVALID_ARG, "NULL pts");
    for (uint32_t h = 0; h < nh; ++h) {
        if (hyp_pair[h] >= np) return fail(SLM_INVALID_ARG, "hyp_pair names no pair");
        if (mask_off && mask_off[h] != ~0ull) {
            const uint64_t n = pair_off[hyp_pair[h] + 1] - pair_off[hyp_pair[h]];
            if (mask_off[h] > mask_words || (n + 31) / 32 > mask_words - mask_off[h])
                return fail(SLM_INVALID_ARG, "a mask does not fit in mask_words");
        }
    }
    if (!nh) return SLM_OK;
    SLM_TRY(ctx_check_device(c));
    Workspace *w = nullptr;
    SLM_TRY(ws_acquire(c, &w));
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    const size_t o_pts = 0, o_off = al(o_pts + 32 * m), o_th = al(o_off + 8 * (uint64_t)(np + 1)),
                 o_e = al(o_th + 8 * (uint64_t)np), o_hp = al(o_e + 72 * (uint64_t)nh),
                 o_cnt = al(o_hp + 4 * (uint64_t)nh), o_moff = al(o_cnt + 4 * (uint64_t)nh),
                 o_mask = al(o_moff + (mask_off ? 8 * (uint64_t)nh : 0)),
                 bytes = al(o_mask + (mask_off ? 4 * mask_words : 0));
    slm_status st = w->score.ensure(c, bytes);
    if (st == SLM_OK) {
        unsigned char *d = w->score.as<unsigned char>();
        cudaStream_t s = w->stream;
        auto up = [&](size_t off, const void *src, size_t n) {
            return n ? cudaMemcpyAsync(d + off, src, n, cudaMemcpyHostToDevice, s) : cudaSuccess;
        };
        cudaError_t e = up(o_pts, pts, 32 * m);
        if (e == cudaSuccess) e = up(o_off, pair_off, 8 * (uint64_t)(np + 1));
        if (e == cudaSuccess) e = up(o_th, thresh, 8 * (uint64_t)np);
        if (e == cudaSuccess) e = up(o_e, E, 72 * (uint64_t)nh);
        if (e == cudaSuccess) e = up(o_hp, hyp_pair, 4 * (uint64_t)nh);
        if (e == cudaSuccess && mask_off) e = up(o_moff, mask_off, 8 * (uint64_t)nh);
        if (e == cudaSuccess && mask_off && mask_words) e = cudaMemsetAsync(d + o_mask, 0, 4 * mask_words, s);
        if (e == cudaSuccess) {
            SampsonArgs a{};
            a.pts = reinterpret_cast<const double4 *>(d + o_pts);
            a.pair_off = reinterpret_cast<const uint64_t *>(d + o_off);
            a.thresh = reinterpret_cast<const double *>(d + o_th);
            a.E = reinterpret_cast<const double *>(d + o_e);
            a.hyp_pair = reinterpret_cast<const uint32_t *>(d + o_hp);
            a.nh = nh;
            a.counts = reinterpret_cast<uint32_t *>(d + o_cnt);
            a.mask_off = mask_off ? reinterpret_cast<const uint64_t *>(d + o_moff) : nullptr;
            a.masks = mask_off ? reinterpret_cast<uint32_t *>(d + o_mask) : nullptr;
            launch_sampson(a, s);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(counts, d + o_cnt, 4 * (uint64_t)nh, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess && mask_off && mask_words)
            e = cudaMemcpyAsync(masks, d + o_mask, 4 * mask_words, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) st = fail(SLM_CUDA_ERROR, std::string("slm_sampson_score: ") + cudaGetErrorString(e));
    }
    ws_release(c, w);
    return st;
}

// ------------------------------------------------------------- coalescing
//
// Concurrent single-pair calls (the reference's rayon workers call
// ratio_match once per pair, matching.rs:167 from pipeline.rs:487-493) are
// queued when coalescing is on: a worker thread gathers the waiting calls into
// one batch plan (each call's two arrays become two views of the batch's
// store), runs it on one of two slots so that one batch gathers while the
// other runs, and hands every caller its own list. Results are those of the
// call made alone (every precision is bit-exact).

namespace {

struct CoalReq {
    const float *a = nullptr, *b = nullptr;
    uint32_t na = 0, nb = 0;
    float ratio = 0.f;
    int mutual = 0;
    slm_pair *out = nullptr;
    uint32_t cap = 0;
    uint32_t *n_out = nullptr;
    slm_stats *st = nullptr;
    slm_status status = SLM_OK;
    std::string error;
    bool done = false;
    Clock::time_point t_submit;
};

struct CoalSlot {
    Workspace w;
    cudaEvent_t done = nullptr;
    std::vector<CoalReq *> reqs;
    bool busy = false;
    // pinned host copy of a finished batch: [error word, pad, offsets (np + 1), pairs]
    void *host = nullptr;
    size_t host_bytes = 0;
    ~CoalSlot() {
        if (host) cudaFreeHost(host);
    }
};

}  // namespace

struct Coalescer {
    slm_ctx *ctx = nullptr;
    uint32_t window_us = 0, max_pairs = 0;
    CoalSlot slots[2];
    std::thread worker;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<CoalReq *> pending;
    Clock::time_point last_arrival;
    bool stop = false;
    uint64_t batches = 0, pairs = 0, max_batch = 0;
};

namespace {

void coal_finish(Coalescer *co, CoalReq *r, slm_status s, const std::string &err) {
    r->status = s;
    r->error = err;
    r->done = true;
}

// Results of a finished slot, distributed to its callers (called with co->mu held).
void coal_collect(Coalescer *co, CoalSlot *s) {
    slm_plan *p = &s->w.plan;
    const uint32_t *hw = static_cast<const uint32_t *>(s->host);
    const uint64_t *off = reinterpret_cast<const uint64_t *>(hw + 2);
    const slm_pair *dense = reinterpret_cast<const slm_pair *>(off + p->np + 1);
    slm_status rs = SLM_OK;
    if (cudaEventQuery(s->done) != cudaSuccess) {
        cudaGetLastError();
        rs = fail(SLM_CUDA_ERROR, "batch failed on the device");
    } else if (hw[0] == DERR_TIMEOUT_BAR || hw[0] == DERR_TIMEOUT_MMA) {
        rs = fail(SLM_TIMEOUT, "device wait gave up (code " + std::to_string(hw[0]) + ")");
    } else if (hw[0]) {
        rs = fail(SLM_INTERNAL, "device invariant failed (code " + std::to_string(hw[0]) + ")");
    }
    const std::string err = rs == SLM_OK ? std::string() : g_last_error;
    for (size_t k = 0; k < s->reqs.size(); ++k) {
        CoalReq *r = s->reqs[k];
        if (rs != SLM_OK) {
            coal_finish(co, r, rs, err);
            continue;
        }
        const uint64_t n = off[k + 1] - off[k];
        *r->n_out = (uint32_t)n;
        if (r->st) {
            std::memset(r->st, 0, sizeof(*r->st));
            r->st->pairs = 1;
            r->st->distances = (uint64_t)r->na * r->nb;
            r->st->matches = n;
        }
        if (n > r->cap) {
            coal_finish(co, r, SLM_CAPACITY, "need " + std::to_string(n) + " pairs, have " + std::to_string(r->cap));
            continue;
        }
        if (n) std::memcpy(r->out, dense + off[k], sizeof(slm_pair) * n);
        coal_finish(co, r, SLM_OK, std::string());
    }
    s->reqs.clear();
    s->busy = false;
}

// Upload, plan and launch one batch on a free slot (called with co->mu held).
slm_status coal_issue(Coalescer *co, CoalSlot *s, std::vector<CoalReq *> &take) {
    slm_ctx *c = co->ctx;
    Workspace *w = &s->w;
    uint64_t rows = 0, dist = 0;
    for (CoalReq *r : take) {
        rows += pad_rows(r->na) + pad_rows(r->nb);
        dist += (uint64_t)r->na * r->nb;
    }
    slm_store *st = &w->store;
    SLM_TRY(store_reserve(st, std::max<uint64_t>(rows, kTile)));
    slm_store_clear(st);
    std::vector<slm_pair> pr(take.size());
    bool direct = c->host_direct;
    for (CoalReq *r : take) direct &= ((reinterpret_cast<uintptr_t>(r->a) | reinterpret_cast<uintptr_t>(r->b)) & 15) == 0;
    if (direct) {
        // one kernel reads every caller's arrays where they lie (no copies by this thread)
        std::vector<const float *> src(2 * take.size());
        std::vector<uint32_t> n(2 * take.size()), ids(2 * take.size());
        for (size_t k = 0; k < take.size(); ++k) {
            src[2 * k] = take[k]->a, n[2 * k] = take[k]->na;
            src[2 * k + 1] = take[k]->b, n[2 * k + 1] = take[k]->nb;
        }
        SLM_TRY(store_append_direct(st, src.size(), src.data(), n.data(), ids.data(), w->stream));
        for (size_t k = 0; k < take.size(); ++k) pr[k] = slm_pair{ids[2 * k], ids[2 * k + 1]};
    } else {
        for (size_t k = 0; k < take.size(); ++k) {
            SLM_TRY(store_append(st, take[k]->a, take[k]->na, false, w->stream, &pr[k].i));
            SLM_TRY(store_append(st, take[k]->b, take[k]->nb, false, w->stream, &pr[k].j));
        }
    }
    slm_tune t{};
    t.use_graph = 2;  // a new shape every batch: plain launches
    SLM_TRY(plan_init(&w->plan, c, st, pr.data(), (uint32_t)pr.size(), take[0]->ratio, take[0]->mutual,
                      resolve_prec(SLM_PREC_AUTO, dist), &t, w->stream));
    SLM_TRY(plan_launch_on(&w->plan, w->stream, false));
    // results come back with the batch: one pinned copy of the error word,
    // the offsets and every slot the pairs may fill
    slm_plan *p = &w->plan;
    const size_t off_bytes = sizeof(uint64_t) * (p->np + 1), pair_bytes = sizeof(slm_pair) * p->n_slots;
    const size_t need = 8 + off_bytes + pair_bytes;
    if (need > s->host_bytes) {
        if (s->host) {
            cudaStreamSynchronize(w->stream);  // a failed earlier batch may have left copies pending
            cudaFreeHost(s->host);
        }
        s->host = nullptr;
        s->host_bytes = 0;
        SLM_CU(cudaHostAlloc(&s->host, need + need / 4, cudaHostAllocDefault));
        s->host_bytes = need + need / 4;
    }
    unsigned char *h = static_cast<unsigned char *>(s->host);
    SLM_CU(cudaMemcpyAsync(h, p->d_ctl.as<uint32_t>() + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, w->stream));
    SLM_CU(cudaMemcpyAsync(h + 8, p->d_offsets.p, off_bytes, cudaMemcpyDeviceToHost, w->stream));
    if (pair_bytes) SLM_CU(cudaMemcpyAsync(h + 8 + off_bytes, p->d_dense.p, pair_bytes, cudaMemcpyDeviceToHost, w->stream));
    SLM_CU(cudaEventRecord(s->done, w->stream));
    return SLM_OK;
}

void coal_loop(Coalescer *co) {
    cudaSetDevice(co->ctx->device);
    std::unique_lock<std::mutex> lk(co->mu);
    const auto tick = std::chrono::microseconds(20);  // completion polling while a batch runs
    const auto win = std::chrono::microseconds(co->window_us);
    for (;;) {
        // completions
        bool finished = false;
        for (CoalSlot &s : co->slots)
            if (s.busy && cudaEventQuery(s.done) != cudaErrorNotReady) {
                cudaGetLastError();
                coal_collect(co, &s);
                finished = true;
            }
        if (finished) co->cv_done.notify_all();
        // admission: a free slot takes the waiting calls with the oldest call's
        // ratio and cross-check once the batch is full, the queue has been quiet
        // for the window (callers released together have all come back), or the
        // oldest call has waited 8 windows
        for (CoalSlot &s : co->slots) {
            if (s.busy || co->pending.empty()) continue;
            const CoalReq *first = co->pending.front();
            const auto now = Clock::now();
            const bool full = co->pending.size() >= co->max_pairs;
            const bool quiet = now - co->last_arrival >= win;
            const bool overdue = now - first->t_submit >= 8 * win;
            if (!full && !quiet && !overdue && !co->stop) break;
            std::vector<CoalReq *> take;
            for (auto it = co->pending.begin(); it != co->pending.end() && take.size() < co->max_pairs;) {
                if ((*it)->ratio == first->ratio && (*it)->mutual == first->mutual) {
                    take.push_back(*it);
                    it = co->pending.erase(it);
                } else {
                    ++it;
                }
            }
            const slm_status is = coal_issue(co, &s, take);
            if (is != SLM_OK) {
                for (CoalReq *r : take) coal_finish(co, r, is, g_last_error);
                co->cv_done.notify_all();
                continue;
            }
            s.reqs = std::move(take);
            s.busy = true;
            co->batches++;
            co->pairs += s.reqs.size();
            co->max_batch = std::max<uint64_t>(co->max_batch, s.reqs.size());
        }
        const bool busy = co->slots[0].busy || co->slots[1].busy;
        const bool slot_free = !co->slots[0].busy || !co->slots[1].busy;
        if (co->stop && !busy && co->pending.empty()) break;
        // sleep until a call arrives (idle), the next completion poll (a batch
        // runs) or the moment the waiting calls may start
        if (co->pending.empty() && !busy) {
            co->cv_work.wait(lk, [&] { return co->stop || !co->pending.empty(); });
            continue;
        }
        auto wake = Clock::now() + tick;
        if (!co->pending.empty() && slot_free) {
            const auto ready = std::min(co->last_arrival + win, co->pending.front()->t_submit + 8 * win);
            wake = busy ? std::min(wake, ready) : ready;
        }
        const size_t npend = co->pending.size();
        co->cv_work.wait_until(lk, wake, [&] {
            return co->stop || (slot_free && co->pending.size() >= co->max_pairs && co->pending.size() != npend);
        });
    }
}

void coal_stop(slm_ctx *c) {
    Coalescer *co = c->coal;
    if (!co) return;
    {
        std::lock_guard<std::mutex> g(co->mu);
        co->stop = true;
    }
    co->cv_work.notify_all();
    if (co->worker.joinable()) co->worker.join();
    for (CoalSlot &s : co->slots) {
        if (s.w.stream) cudaStreamSynchronize(s.w.stream);
        if (s.done) cudaEventDestroy(s.done);
        plan_release(&s.w.plan);
        if (s.w.stream) cudaStreamDestroy(s.w.stream);
        s.w.stream = nullptr;
    }
    delete co;
    c->coal = nullptr;
}

}  // namespace

void coalescer_destroy(slm_ctx *c) { coal_stop(c); }

// Queues one AUTO call on the context's coalescer and waits for its result.
slm_status coalesce_call(slm_ctx *c, const float *a, uint32_t na, const float *b, uint32_t nb, float ratio,
                         int mutual, slm_pair *out, uint32_t cap, uint32_t *n_out, slm_stats *st) {
    Coalescer *co = c->coal;
    CoalReq r;
    r.a = a;
    r.b = b;
    r.na = na;
    r.nb = nb;
    r.ratio = ratio;
    r.mutual = mutual;
    r.out = out;
    r.cap = cap;
    r.n_out = n_out;
    r.st = st;
    r.t_submit = Clock::now();
    std::unique_lock<std::mutex> lk(co->mu);
    if (co->stop) return fail(SLM_INVALID_ARG, "context is being destroyed");
    co->pending.push_back(&r);
    co->last_arrival = r.t_submit;
    co->cv_work.notify_all();
    co->cv_done.wait(lk, [&] { return r.done; });
    if (r.status != SLM_OK) {
        g_last_error = r.error;
        return r.status;
    }
    return SLM_OK;
}

extern "C" slm_status slm_ctx_set_coalescing(slm_ctx *c, uint32_t window_us, uint32_t max_pairs) {
    if (!c) return fail(SLM_INVALID_ARG, "NULL context");
    if (max_pairs > 4096) return fail(SLM_INVALID_ARG, "max_pairs must be at most 4096");
    if (window_us > 1000000) return fail(SLM_INVALID_ARG, "window_us must be at most 1000000");
    SLM_TRY(ctx_check_device(c));
    coal_stop(c);  // waits for calls in flight; a new setting starts a new worker
    if (max_pairs == 0) return SLM_OK;
    auto *co = new (std::nothrow) Coalescer();
    if (!co) return fail(SLM_OOM, "host allocation failed");
    co->ctx = c;
    co->window_us = window_us;
    co->max_pairs = max_pairs;
    for (CoalSlot &s : co->slots) {
        if (cudaStreamCreateWithFlags(&s.w.stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            for (CoalSlot &q : co->slots) {
                if (q.done) cudaEventDestroy(q.done);
                if (q.w.stream) cudaStreamDestroy(q.w.stream);
            }
            delete co;
            return fail(SLM_CUDA_ERROR, "coalescer stream or event creation failed");
        }
        s.w.store.ctx = c;
        s.w.plan.ctx = c;
        s.w.plan.st = &s.w.store;
    }
    c->coal = co;
    co->worker = std::thread(coal_loop, co);
    return SLM_OK;
}

extern "C" slm_status slm_ctx_coalescing_stats(slm_ctx *c, uint64_t *batches, uint64_t *calls, uint64_t *max_batch) {
    if (!c || !batches || !calls || !max_batch) return fail(SLM_INVALID_ARG, "NULL argument");
    *batches = *calls = *max_batch = 0;
    Coalescer *co = c->coal;
    if (!co) return SLM_OK;
    std::lock_guard<std::mutex> g(co->mu);
    *batches = co->batches;
    *calls = co->pairs;
    *max_batch = co->max_batch;
    return SLM_OK;
}

// ----------------------------------------------------- descriptor producer
//
// detect_and_describe (features.rs:594-648) over a batch of images of one
// size. The pyramid, gradient tables, extrema, orientations and descriptors
// run on the device (k_features.cu); the host makes the per-layer blur taps
// with the platform's expf and the scale step with its powf (the reference
// computes these scalars with the same library calls), orders the candidates
// as the reference emits them, applies its stable sort by |response| and the
// max_features cut, and runs the upsampled detection's de-duplication.

namespace {

// gaussian_blur's taps (features.rs:215-220)
slm_status make_blur_taps(float sigma, BlurTaps &t) {
    float rf = std::ceil(3.0f * sigma);
    if (!(rf >= 1.0f)) rf = 1.0f;  // f32::max(1.0), NaN included
    if (!(rf <= (float)kMaxBlurR)) return fail(SLM_INVALID_ARG, "blur radius ceil(3 sigma) above 127");
    const int r = (int)rf;
    for (int i = -r; i <= r; ++i) t.k[i + r] = expf((float)(-(i * i)) / (2.0f * sigma * sigma));
    float sum = -0.0f;
    for (int i = 0; i < 2 * r + 1; ++i) sum += t.k[i];
    for (int i = 0; i < 2 * r + 1; ++i) t.k[i] /= sum;
    t.r = r;
    return SLM_OK;
}

// f32::powi with a run-time exponent (compiler-rt __powisf2: square and
// multiply over the exponent's bits)
float powi_f32(float a, int b) {
    const bool recip = b < 0;
    float r = 1.0f;
    for (;;) {
        if (b & 1) r *= a;
        b /= 2;
        if (b == 0) break;
        a *= a;
    }
    return recip ? 1.0f / r : r;
}

uint64_t feat_align(uint64_t x) { return (x + 255) & ~uint64_t(255); }

// One detect_core over a batch (its device state stays in `pyr` until the
// next run): the kept features of every image, in the reference's order.
struct FeatCore {
    std::vector<OctaveGeom> geom;
    // read back into the workspace's pinned block (valid until its next use)
    const FeatCand *cands = nullptr;
    const float *angles = nullptr;  // kMaxAngles per candidate
    std::vector<std::vector<std::pair<uint32_t, uint32_t>>> kept;  // per image: (candidate, angle slot)
    // device addresses inside pyr
    float2 *d_grads = nullptr;
    FeatCand *d_cands = nullptr;
    OctaveGeom *d_geom = nullptr;
    int s = 0;
};

slm_status feat_core(slm_ctx *c, Workspace *ws, const float *d_img, uint32_t n, int w, int h,
                     const slm_detector_config &cfg, float in_sigma, FeatCore &out) {
    cudaStream_t st = ws->stream;
    DevBuf &pyr = ws->feat_pyr;
    out = FeatCore();
    out.kept.assign(n, {});
    const int s = (int)cfg.scales, ng = s + 3;
    out.s = s;
    {
        int wo = w, ho = h;
        uint64_t goff = 0;
        for (uint32_t o = 0; o < cfg.octaves; ++o) {
            if (wo < 16 || ho < 16) break;
            OctaveGeom g{};
            g.w = wo;
            g.h = ho;
            g.layer_stride = (uint64_t)wo * ho;
            g.grad_off = goff;
            goff += (uint64_t)n * s * g.layer_stride;
            out.geom.push_back(g);
            wo /= 2;
            ho /= 2;
        }
    }
    if (out.geom.empty() || n == 0) return SLM_OK;
    const uint64_t wh0 = out.geom[0].layer_stride;
    const uint64_t wh1 = out.geom.size() > 1 ? out.geom[1].layer_stride : 0;
    uint64_t ngrad = 0;
    for (const OctaveGeom &g : out.geom) ngrad += (uint64_t)n * s * g.layer_stride;
    uint32_t cap = std::max<uint32_t>(4096, std::min<uint64_t>(uint64_t(n) * 16384, 1u << 26));
    const float kstep = powf(2.0f, 1.0f / (float)s);
    float sb = cfg.sigma0 * cfg.sigma0 - in_sigma * in_sigma;
    if (!(sb >= 0.01f)) sb = 0.01f;  // f32::max(0.01)
    const float sigma_base = std::sqrt(sb);
    const float er1 = cfg.edge_ratio + 1.0f;
    const float edge_thr = er1 * er1 / cfg.edge_ratio;
    std::vector<BlurTaps> taps(ng);
    SLM_TRY(make_blur_taps(sigma_base, taps[0]));
    for (int i = 1; i < ng; ++i) {
        const float prev = cfg.sigma0 * powi_f32(kstep, i - 1);
        const float cur = prev * kstep;
        SLM_TRY(make_blur_taps(std::sqrt(cur * cur - prev * prev), taps[i]));
    }
    for (int attempt = 0; attempt < 2; ++attempt) {
        const uint64_t o_geom = 0, o_gauss = feat_align(o_geom + sizeof(OctaveGeom) * out.geom.size()),
                       o_dog = feat_align(o_gauss + 4 * (uint64_t)n * ng * wh0),
                       o_tmp = feat_align(o_dog + 4 * (uint64_t)n * (ng - 1) * wh0),
                       o_base = feat_align(o_tmp + 4 * (uint64_t)n * wh0),
                       o_grad = feat_align(o_base + 4 * (uint64_t)n * wh1),
                       o_cand = feat_align(o_grad + 8 * ngrad), o_cnt = feat_align(o_cand + sizeof(FeatCand) * cap),
                       o_ang = feat_align(o_cnt + 16), o_nang = feat_align(o_ang + 4ull * kMaxAngles * cap),
                       bytes = feat_align(o_nang + cap);
        SLM_TRY(pyr.ensure(c, bytes));
        unsigned char *d = pyr.as<unsigned char>();
        float *gauss = reinterpret_cast<float *>(d + o_gauss), *dog = reinterpret_cast<float *>(d + o_dog),
              *tmp = reinterpret_cast<float *>(d + o_tmp), *base = reinterpret_cast<float *>(d + o_base);
        out.d_geom = reinterpret_cast<OctaveGeom *>(d + o_geom);
        out.d_grads = reinterpret_cast<float2 *>(d + o_grad);
        out.d_cands = reinterpret_cast<FeatCand *>(d + o_cand);
        uint32_t *d_count = reinterpret_cast<uint32_t *>(d + o_cnt);
        float *d_ang = reinterpret_cast<float *>(d + o_ang);
        uint8_t *d_nang = reinterpret_cast<uint8_t *>(d + o_nang);
        SLM_CU(cudaMemcpyAsync(out.d_geom, out.geom.data(), sizeof(OctaveGeom) * out.geom.size(),
                               cudaMemcpyHostToDevice, st));
        SLM_CU(cudaMemsetAsync(d_count, 0, 4, st));
        for (size_t o = 0; o < out.geom.size(); ++o) {
            const OctaveGeom &G = out.geom[o];
            const uint64_t wh = G.layer_stride;
            if (o == 0) {
                launch_blur(d_img, tmp, gauss, nullptr, nullptr, G.w, G.h, (int)n, wh, ng * wh, 0, taps[0], st);
            } else {
                const OctaveGeom &P = out.geom[o - 1];
                launch_downsample(gauss + s * P.layer_stride, base, P.w, P.h, (int)n, ng * P.layer_stride, wh, st);
                SLM_CU(cudaMemcpy2DAsync(gauss, 4 * ng * wh, base, 4 * wh, 4 * wh, n, cudaMemcpyDeviceToDevice, st));
            }
            for (int i = 1; i < ng; ++i)
                launch_blur(gauss + (i - 1) * wh, tmp, gauss + i * wh, gauss + (i - 1) * wh, dog + (i - 1) * wh, G.w,
                            G.h, (int)n, ng * wh, ng * wh, (ng - 1) * wh, taps[i], st);
            launch_grad(gauss, out.d_grads + G.grad_off, G.w, G.h, s, ng * wh, 1, (int)n, st);
            ExtremaArgs ea{};
            ea.dog = dog;
            ea.layer_stride = wh;
            ea.w = G.w;
            ea.h = G.h;
            ea.s = s;
            ea.ng = ng;
            ea.octave = (int)o;
            ea.contrast = cfg.contrast;
            ea.edge_thr = edge_thr;
            ea.sigma0 = cfg.sigma0;
            ea.kstep = kstep;
            ea.cands = out.d_cands;
            ea.count = d_count;
            ea.cap = cap;
            launch_extrema(ea, (int)n, st);
        }
        SLM_CU(cudaGetLastError());
        uint32_t count = 0;
        SLM_CU(cudaMemcpyAsync(&count, d_count, 4, cudaMemcpyDeviceToHost, st));
        SLM_CU(cudaStreamSynchronize(st));
        if (count > cap) {  // the list overflowed: run again with room for every candidate
            if (attempt) return fail(SLM_INTERNAL, "feature candidates overflowed twice");
            cap = count;
            continue;
        }
        OrientArgs oa{};
        oa.cands = out.d_cands;
        oa.count = d_count;
        oa.cap = cap;
        oa.grads = out.d_grads;
        oa.geom = out.d_geom;
        oa.s = s;
        oa.angles = d_ang;
        oa.nang = d_nang;
        launch_orient(oa, count, st);
        SLM_CU(cudaGetLastError());
        // candidates, angle counts and angles into pinned host memory
        const uint64_t h_ang = feat_align(sizeof(FeatCand) * (uint64_t)count),
                       h_nang = feat_align(h_ang + 4ull * kMaxAngles * count), h_bytes = h_nang + count + 16;
        SLM_TRY(ws_host_block(ws, h_bytes));
        unsigned char *hb = ws->single_host;
        out.cands = reinterpret_cast<const FeatCand *>(hb);
        out.angles = reinterpret_cast<const float *>(hb + h_ang);
        const uint8_t *nang = hb + h_nang;
        if (count) {
            SLM_CU(cudaMemcpyAsync(hb, out.d_cands, sizeof(FeatCand) * count, cudaMemcpyDeviceToHost, st));
            SLM_CU(cudaMemcpyAsync(hb + h_ang, d_ang, 4ull * kMaxAngles * count, cudaMemcpyDeviceToHost, st));
            SLM_CU(cudaMemcpyAsync(hb + h_nang, d_nang, count, cudaMemcpyDeviceToHost, st));
        }
        SLM_CU(cudaStreamSynchronize(st));
        // the reference's emission order (octave, layer, row, column of the
        // scanned extremum; angles in bin order), then its stable sort by
        // |response| descending (f32::total_cmp of abs(): the bits of |v|) and
        // the max_features cut (features.rs:776-778)
        // One sort per image of compact candidate records by (|response|
        // descending, emission key); a candidate's features follow in angle
        // order: the same list as the stable sort of the emitted features,
        // since every feature of a candidate shares its |response| and key.
        struct Ord {
            uint32_t nmag;  // ~bits(|value|): ascending = |value| descending
            uint32_t idx;
            uint64_t key;
        };
        std::vector<uint32_t> per(n + 1, 0);
        for (uint32_t i = 0; i < count; ++i) per[out.cands[i].img + 1]++;
        for (uint32_t k = 0; k < n; ++k) per[k + 1] += per[k];
        std::vector<Ord> ord(count);
        {
            std::vector<uint32_t> fill(per.begin(), per.end() - 1);
            for (uint32_t i = 0; i < count; ++i) {
                const FeatCand &fc = out.cands[i];
                uint32_t u;
                std::memcpy(&u, &fc.value, 4);
                ord[fill[fc.img]++] = Ord{~(u & 0x7fffffffu), i, fc.key};
            }
        }
        for (uint32_t k = 0; k < n; ++k) {
            std::sort(ord.begin() + per[k], ord.begin() + per[k + 1], [](const Ord &a, const Ord &b) {
                return a.nmag != b.nmag ? a.nmag < b.nmag : a.key < b.key;
            });
            std::vector<std::pair<uint32_t, uint32_t>> f;
            for (uint32_t q = per[k]; q < per[k + 1] && f.size() < cfg.max_features; ++q)
                for (uint32_t a = 0; a < nang[ord[q].idx] && f.size() < cfg.max_features; ++a)
                    f.emplace_back(ord[q].idx, a);
            out.kept[k] = std::move(f);
        }
        return SLM_OK;
    }
    return fail(SLM_INTERNAL, "feature candidates overflowed");
}

// Keypoint of a kept feature in input-image pixels (features.rs:755-763).
slm_keypoint feat_keypoint(const FeatCore &fc, uint32_t cand, uint32_t a) {
    const FeatCand &c = fc.cands[cand];
    const float scale = (float)(1ull << c.octave);
    slm_keypoint k;
    k.x = c.x * scale;
    k.y = c.y * scale;
    k.sigma = c.sig * scale;
    k.response = c.value;
    k.angle = fc.angles[(size_t)cand * kMaxAngles + a];
    return k;
}

// Descriptors of the listed features of one run, into rows 0.. of `buf`
// (after its job table).
slm_status feat_describe(slm_ctx *c, cudaStream_t st, DevBuf &buf, const FeatCore &fc,
                         const std::vector<std::pair<uint32_t, uint32_t>> &list, float **d_desc) {
    *d_desc = nullptr;
    if (list.empty()) return SLM_OK;
    if (list.size() >= (1ull << 31)) return fail(SLM_INVALID_ARG, "too many features in one call");
    const uint64_t o_jobs = 0, o_desc = feat_align(sizeof(DescJob) * list.size()),
                   bytes = o_desc + 4ull * kDesc * list.size();
    SLM_TRY(buf.ensure(c, bytes));
    std::vector<DescJob> jobs(list.size());
    for (size_t i = 0; i < list.size(); ++i) {
        jobs[i].cand = list[i].first;
        jobs[i].angle = fc.angles[(size_t)list[i].first * kMaxAngles + list[i].second];
        jobs[i].out_row = (uint32_t)i;
        jobs[i].pad = 0;
    }
    unsigned char *d = buf.as<unsigned char>();
    SLM_CU(cudaMemcpyAsync(d + o_jobs, jobs.data(), sizeof(DescJob) * jobs.size(), cudaMemcpyHostToDevice, st));
    DescribeArgs da{};
    da.jobs = reinterpret_cast<const DescJob *>(d + o_jobs);
    da.cands = fc.d_cands;
    da.grads = fc.d_grads;
    da.geom = fc.d_geom;
    da.s = fc.s;
    da.desc = reinterpret_cast<float *>(d + o_desc);
    launch_describe(da, (uint32_t)jobs.size(), st);
    SLM_CU(cudaGetLastError());
    // (the pageable job table was staged by the copy call: the vector may go)
    *d_desc = da.desc;
    return SLM_OK;
}

slm_status check_detector_config(const slm_detector_config *cfg) {
    if (!cfg) return fail(SLM_INVALID_ARG, "NULL detector config");
    if (cfg->scales < 1 || cfg->scales > 32) return fail(SLM_INVALID_ARG, "scales must be in 1..32");
    if (cfg->octaves > 16) return fail(SLM_INVALID_ARG, "octaves must be at most 16");
    if (!(cfg->sigma0 > 0.0f) || !std::isfinite(cfg->sigma0)) return fail(SLM_INVALID_ARG, "sigma0 must be > 0");
    if (!std::isfinite(cfg->contrast) || !std::isfinite(cfg->edge_ratio) || !(cfg->edge_ratio > 0.0f))
        return fail(SLM_INVALID_ARG, "contrast and edge_ratio must be finite, edge_ratio > 0");
    return SLM_OK;
}

// One batch's features, held in its workspace until they are copied out:
// per image the keypoints of the input-size and of the upsampled detection,
// and where their descriptors lie in the two device staging arrays.
struct FeatOut {
    std::vector<std::vector<slm_keypoint>> kp, kp2;
    std::vector<uint64_t> first1, first2;
    float *d_desc1 = nullptr, *d_desc2 = nullptr;
};

// detect_and_describe of the n images at d_gray (in the workspace), up to
// the copies out.
slm_status detect_describe_run(slm_ctx *c, Workspace *ws, const float *d_gray, uint32_t n, uint32_t w, uint32_t h,
                               const slm_detector_config &cfg, FeatOut &fo) {
    cudaStream_t st = ws->stream;
    FeatCore run;
    SLM_TRY(feat_core(c, ws, d_gray, n, (int)w, (int)h, cfg, 0.5f, run));
    std::vector<std::pair<uint32_t, uint32_t>> all1;
    std::vector<uint64_t> first1(n + 1, 0);
    for (uint32_t k = 0; k < n; ++k) {
        first1[k] = all1.size();
        all1.insert(all1.end(), run.kept[k].begin(), run.kept[k].end());
    }
    first1[n] = all1.size();
    float *d_desc1 = nullptr;
    SLM_TRY(feat_describe(c, st, ws->feat_desc[0], run, all1, &d_desc1));
    std::vector<std::vector<slm_keypoint>> kp(n);
    for (uint32_t k = 0; k < n; ++k)
        for (const auto &f : run.kept[k]) kp[k].push_back(feat_keypoint(run, f.first, f.second));
    // the 2x upsampled detection of small images short of features
    // (features.rs:595-647)
    std::vector<uint32_t> up;
    const uint32_t big = std::max(w, h);
    if (!(cfg.upscale_below == 0 || big >= cfg.upscale_below))
        for (uint32_t k = 0; k < n; ++k) {
            const uint64_t nk = kp[k].size();
            if (nk >= cfg.max_features || (!cfg.upscale_fill && nk * 2 >= cfg.max_features)) continue;
            up.push_back(k);
        }
    std::vector<std::vector<slm_keypoint>> kp2(n);
    std::vector<uint64_t> first2(n + 1, 0);
    std::vector<std::pair<uint32_t, uint32_t>> all2;
    float *d_desc2 = nullptr;
    if (!up.empty()) {
        const uint64_t wh = (uint64_t)w * h, nu = up.size();
        // the images to upsample, gathered, then their upsampling
        const uint64_t o_up = feat_align(4 * nu * wh) / 4;
        SLM_TRY(ws->feat_up.ensure(c, 4 * (o_up + 4 * nu * wh)));
        float *fu = ws->feat_up.as<float>();
        for (uint64_t q = 0; q < nu; ++q)
            SLM_CU(cudaMemcpyAsync(fu + q * wh, d_gray + up[q] * wh, 4 * wh, cudaMemcpyDeviceToDevice, st));
        launch_upsample2(fu, fu + o_up, (int)w, (int)h, (int)nu, st);
        SLM_CU(cudaGetLastError());
        FeatCore run2;
        SLM_TRY(feat_core(c, ws, fu + o_up, (uint32_t)nu, 2 * (int)w, 2 * (int)h, cfg, 1.0f, run2));
        const float cell = 4.0f;
        const int64_t gw = (int64_t)((float)w / cell) + 2, gh = (int64_t)((float)h / cell) + 2;
        auto key = [&](float x, float y) {
            return std::make_pair(std::clamp<int64_t>((int64_t)std::floor(x / cell), -1, gw - 1),
                                  std::clamp<int64_t>((int64_t)std::floor(y / cell), -1, gh - 1));
        };
        for (uint64_t q = 0; q < nu; ++q) {
            const uint32_t k = up[q];
            const uint64_t need = cfg.max_features - kp[k].size();
            std::map<std::pair<int64_t, int64_t>, std::vector<const slm_keypoint *>> grid;
            for (const slm_keypoint &o : kp[k]) grid[key(o.x, o.y)].push_back(&o);
            first2[k] = all2.size();
            for (const auto &f : run2.kept[q]) {
                if (kp2[k].size() >= need) break;
                slm_keypoint e = feat_keypoint(run2, f.first, f.second);
                e.x = e.x / 2.0f - 0.25f;
                e.y = e.y / 2.0f - 0.25f;
                e.sigma /= 2.0f;
                const auto kk = key(e.x, e.y);
                bool dup = false;
                for (int64_t i = kk.first - 1; i <= kk.first + 1 && !dup; ++i)
                    for (int64_t j = kk.second - 1; j <= kk.second + 1 && !dup; ++j) {
                        auto it = grid.find({i, j});
                        if (it == grid.end()) continue;
                        for (const slm_keypoint *o : it->second) {
                            const float r = std::fmax(o->sigma / e.sigma, e.sigma / o->sigma);
                            if (hypotf(o->x - e.x, o->y - e.y) <= 1.0f && r <= 1.5f) {
                                dup = true;
                                break;
                            }
                        }
                    }
                if (!dup) {
                    kp2[k].push_back(e);
                    all2.push_back(f);
                }
            }
        }
        // first2 as offsets into all2 by image (images without upsampling add nothing)
        uint64_t acc = 0;
        for (uint32_t k = 0; k < n; ++k) {
            first2[k] = acc;
            acc += kp2[k].size();
        }
        first2[n] = acc;
        SLM_TRY(feat_describe(c, st, ws->feat_desc[1], run2, all2, &d_desc2));
    }
    fo.kp = std::move(kp);
    fo.kp2 = std::move(kp2);
    fo.first1 = std::move(first1);
    fo.first2 = std::move(first2);
    fo.d_desc1 = d_desc1;
    fo.d_desc2 = d_desc2;
    return SLM_OK;
}

// Copies a batch's features out: image k to kps / desc rows from off[k] on.
slm_status feat_emit(const FeatOut &fo, uint32_t n, const uint64_t *off, slm_keypoint *kps, float *desc,
                     cudaStream_t st) {
    for (uint32_t k = 0; k < n; ++k) {
        const uint64_t n1 = fo.kp[k].size(), n2 = fo.kp2[k].size();
        if (kps) {
            std::memcpy(kps + off[k], fo.kp[k].data(), sizeof(slm_keypoint) * n1);
            if (n2) std::memcpy(kps + off[k] + n1, fo.kp2[k].data(), sizeof(slm_keypoint) * n2);
        }
        if (desc) {
            if (n1)
                SLM_CU(cudaMemcpyAsync(desc + off[k] * kDesc, fo.d_desc1 + fo.first1[k] * kDesc, 4ull * kDesc * n1,
                                       cudaMemcpyDefault, st));
            if (n2)
                SLM_CU(cudaMemcpyAsync(desc + (off[k] + n1) * kDesc, fo.d_desc2 + fo.first2[k] * kDesc,
                                       4ull * kDesc * n2, cudaMemcpyDefault, st));
        }
    }
    return SLM_OK;
}

// The body of both entry points: the images (gray f32, or RGB8 converted on
// the device) go in two halves to two workspaces run from two host threads,
// so one half's host work (candidate ordering, keypoints) overlaps the other
// half's kernels; one workspace below 4 images. Features come out in image
// order whatever the split.
slm_status feat_call(slm_ctx *c, const void *imgs, bool rgb, uint32_t n, uint32_t w, uint32_t h,
                     const slm_detector_config &cfg, slm_keypoint *kps, float *desc, uint64_t cap, uint64_t *off) {
    const uint64_t wh = (uint64_t)w * h;
    const uint32_t parts = n >= 4 ? 2 : 1;
    const uint32_t bnd[3] = {0, parts == 2 ? n / 2 : n, n};
    Workspace *ws[2] = {nullptr, nullptr};
    for (uint32_t p = 0; p < parts; ++p) {
        slm_status a = ws_acquire(c, &ws[p]);
        if (a != SLM_OK) {
            for (uint32_t q = 0; q < p; ++q) ws_release(c, ws[q]);
            return a;
        }
    }
    FeatOut outs[2];
    slm_status sts[2] = {SLM_OK, SLM_OK};
    std::string errs[2];
    auto job = [&](uint32_t p) {
        Workspace *W = ws[p];
        const uint32_t np = bnd[p + 1] - bnd[p];
        slm_status r = SLM_OK;
        if (np) {
            cudaSetDevice(c->device);
            const uint64_t o_rgb = feat_align(4 * np * wh);
            r = W->feat_in.ensure(c, rgb ? o_rgb + 3 * np * wh : 4 * np * wh);
            unsigned char *d = W->feat_in.as<unsigned char>();
            if (r == SLM_OK) {
                const unsigned char *src = static_cast<const unsigned char *>(imgs) + (rgb ? 3 : 4) * bnd[p] * wh;
                if (cudaMemcpyAsync(rgb ? d + o_rgb : d, src, (rgb ? 3 : 4) * np * wh, cudaMemcpyDefault,
                                    W->stream) != cudaSuccess)
                    r = fail(SLM_CUDA_ERROR, std::string("image upload: ") + cudaGetErrorString(cudaGetLastError()));
            }
            if (r == SLM_OK && rgb) {
                launch_gray_from_rgb8(d + o_rgb, reinterpret_cast<float *>(d), np * wh, W->stream);
                if (cudaGetLastError() != cudaSuccess) r = fail(SLM_CUDA_ERROR, "gray conversion launch failed");
            }
            if (r == SLM_OK) r = detect_describe_run(c, W, W->feat_in.as<float>(), np, w, h, cfg, outs[p]);
        }
        sts[p] = r;
        if (r != SLM_OK) errs[p] = g_last_error;
    };
    if (parts == 2) {
        std::thread helper;
        try {
            helper = std::thread(job, 1u);
        } catch (...) {  // no thread to be had: the halves one after the other
        }
        job(0);
        if (helper.joinable())
            helper.join();
        else
            job(1);
    } else {
        job(0);
    }
    slm_status st = SLM_OK;
    for (uint32_t p = 0; p < parts && st == SLM_OK; ++p)
        if (sts[p] != SLM_OK) {
            st = sts[p];
            g_last_error = errs[p];
        }
    if (st == SLM_OK) {
        uint64_t total = 0;
        for (uint32_t p = 0; p < parts; ++p)
            for (uint32_t k = 0; k < bnd[p + 1] - bnd[p]; ++k) {
                off[bnd[p] + k] = total;
                total += outs[p].kp[k].size() + outs[p].kp2[k].size();
            }
        off[n] = total;
        if (total > cap)
            st = fail(SLM_CAPACITY, "feature output holds " + std::to_string(cap) + " of " + std::to_string(total) +
                                        " features");
    }
    for (uint32_t p = 0; p < parts && st == SLM_OK; ++p)
        if (bnd[p + 1] > bnd[p]) st = feat_emit(outs[p], bnd[p + 1] - bnd[p], off + bnd[p], kps, desc, ws[p]->stream);
    for (uint32_t p = 0; p < parts; ++p) {
        const cudaError_t e = cudaStreamSynchronize(ws[p]->stream);
        if (st == SLM_OK && e != cudaSuccess)
            st = fail(SLM_CUDA_ERROR, std::string("slm_detect_and_describe: ") + cudaGetErrorString(e));
        ws_release(c, ws[p]);
    }
    return st;
}

slm_status feat_entry_checks(slm_ctx *c, const void *imgs, uint32_t n, uint32_t w, uint32_t h,
                             const slm_detector_config *cfg, uint64_t *off) {
    if (!c || !off) return fail(SLM_INVALID_ARG, "NULL argument");
    if (n && !imgs) return fail(SLM_INVALID_ARG, "NULL images");
    if (n > 65535) return fail(SLM_INVALID_ARG, "at most 65535 images per call");
    if (w > 32767 || h > 32767) return fail(SLM_INVALID_ARG, "images up to 32767 pixels a side");
    SLM_TRY(check_detector_config(cfg));
    // launch grids put (image, layer) in one 16-bit grid dimension
    if ((uint64_t)n * cfg->scales > 65535) return fail(SLM_INVALID_ARG, "n * scales must be at most 65535");
    return SLM_OK;
}

}  // namespace

extern "C" void slm_detector_config_default(slm_detector_config *cfg) {
    if (!cfg) return;
    cfg->octaves = 4;
    cfg->scales = 3;
    cfg->sigma0 = 1.6f;
    cfg->contrast = 0.01f;
    cfg->edge_ratio = 10.0f;
    cfg->max_features = 8192;
    cfg->upscale_below = 800;
    cfg->upscale_fill = 0;
}

extern "C" slm_status slm_detect_and_describe(slm_ctx *c, const float *imgs, uint32_t n, uint32_t w, uint32_t h,
                                              const slm_detector_config *cfg, slm_keypoint *kps, float *desc,
                                              uint64_t cap, uint64_t *off) {
    NvtxRange range_("slm_detect_and_describe");
    SLM_TRY(feat_entry_checks(c, imgs, n, w, h, cfg, off));
    for (uint32_t k = 0; k <= n; ++k) off[k] = 0;
    if (!n || !((uint64_t)w * h)) return SLM_OK;
    SLM_TRY(ctx_check_device(c));
    return feat_call(c, imgs, false, n, w, h, *cfg, kps, desc, cap, off);
}

extern "C" slm_status slm_detect_and_describe_rgb8(slm_ctx *c, const uint8_t *rgb, uint32_t n, uint32_t w,
                                                   uint32_t h, const slm_detector_config *cfg, slm_keypoint *kps,
                                                   float *desc, uint64_t cap, uint64_t *off) {
    NvtxRange range_("slm_detect_and_describe_rgb8");
    SLM_TRY(feat_entry_checks(c, rgb, n, w, h, cfg, off));
    for (uint32_t k = 0; k <= n; ++k) off[k] = 0;
    if (!n || !((uint64_t)w * h)) return SLM_OK;
    SLM_TRY(ctx_check_device(c));
    return feat_call(c, rgb, true, n, w, h, *cfg, kps, desc, cap, off);
}

extern "C" slm_status slm_describe(slm_ctx *c, const float *img, uint32_t w, uint32_t h, const slm_keypoint *kps,
                                   uint32_t n, float *desc) {
    NvtxRange range_("slm_describe");
    if (!c || (n && (!img || !kps || !desc))) return fail(SLM_INVALID_ARG, "NULL argument");
    if (w > 32767 || h > 32767) return fail(SLM_INVALID_ARG, "images up to 32767 pixels a side");
    const uint64_t wh = (uint64_t)w * h;
    if (!n) return SLM_OK;
    for (uint32_t i = 0; i < n; ++i)
        if (!std::isfinite(kps[i].x) || !std::isfinite(kps[i].y) || !std::isfinite(kps[i].angle) ||
            !(kps[i].sigma > 0.0f) || kps[i].sigma > 64.0f || std::fabs(kps[i].x) > 1e6f ||
            std::fabs(kps[i].y) > 1e6f)
            return fail(SLM_INVALID_ARG, "keypoints need |x|, |y| <= 1e6, a finite angle and 0 < sigma <= 64");
    SLM_TRY(ctx_check_device(c));
    Workspace *ws = nullptr;
    SLM_TRY(ws_acquire(c, &ws));
    cudaStream_t st_ = ws->stream;
    // image, its gradient table, the geometry, keypoints, jobs, descriptors
    const uint64_t o_img = 0, o_grad = feat_align(4 * wh), o_geom = feat_align(o_grad + 8 * wh),
                   o_kps = feat_align(o_geom + sizeof(OctaveGeom)), o_jobs = feat_align(o_kps + sizeof(slm_keypoint) * n),
                   o_desc = feat_align(o_jobs + sizeof(DescJob) * n), bytes = o_desc + 4ull * kDesc * n;
    slm_status st = ws->feat_pyr.ensure(c, bytes);
    if (st == SLM_OK) {
        unsigned char *d = ws->feat_pyr.as<unsigned char>();
        OctaveGeom g{};
        g.w = (int)w;
        g.h = (int)h;
        g.layer_stride = wh;
        std::vector<DescJob> jobs(n);
        for (uint32_t i = 0; i < n; ++i) jobs[i] = DescJob{i, kps[i].angle, i, 0};
        cudaError_t e = wh ? cudaMemcpyAsync(d + o_img, img, 4 * wh, cudaMemcpyDefault, st_) : cudaSuccess;
        if (e == cudaSuccess) e = cudaMemcpyAsync(d + o_geom, &g, sizeof g, cudaMemcpyHostToDevice, st_);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d + o_kps, kps, sizeof(slm_keypoint) * n, cudaMemcpyDefault, st_);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d + o_jobs, jobs.data(), sizeof(DescJob) * n, cudaMemcpyHostToDevice, st_);
        if (e == cudaSuccess && wh) {
            launch_grad(reinterpret_cast<const float *>(d + o_img), reinterpret_cast<float2 *>(d + o_grad), (int)w,
                        (int)h, 1, wh, 0, 1, st_);
            DescribeArgs da{};
            da.jobs = reinterpret_cast<const DescJob *>(d + o_jobs);
            da.kps = reinterpret_cast<const slm_keypoint *>(d + o_kps);
            da.grads = reinterpret_cast<const float2 *>(d + o_grad);
            da.geom = reinterpret_cast<const OctaveGeom *>(d + o_geom);
            da.s = 1;
            da.desc = reinterpret_cast<float *>(d + o_desc);
            launch_describe(da, n, st_);
            e = cudaGetLastError();
        } else if (e == cudaSuccess) {
            e = cudaMemsetAsync(d + o_desc, 0, 4ull * kDesc * n, st_);  // no pixels: every histogram is empty
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(desc, d + o_desc, 4ull * kDesc * n, cudaMemcpyDefault, st_);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
        if (e != cudaSuccess) st = fail(SLM_CUDA_ERROR, std::string("slm_describe: ") + cudaGetErrorString(e));
    }
    ws_release(c, ws);
    return st;
}

// ------------------------------------------------------------------- tracks
//
// build_tracks with ConflictPolicy::Drop (tracks.rs:190-259): the edge set
// and the connected components on the device (k_tracks.cu), then the
// components in node order, the conflict and length rules and select_tracks
// (tracks.rs:472-500, 786-799) on the host from the representatives.

extern "C" slm_status slm_build_tracks_drop(slm_ctx *c, const uint32_t *n_features, uint32_t n_images,
                                            const slm_pair_matches *pairs, uint32_t n_pairs, const slm_pair *matches,
                                            uint32_t min_length, uint64_t max_tracks, uint64_t *track_off,
                                            uint64_t cap_tracks, slm_pair *obs, uint64_t cap_obs, uint64_t *n_tracks,
                                            uint64_t *n_obs, slm_track_stats *stats) {
    NvtxRange range_("slm_build_tracks_drop");
    if (!c || !n_tracks || !n_obs || (n_images && !n_features) || (n_pairs && !pairs) || (cap_tracks && !track_off) ||
        (cap_obs && !obs))
        return fail(SLM_INVALID_ARG, "NULL argument");
    *n_tracks = *n_obs = 0;
    slm_track_stats stt{};
    // node offsets, the matches the pairs name, validity of the ranges
    std::vector<uint64_t> off(n_images + 1, 0);
    for (uint32_t i = 0; i < n_images; ++i) off[i + 1] = off[i] + n_features[i];
    const uint64_t n = off[n_images];
    if (n >= 0xffffffffull) return fail(SLM_INVALID_ARG, "at most 2^32 - 2 features in all");
    uint64_t n_match = 0;
    for (uint32_t p = 0; p < n_pairs; ++p) {
        if (pairs[p].count > ~0ull - pairs[p].first) return fail(SLM_INVALID_ARG, "a pair's match range overflows");
        n_match = std::max(n_match, pairs[p].first + pairs[p].count);
    }
    if (n_match && !matches) return fail(SLM_INVALID_ARG, "NULL matches");
    if (n_match > (1ull << 34)) return fail(SLM_INVALID_ARG, "more than 2^34 matches");
    std::vector<uint32_t> node_image(n);
    for (uint32_t i = 0; i < n_images; ++i)
        std::fill(node_image.begin() + off[i], node_image.begin() + off[i + 1], i);
    SLM_TRY(ctx_check_device(c));
    Workspace *ws = nullptr;
    SLM_TRY(ws_acquire(c, &ws));
    cudaStream_t s = ws->stream;
    uint64_t slots = 1024;
    while (slots < 2 * n_match) slots <<= 1;
    const uint64_t o_pairs = 0, o_match = feat_align(sizeof(TrackPair) * (uint64_t)n_pairs),
                   o_nf = feat_align(o_match + 8 * n_match), o_off = feat_align(o_nf + 4ull * n_images),
                   o_table = feat_align(o_off + 8ull * (n_images + 1)), o_edges = feat_align(o_table + 8 * slots),
                   o_cnt = feat_align(o_edges + 8 * (n_match + 1)), o_parent = feat_align(o_cnt + 32),
                   o_used = feat_align(o_parent + 4 * (n + 1)), bytes = feat_align(o_used + n + 1);
    slm_status st = ws->feat_pyr.ensure(c, bytes);
    std::vector<uint32_t> parent;
    std::vector<uint8_t> used;
    if (st == SLM_OK) {
        unsigned char *d = ws->feat_pyr.as<unsigned char>();
        std::vector<TrackPair> tp(n_pairs);
        for (uint32_t p = 0; p < n_pairs; ++p)
            tp[p] = TrackPair{pairs[p].image_a, pairs[p].image_b, pairs[p].first, pairs[p].count};
        TrackArgs a{};
        a.pairs = reinterpret_cast<const TrackPair *>(d + o_pairs);
        // matches in device memory, or in host memory the device reads directly
        // (8-byte aligned): read where they lie; otherwise copied first
        cudaPointerAttributes pa{};
        const bool on_device = n_match && cudaPointerGetAttributes(&pa, matches) == cudaSuccess &&
                               pa.type == cudaMemoryTypeDevice;
        cudaGetLastError();
        const bool in_place = n_match && (reinterpret_cast<uintptr_t>(matches) & 7) == 0 && (on_device || c->host_direct);
        a.matches = in_place ? reinterpret_cast<const uint2 *>(matches) : reinterpret_cast<const uint2 *>(d + o_match);
        a.nf = reinterpret_cast<const uint32_t *>(d + o_nf);
        a.off = reinterpret_cast<const uint64_t *>(d + o_off);
        a.n_images = n_images;
        a.table = reinterpret_cast<unsigned long long *>(d + o_table);
        a.table_mask = slots - 1;
        a.edges = reinterpret_cast<unsigned long long *>(d + o_edges);
        unsigned long long *cnt = reinterpret_cast<unsigned long long *>(d + o_cnt);
        a.n_edges = cnt;
        a.n_invalid = cnt + 1;
        uint32_t *changed = reinterpret_cast<uint32_t *>(cnt + 2);
        uint32_t *d_parent = reinterpret_cast<uint32_t *>(d + o_parent);
        uint8_t *d_used = d + o_used;
        const int grid = 4 * c->sms;
        cudaError_t e = n_pairs ? cudaMemcpyAsync(d + o_pairs, tp.data(), sizeof(TrackPair) * n_pairs,
                                                  cudaMemcpyHostToDevice, s)
                                : cudaSuccess;
        if (e == cudaSuccess && n_match && !in_place)
            e = cudaMemcpyAsync(d + o_match, matches, 8 * n_match, cudaMemcpyDefault, s);
        if (e == cudaSuccess && n_images)
            e = cudaMemcpyAsync(d + o_nf, n_features, 4ull * n_images, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d + o_off, off.data(), 8ull * (n_images + 1), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(a.table, 0xff, 8 * slots, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(cnt, 0, 32, s);
        if (e == cudaSuccess) {
            launch_track_edges(a, n_pairs, s);
            launch_track_init(d_parent, d_used, n, grid, s);
            launch_track_mark(a.edges, a.n_edges, d_used, grid, s);
            e = cudaGetLastError();
        }
        // hooking and pointer jumping until no edge joins two roots (each round
        // at least halves the number of roots joined by an edge in practice;
        // bounded by the node count in any case)
        for (uint64_t round = 0; e == cudaSuccess && round <= n + 1; ++round) {
            uint32_t h_changed = 0;
            e = cudaMemsetAsync(changed, 0, 4, s);
            if (e == cudaSuccess) {
                launch_track_hook(a.edges, a.n_edges, d_parent, changed, grid, s);
                launch_track_jump(d_parent, n, grid, s);
                e = cudaGetLastError();
            }
            if (e == cudaSuccess) e = cudaMemcpyAsync(&h_changed, changed, 4, cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess || !h_changed) break;
        }
        unsigned long long h_cnt[2] = {0, 0};
        parent.resize(n);
        used.resize(n);
        if (e == cudaSuccess) e = cudaMemcpyAsync(h_cnt, cnt, 16, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess && n) e = cudaMemcpyAsync(parent.data(), d_parent, 4 * n, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess && n) e = cudaMemcpyAsync(used.data(), d_used, n, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) st = fail(SLM_CUDA_ERROR, std::string("slm_build_tracks_drop: ") + cudaGetErrorString(e));
        stt.edges = h_cnt[0];
        stt.invalid_matches = h_cnt[1];
    }
    if (st != SLM_OK) cudaStreamSynchronize(s);
    ws_release(c, ws);
    if (st != SLM_OK) return st;
    // components in node order: count per representative, then fill
    std::vector<uint64_t> start(n + 1, 0);
    for (uint64_t x = 0; x < n; ++x)
        if (used[x]) start[parent[x] + 1]++;
    for (uint64_t x = 0; x < n; ++x) start[x + 1] += start[x];
    std::vector<uint32_t> members(start[n]);
    {
        std::vector<uint64_t> fill(start.begin(), start.end() - 1);
        for (uint64_t x = 0; x < n; ++x)
            if (used[x]) members[fill[parent[x]]++] = (uint32_t)x;
    }
    struct TrackRef {
        uint64_t first, begin, len, span;
    };
    std::vector<TrackRef> tr;
    const uint64_t min_len = std::max<uint64_t>(min_length, 2);
    for (uint64_t r = 0; r < n; ++r) {
        const uint64_t b = start[r], e = start[r + 1];
        if (b == e) continue;
        bool conflict = false;
        for (uint64_t q = b + 1; q < e && !conflict; ++q)
            conflict = node_image[members[q]] == node_image[members[q - 1]];
        if (conflict) {
            stt.conflicts++;
        } else if (e - b < min_len) {
            stt.too_short++;
        } else {
            tr.push_back(TrackRef{members[b], b, e - b, node_image[members[e - 1]] - node_image[members[b]]});
        }
    }
    // select_tracks (tracks.rs:786-799); tr is already in first-observation order
    if (tr.size() > max_tracks) {
        std::sort(tr.begin(), tr.end(), [](const TrackRef &x, const TrackRef &y) {
            if (x.len != y.len) return x.len > y.len;
            if (x.span != y.span) return x.span > y.span;
            return x.first < y.first;
        });
        stt.truncated = tr.size() - max_tracks;
        tr.resize(max_tracks);
        std::sort(tr.begin(), tr.end(), [](const TrackRef &x, const TrackRef &y) { return x.first < y.first; });
    }
    stt.tracks = tr.size();
    uint64_t total = 0;
    for (const TrackRef &t : tr) total += t.len;
    *n_tracks = tr.size();
    *n_obs = total;
    if (stats) *stats = stt;
    if (tr.size() > cap_tracks || total > cap_obs)
        return fail(SLM_CAPACITY, "track output holds " + std::to_string(cap_tracks) + " tracks / " +
                                      std::to_string(cap_obs) + " observations of " + std::to_string(tr.size()) +
                                      " / " + std::to_string(total));
    uint64_t w = 0;
    if (cap_tracks) track_off[0] = 0;
    for (uint64_t t = 0; t < tr.size(); ++t) {
        for (uint64_t q = 0; q < tr[t].len; ++q, ++w) {
            const uint32_t x = members[tr[t].begin + q];
            obs[w].i = node_image[x];
            obs[w].j = (uint32_t)(x - off[node_image[x]]);
        }
        track_off[t + 1] = w;
    }
    return SLM_OK;
}
