// slm_shortlist.h — the low-precision shortlist path (BF16 / FP8 tcgen05).
//
// ratio_match's decision (crates/core/src/matching.rs:167-215) depends only on
// a few distances per row: the two smallest, and, for the mutual check, the
// smallest in the chosen column. The shortlist path finds them with tensor-core
// distances d~ = |a|^2 + |b|^2 - 2 a.b whose error against the exact f32
// distance d is bounded per image pair by eps (see shortlist_eps), then
// settles every decision the bound cannot certify with exact spec-order FP32
// arithmetic, so the match list is the reference's bit for bit.
//
//   pass 1  (tcgen05)  per row: m1 = min d~ and m2' = second smallest of the
//                      per-32-column minima (an upper bound of the second
//                      smallest d~); per column: c1 = min d~.
//   mid                per row: threshold T = m2' + 2 eps, or "certain no
//                      match" when m1 - eps >= r^2 (m2' + eps); per column:
//                      threshold c1 + 2 eps.
//   pass 2  (tcgen05)  recomputes d~; for every group of 4 consecutive
//                      columns holding a d~ <= T, appends the group (its first
//                      column and its 4 values) to the row's records; S = the
//                      records' columns with d~ <= T. Counts, per column, the
//                      rows with d~ <= c1 + 2 eps (|C|).
//   finalize           per row, from S: certain outcomes from the bounds; the
//                      mutual check from |C| (a row above the column window
//                      loses, the only row inside it wins). Everything else is
//                      queued: rows to rescore exactly, rows to rescan, columns
//                      to rescan.
//   rescore            one warp per queued row: exact distances of S.
//   scan               one CTA per queued row or column: exact full scans.
//
// Pair routing. When the bound is too loose for a pair's distances (FP8 on
// unit-length descriptors: eps ~ 0.1 against distance gaps of the same size),
// most rows would overflow S and be settled one row at a time. Such a pair is
// routed instead to the tiled exact FP32 kernel, which settles every row and
// column of it:
//   - before pass 1: a pair with non-finite or huge inputs (unsafe);
//   - after pass 1 (mid, FP8): more than 1/8 of its undecided rows are "wide":
//     more than half of their 16-column chunks (and more than kSlRowSlots) had
//     a minimum within 2 eps above the running row minimum; pass 2 skips
//     routed pairs;
//   - after pass 2 (finalize): more than 1/8 as many row halves as rows
//     had a wide shortlist, more than half_recs / 2 hit groups of one
//     column range (pass 2 counts them).
// The routed pairs' exact work items are planned on the device (route_plan,
// route_apply), run by exact_kernel, and route_finalize writes their rows'
// decisions; the results stay bit-exact whichever way a pair goes.
#pragma once
#include <cstdint>

#include "slm_internal.h"

namespace slm {

// Pass 2 keeps, per row, column range and column half, up to half_recs
// (SlArgs; the autotuner's shortlist_k, default kSlHalfRecs) records of 4
// consecutive columns (the group's first column and its 4 d~ values): one
// vector store per hit group. A half with more hit groups overflows and the
// row is settled by an exact scan.
constexpr int kSlHalfRecs = 16;
constexpr int kSlHalfRecsMax = 32;
// Routing estimate of a row's shortlist size (in columns).
constexpr int kSlRowSlots = 32;
// A pair's columns split into at most this many ranges (items that share its
// rows); each range keeps its own records per row, so their memory is
// (rows x ranges) x 2 half_recs records.
constexpr uint32_t kSlMaxRanges = 4;
constexpr int kSlStages = 4;       // b-tile ring depth (FP8; BF16 tiles are larger: 3)
constexpr int kSlEpWarps = 16;     // epilogue warps
constexpr int kSlThreads = 32 * (2 + kSlEpWarps);  // producer, MMA, epilogue

// Operand tile sizes per 128 descriptors.
//
// BF16 tiles carry the squared norms into the tensor-core product: after the
// 32 KiB K-major 128B-swizzled image of the components comes a 6 KiB
// extension, K-major without swizzle, with three 16-byte core-matrix columns
// per row: kc0 = [hi, lo, 1, 1, 0..], kc1 = [1, 1, hi, lo, 0..], kc2 = 0, where
// hi + lo is |v|^2 / 2 split into two bf16. A tile read as operand A from kc0
// and as operand B from kc1 contributes (|a|^2 + |b|^2) / 2 in one K = 16 step;
// the 8 steps over the components run with B negated, so the accumulator holds
// d~ / 2 = (|a|^2 + |b|^2) / 2 - a.b directly.
constexpr uint32_t kBf16TileBytes = 128 * 128 * 2;                    // 32 KiB components
constexpr uint32_t kBf16ExtBytes = 16 * 3 * 128;                      // 6 KiB: 16 row groups x 3 core matrices
constexpr uint32_t kBf16TileStride = kBf16TileBytes + kBf16ExtBytes;  // 38 KiB per tile (1024-byte multiple)
constexpr uint32_t kFp8TileBytes = 128 * 128;                         // 16 KiB

// Per view, from the pack kernel: float bits of non-negative maxima
// (atomicMax on the bit pattern orders them), and a non-finite flag.
struct ViewStat {
    uint32_t nmax;   // max |a|
    uint32_t rho;    // max |a - q(a)| (q: the low-precision rounding, scale removed)
    uint32_t nqmax;  // max |q(a)|
    uint32_t bad;    // nonzero: some component is not finite
};

// Work item: nat (1 or 2) a tiles of 128 rows against column tiles [ct0, ct1)
// of one b view. A tile a is row tile rt[a] of pair pair[a]; its pass-1 row
// partials go to block part[a] (slot (rt[a] * 128 + row) % 256 of it). Both
// tiles usually belong to one pair (rt[1] = rt[0] + 1, part[1] = part[0]);
// two pairs with the same b view and column range, each with an odd number of
// row tiles, share an item for their last tiles, so that no item runs with
// half of the epilogue warps idle.
struct SlItem {
    uint32_t pair[2], rt[2], part[2];
    uint32_t nat, ct0, ct1;
    uint32_t pad[3];
};

// Per-pair extras of the shortlist path.
struct SlPair {
    uint32_t rbase;    // first entry in per-row arrays (multiple of 128)
    uint32_t cbase;    // first entry in per-column arrays (multiple of 128)
    uint32_t part_base, nchunk;  // pass-1 row partials: (part_base + (rt0/2)*nchunk + c) * 256 + r
    uint32_t view_a, view_b;
    float eps;         // written by the eps kernel
    uint32_t unsafe;   // written by the eps kernel: no certification possible
    uint32_t routed;   // per launch: settled by the exact FP32 kernel
    uint32_t xchunk;   // routed: column chunks per 128-row tile
    uint32_t xpart;    // routed: first exact work item (= first RowPart block)
    uint32_t blk;      // first entry of the pair's row blocks in SlArgs::blkcnt
    uint32_t rescued;  // per launch (FP8 plans): settled by the BF16 passes instead
    uint32_t crbase;   // first candidate row: the records of row i and column range c at
                       // crbase + c * (na padded to 128) + i (sl_cand_row)
};

// Candidate row of pair row i in column range c. Each range of a pair's
// columns (an item's ct0..ct1) keeps its own records per row, so exactly one
// item writes them and pass 2 needs no atomics for its slots.
__host__ __device__ inline uint32_t sl_cand_row(const SlPair &sp, uint32_t na, uint32_t c, uint32_t i) {
    return sp.crbase + c * ((na + kTile - 1) / kTile * kTile) + i;
}

// The per-pair kernels after pass 1 (mid, finalize, compact, route_finalize)
// run one CTA per pair and block of this many rows (and columns), so that a
// single large pair spreads over many CTAs.
constexpr uint32_t kSlRowBlock = 2048;

// Per-pair counters of one launch (SlArgs::pairctl, 4 words per pair).
enum : int { kPcWide = 0, kPcOpen = 1, kPcMidDone = 2, kPcOver = 3 };

// Row decision codes (per pair row).
constexpr uint32_t kDecNone = 0xffffffffu;
constexpr uint32_t kDecPending = 0xfffffffeu;

// Queue entries: the scan queue holds kind 0 (exact row scan of row i) and
// kind 1 (exact column check: is row i the argmin of column j); the rescore
// queue holds rows i whose S is rescored exactly.
struct SlQueue {
    uint32_t pair, kind, i, j;
};

// Counters in the plan's control block (u32 words after work/error).
enum : int { kCtlRescored = 2, kCtlQueueRows = 3, kCtlQueueCols = 4, kCtlMaxErr = 5, kCtlScanLen = 6,
             kCtlRescoreLen = 7, kCtlXItems = 8, kCtlXWork = 9, kCtlRoutedPairs = 10, kCtlRoutedRows = 11,
             kCtlRoutedCols = 12, kCtlRouteMarks = 13, kCtlRescuedPairs = 14, kCtlRescuedRows = 15 };

// Routed pairs: at most this many column chunks per 128-row tile; the exact
// items of a launch number at most (routed row tiles) + (4 x SMs).
constexpr uint32_t kXChunkMax = 16;

struct SlArgs {
    const uint8_t *optiles;      // operand tiles by store row / 128
    const float *norms;          // squared f32 norms by store row
    const float *raw;            // row-major f32 descriptors by store row
    const float *qscale;         // FP8: per-row inverse scale (nullptr for BF16)
    const ViewStat *vstats;
    const PairMeta *pairs;
    SlPair *spairs;
    uint32_t npairs;
    const SlItem *items;
    uint32_t n_items;
    float2 *rowpart;             // pass 1: (m1, m2') per row and column range
    uint32_t *rownear;           // pass 1: chunks near the running row minimum (routing estimate)
    uint32_t *colmin;            // pass 1: order-preserving encoding of c1
    float *rowthr;               // mid -> pass 2
    float *colthr;               // mid -> pass 2
    uint32_t *rowcnt;            // pass 2: records per candidate row and column half
    float4 *rowrec;              // pass 2: a record's 4 d~ values (BF16: d~ / 2), 2 half_recs per candidate row
    uint32_t *rowrecj;           // the record's first column
    float *colcnt;               // |C| per column (f32 counts: exact below 2^24)
    uint32_t *rowdec;            // finalize / rescore / scan
    SlQueue *queue;              // scan queue
    SlQueue *rqueue;             // rescore queue
    uint32_t queue_cap;          // capacity of each queue
    uint32_t *ctl;               // [1] error word, counters at kCtl*
    float ratio2;
    int mutual;
    int fp8;
    float *dump;                 // debug: d~ of pair 0, [na][nb] (nullptr: off)
    uint2 *slots;                // pair p, row block b: matches from slot_off + b * kSlRowBlock
    uint32_t *counts;
    uint32_t *blkcnt;            // matches per row block
    uint32_t *pairctl;           // kPc* counters, zeroed per launch
    uint32_t row_blocks;         // the most row blocks of any pair (second grid dimension)
    // pair routing to the exact kernel
    const float *tiled;          // FP32 store tiles
    uint32_t *xlist;             // routed pair ids
    Item *xitems;                // exact work items
    uint32_t xitem_cap;
    RowPart *xparts;             // one 128-row block per item
    unsigned long long *colbest; // by PairMeta::col_base
    uint32_t want_items;         // exact items wanted to fill the GPU (4 x SMs)
    // FP8 plans: pairs the FP8 bound cannot settle (mid: too many wide rows) are
    // rescued by a second, BF16 run of eps / pass 1 / mid / pass 2 / finalize
    // over those pairs only (tier 1), instead of the exact kernel
    uint32_t half_recs;          // records per candidate row and column half (1..kSlHalfRecsMax)
    uint32_t rescue;             // tier 0 of an FP8 plan: mid marks pairs rescued, not routed
    uint32_t tier;               // 0: the plan's precision; 1: the BF16 rescue of an FP8 plan
};

// Whether a pair takes part in this tier's per-pair kernels (pass 2, finalize,
// and, in tier 1, everything): tier 0 skips pairs routed to the exact kernel or
// rescued by tier 1; tier 1 runs the rescued pairs only.
__host__ __device__ inline bool sl_pair_on(const SlArgs &g, const SlPair &sp) {
    return g.tier ? (sp.rescued && !sp.routed) : !(sp.routed || sp.rescued);
}

// Store-side builder: one CTA per entry {first store row of the view, rows,
// tile within the view, view} of the tile table.
void launch_pack_lowp(const uint4 *tab, uint32_t ntiles, const float *raw, int fp8, uint8_t *optiles, float *norms,
                      float *qscale, ViewStat *vstats, cudaStream_t s);

// Kernel image / attribute set-up (outside stream capture).
cudaError_t init_shortlist_kernels();

// The pipeline of one shortlist launch (after counters are cleared):
// eps, pass 1, mid, pass 2, then finalize / routing / rescore / scan / compact.
// Returns the number of kernels the call launched.
int launch_shortlist_eps(const SlArgs &a, cudaStream_t s);
int launch_shortlist_pass(const SlArgs &a, int pass, int sms, cudaStream_t s);
int launch_shortlist_mid(const SlArgs &a, cudaStream_t s);
int launch_shortlist_finalize(const SlArgs &a, cudaStream_t s);
// Tier 1 before its pass 1: the rescued pairs' BF16 eps, column minima and counters.
int launch_shortlist_rescue_prep(const SlArgs &a, cudaStream_t s);
// After every tier's finalize: routing to the exact kernel, rescore, scans, compaction.
int launch_shortlist_tail(const SlArgs &a, int sms, cudaStream_t s);
// Dense results of a shortlist launch: pair p's row blocks in order, pairs
// with counts[p] == 0 (none, or filtered out) skipped.
void launch_gather_blocks(const SlArgs &a, const uint64_t *slot_off, const uint64_t *offsets, uint2 *dense,
                          uint64_t cap, cudaStream_t s);

}  // namespace slm
