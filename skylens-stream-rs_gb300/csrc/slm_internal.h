// slm_internal.h — data layouts and kernel launchers shared by the host
// library (slm.cpp) and the CUDA translation units. Not part of the ABI.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "slm.h"

namespace slm {

// Device error codes written to a launch's error word: a bounded wait gave up
// (TIMEOUT_*), or an invariant failed (BAD_ITEM: a work queue overflowed, a
// routing plan did not fit, a row was left undecided).
enum : uint32_t { DERR_NONE = 0, DERR_TIMEOUT_BAR = 1, DERR_BAD_ITEM = 2, DERR_TIMEOUT_MMA = 3 };

constexpr int kDesc = 128;      // descriptor length (features.rs:496)
constexpr int kTile = 128;      // rows per store tile
constexpr int kTileFloats = kTile * kDesc;

// Component k of a descriptor goes to slot perm(k) inside a store tile so that
// walking the slots in order walks the reference's accumulation order
// (matching.rs:146-155: lane k % 8, step k / 8): slot = (k % 8) * 16 + k / 8.
__host__ __device__ inline int perm_slot(int k) { return (k & 7) * 16 + (k >> 3); }

// Store tile layout (FP32): tile[slot][row], 128 x 128 floats = 64 KiB.

// Batches of at most this many pairs run their per-pair kernels (finalize,
// mid) with 1024 threads per pair instead of 256: with few pairs the GPU is
// not full and each pair's rows are a chain of dependent loads.
constexpr uint32_t kFewPairs = 64;

// Per-row partial state of an exact scan over a column range.
struct __align__(16) RowPart {
    float d1, d2;   // smallest and second smallest distance (multiset)
    uint32_t j1;    // lowest column index attaining d1 (0xffffffff: none)
    uint32_t pad;
};

#ifdef __CUDACC__
// Merges a column range's partial into a row state: (d1, lowest j1) and the
// second smallest of the multiset (matching.rs:182-187 applied per range).
__device__ __forceinline__ void merge_rowpart(const RowPart &p, float &d1, float &d2, uint32_t &j1) {
    const float nd2 = fminf(fmaxf(d1, p.d1), fminf(d2, p.d2));
    if (p.d1 < d1 || (p.d1 == d1 && p.j1 < j1)) {
        d1 = p.d1;
        j1 = p.j1;
    }
    d2 = nd2;
}
#endif

// Per image pair, as planned on the host.
struct PairMeta {
    uint32_t a_row0, b_row0;  // first store row of the two views (multiples of 128)
    uint32_t na, nb;          // descriptor counts
    uint32_t nchunk;          // column chunks per row tile (exact path)
    uint32_t part_base;       // first RowPart block (128 rows per block)
    uint64_t col_base;        // first column-best entry
    uint64_t slot_off;        // first output slot (capacity na)
};

// One unit of the exact kernel: rows [rt*128, rt*128+128) of pair `pair`
// against store column tiles [ct0, ct1) of b.
struct Item {
    uint32_t pair, rt, ct0, ct1;
    uint32_t part;  // RowPart block receiving the result
    uint32_t pad[3];
};

struct ExactArgs {
    const float *tiled;          // FP32 store tiles
    const Item *items;
    uint32_t n_items;            // item capacity
    const uint32_t *n_items_dev; // if set, the item count is min(*n_items_dev, n_items), read on the device
    const PairMeta *pairs;
    RowPart *parts;
    unsigned long long *colbest; // (bits(d) << 32 | i), min-reduced
    uint32_t *work;              // dynamic item counter (zeroed per launch)
    uint32_t *err;               // device error word (zeroed per launch)
    int mutual;
    int x2;                      // 1: packed f32x2 arithmetic
    float zero;                  // 0.0f, read at run time: the addend of the packed squares
};

struct FinalizeArgs {
    const PairMeta *pairs;
    uint32_t npairs;
    const RowPart *parts;
    const unsigned long long *colbest;
    float ratio2;                // ratio * ratio in f32 (matching.rs:206)
    int mutual;
    uint2 *slots;                // output (i, j) slots
    uint32_t *counts;            // per-pair match count
    const uint32_t *err;         // if set: a count of 0xffffffff when this error word is set
};

// Pack n row-major descriptors (src, n x 128) into store tiles starting at
// tile index `tile0` (rows beyond n within the last tile are zeroed).
// The same for many views: tab holds one {row0, n, tile, view} per tile.
void launch_pack_fp32_tiles(const uint4 *tab, uint32_t ntiles, const float *raw, float *tiled, cudaStream_t s);
void launch_exact(const ExactArgs &a, int grid, cudaStream_t s);
// FP32 tiles of both views of the routed pairs xlist[0 .. *count) of a
// low-precision batch (count read on the device).
void launch_pack_routed(const PairMeta *pairs, const uint32_t *xlist, const uint32_t *count, const float *raw,
                        float *tiled, int grid, cudaStream_t s);
// Sets kernel attributes (large shared memory) once per device; called at
// context creation, outside any stream capture. Fails if the kernel image
// cannot load on the device.
cudaError_t init_exact_kernels();
void launch_finalize(const FinalizeArgs &a, cudaStream_t s);
// One thread waits on a barrier that never completes for `polls` polls and
// records DERR_TIMEOUT_BAR in *err (self-test of the bounded waits).
void launch_wait_selftest(uint32_t polls, uint32_t *err, cudaStream_t s);
void launch_fill_u64(unsigned long long *p, uint64_t n, unsigned long long v, cudaStream_t s);
// Sets the message slm_last_error() returns on this host thread.
void set_last_error(const char *msg);

// Scratch layout of one exact FP32 pair match with its metadata made on the
// device (byte offsets; `inputs` adds room for copies of the row-major inputs).
struct SingleLayout {
    size_t tiled, items, parts, meta, colbest, slots, counts, ctl, raw_a, raw_b, bytes;
    uint32_t rt_n, ct_n, chunks;
};
SingleLayout single_layout(uint32_t na, uint32_t nb, int sms, bool inputs);
// Whether finalize may write the match list straight into d_out: there must be
// room for every possible match (cap >= na), and finalize stores each pair as
// one 8-byte vector, while slm_pair itself only needs 4-byte alignment. Any
// other d_out gets the list through single_copy_kernel, which stores the two
// fields separately.
inline bool single_direct_output(const slm_pair *d_out, uint32_t cap, uint32_t na) {
    return cap >= na && (reinterpret_cast<uintptr_t>(d_out) & 7u) == 0;
}
// Enqueues the setup and packing, exact_kernel and finalize, which leave at
// most cap pairs in d_out and the count (0xffffffff: a device wait gave up) in
// *d_count (directly when single_direct_output holds, else through a copy
// kernel). Returns the launch status.
cudaError_t single_exact_enqueue(unsigned char *scratch, const SingleLayout &L, const float *d_a, uint32_t na,
                                 const float *d_b, uint32_t nb, float ratio, int mutual, slm_pair *d_out,
                                 uint32_t cap, uint32_t *d_count, int sms, cudaStream_t s);

// Sampson scoring of essential-matrix hypotheses (k_sampson.cu), all device
// pointers: pair p's matches are pts[pair_off[p] .. pair_off[p+1]) (a.x, a.y,
// b.x, b.y), hypothesis h is E[9 h .. 9 h + 9) (row-major) of pair
// hyp_pair[h]; counts[h] = #{i : |r| < thresh[p]}; with mask_off[h] !=
// ~0, the inlier bits at masks[mask_off[h] ..].
struct SampsonArgs {
    const double4 *pts;
    const uint64_t *pair_off;
    const double *thresh;
    const double *E;
    const uint32_t *hyp_pair;
    uint64_t nh;
    uint32_t *counts;
    const uint64_t *mask_off;  // may be null (no masks)
    uint32_t *masks;
};
void launch_sampson(const SampsonArgs &a, cudaStream_t s);

// ---------------------------------------------------- descriptor producer
// (k_features.cu; crates/core/src/features.rs)

constexpr int kMaxBlurR = 127;  // blur radius ceil(3 sigma) the kernels take
constexpr int kMaxAngles = 18;  // local maxima of a 36-bin circular histogram

// Normalised taps of one gaussian_blur (features.rs:215-220), made on the host.
struct BlurTaps {
    float k[2 * kMaxBlurR + 1];
    int r;
};

// A refined DoG extremum that passed the contrast and edge tests.
struct __align__(16) FeatCand {
    float x, y;        // refined position in octave pixels
    float sig;         // sig_oct = sigma0 * kstep^s
    float value;       // refined DoG response
    uint16_t img;      // image of the batch
    uint8_t octave;
    uint8_t layer;     // refined layer (its gradient table)
    uint32_t pad;
    uint64_t key;      // emission order: octave << 48 | start layer << 32 | start y << 16 | start x
};

// One octave of a batch: its size and where its gradient tables start.
struct OctaveGeom {
    int w, h;
    uint64_t layer_stride;  // w * h
    uint64_t grad_off;      // float2 offset of (image 0, layer 1)
};

struct ExtremaArgs {
    const float *dog;       // [img][ng - 1][h][w]
    uint64_t layer_stride;
    int w, h, s, ng, octave;
    float contrast, edge_thr, sigma0, kstep;
    FeatCand *cands;
    uint32_t *count;
    uint32_t cap;
};

struct OrientArgs {
    const FeatCand *cands;
    const uint32_t *count;
    uint32_t cap;
    const float2 *grads;    // every octave's tables: [img][layer 1..s][h][w] at geom.grad_off
    const OctaveGeom *geom;
    int s;
    float *angles;          // kMaxAngles per candidate
    uint8_t *nang;
};

struct DescJob {
    uint32_t cand;          // candidate (or keypoint) index
    float angle;
    uint32_t out_row;       // descriptor row written
    uint32_t pad;
};

struct DescribeArgs {
    const DescJob *jobs;
    const FeatCand *cands;  // null: keypoints kps (image pixels) on one table, grads, geom[0]
    const slm_keypoint *kps;
    const float2 *grads;
    const OctaveGeom *geom;
    int s;
    float *desc;
};

// Both passes of a blur of nimg images (src -> tmp -> dst); with dog, also
// dog = dst - prev (prev strided as dst). Strides are per image, in floats.
void launch_blur(const float *src, float *tmp, float *dst, const float *prev, float *dog, int w, int h, int nimg,
                 uint64_t stride_src, uint64_t stride_dst, uint64_t stride_dog, const BlurTaps &t, cudaStream_t s);
void launch_downsample(const float *src, float *dst, int w, int h, int nimg, uint64_t stride_src,
                       uint64_t stride_dst, cudaStream_t s);
void launch_upsample2(const float *src, float *dst, int w, int h, int nimg, cudaStream_t s);
void launch_gray_from_rgb8(const uint8_t *rgb, float *out, uint64_t n, cudaStream_t s);
// gradient tables of layers l0 .. l0 + s_ - 1 of each image (image k's layer l
// at gauss + k * img_stride + l * w * h); grad: [img][s_][h][w]
void launch_grad(const float *gauss, float2 *grad, int w, int h, int s_, uint64_t img_stride, int l0, int nimg,
                 cudaStream_t s);
void launch_extrema(const ExtremaArgs &a, int nimg, cudaStream_t s);
void launch_orient(const OrientArgs &a, uint32_t n, cudaStream_t s);
void launch_describe(const DescribeArgs &a, uint32_t njobs, cudaStream_t s);

// ------------------------------------------------------ tracks (k_tracks.cu)

struct TrackPair {  // slm_pair_matches
    uint32_t image_a, image_b;
    uint64_t first, count;
};

struct TrackArgs {
    const TrackPair *pairs;
    const uint2 *matches;     // (feature of image_a, feature of image_b)
    const uint32_t *nf;       // features per image
    const uint64_t *off;      // first node of each image
    uint32_t n_images;
    unsigned long long *table;  // open-addressing edge set, all ones = empty
    uint64_t table_mask;      // slots - 1 (a power of two)
    unsigned long long *edges;  // the distinct edges, in insertion order
    unsigned long long *n_edges;
    unsigned long long *n_invalid;
};

void launch_track_edges(const TrackArgs &a, uint32_t n_pairs, cudaStream_t s);
void launch_track_init(uint32_t *parent, uint8_t *used, uint64_t n, int grid, cudaStream_t s);
void launch_track_mark(const unsigned long long *edges, const unsigned long long *n_edges, uint8_t *used, int grid,
                       cudaStream_t s);
void launch_track_hook(const unsigned long long *edges, const unsigned long long *n_edges, uint32_t *parent,
                       uint32_t *changed, int grid, cudaStream_t s);
void launch_track_jump(uint32_t *parent, uint64_t n, int grid, cudaStream_t s);

}  // namespace slm
