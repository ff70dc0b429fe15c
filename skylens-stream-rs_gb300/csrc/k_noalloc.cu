// k_noalloc.cu — slm_ratio_match_device_noalloc: the exact FP32 matcher for
// callers that must not allocate device memory.
//
// Some callers cannot call cudaMalloc: a host application whose framework
// owns every device allocation through its own pool (and counts any other
// allocation as a leak or an overrun of its budget), or a latency-critical loop
// in which a cudaMalloc/cudaFree, which may synchronise the device, would stall
// the other streams. This entry point runs the same kernels as the exact path
// (pack -> exact_kernel -> finalize) with every scratch buffer carved out of
// one file-scope device array, so it allocates nothing: the caller passes only
// the inputs, the output buffer and the stream.
//
// The array is kNoAllocBytes (about 5.1 MiB: the scratch layout of
// single_layout for 4096 x 4096) and every device that loads the library
// holds it until the process exits. Its size sets the limit: na and nb at
// most SLM_NOALLOC_MAX_DESCS (4096) descriptors each. The same pipeline
// (single_exact_enqueue) serves small host-side FP32 calls of slm_ratio_match
// from a per-workspace scratch block.
//
// The first call on a device sets that device up (resolves the array's device
// address with cudaGetSymbolAddress and sets the exact kernel's shared-memory
// attribute); make that first call before any stream capture. All calls share
// the one array and the array keeps the last call's contents; each call
// re-initialises what must start cleared. Calls whose work overlaps on the GPU
// (different streams, or host threads racing on one device) race on the array.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "pack.cuh"
#include "slm.h"
#include "slm_internal.h"

namespace slm {

namespace {

constexpr uint32_t kNaMax = SLM_NOALLOC_MAX_DESCS;
constexpr uint32_t kChunksMax = 16;  // column chunks per row tile

constexpr size_t align256(size_t x) { return (x + 255) / 256 * 256; }

// Largest layout (na = nb = kNaMax): the size of the static array.
constexpr size_t max_layout_bytes() {
    const size_t tiles = kNaMax / kTile;
    const size_t items = tiles * kChunksMax;
    return align256(sizeof(float) * (size_t)kTileFloats * 2 * tiles) + align256(sizeof(Item) * items) +
           align256(sizeof(RowPart) * kTile * items) + align256(sizeof(PairMeta)) +
           align256(sizeof(unsigned long long) * kNaMax) + align256(sizeof(uint2) * kNaMax) +
           align256(sizeof(uint32_t)) + align256(sizeof(uint32_t) * 16);
}
constexpr size_t kNoAllocBytes = max_layout_bytes();

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

struct DeviceSetup {
    bool ready = false;
    unsigned char *scratch = nullptr;  // device address of g_noalloc_scratch
    int sms = 0;
};

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
DeviceSetup g_setup[kMaxDevices];

// Everything before the exact kernel, in one launch of 4 x (row tiles of a +
// row tiles of b) CTAs: CTA k packs 32-row group k % 4 of tile k / 4 (the
// tiles of a, then those of b); CTA 0 also writes the pair's metadata and work
// items and clears the work counter, error word and match count; with the
// cross-check every CTA clears its share of the column keys.
__global__ void __launch_bounds__(256) single_prep_kernel(unsigned char *scratch, SingleLayout L, const float *d_a,
                                                          uint32_t na, const float *d_b, uint32_t nb, int mutual) {
    __shared__ float sm[32][kDesc + 1];
    if (blockIdx.x == 0) {
        Item *items = reinterpret_cast<Item *>(scratch + L.items);
        PairMeta *meta = reinterpret_cast<PairMeta *>(scratch + L.meta);
        uint32_t *ctl = reinterpret_cast<uint32_t *>(scratch + L.ctl);
        uint32_t *counts = reinterpret_cast<uint32_t *>(scratch + L.counts);
        const uint32_t chunks = L.chunks, n_items = L.rt_n * chunks;
        for (uint32_t k = threadIdx.x; k < n_items; k += blockDim.x) {
            const uint32_t rt = k / chunks, c = k % chunks;
            Item it;
            it.pair = 0;
            it.rt = rt;
            it.ct0 = (uint32_t)((uint64_t)L.ct_n * c / chunks);
            it.ct1 = (uint32_t)((uint64_t)L.ct_n * (c + 1) / chunks);
            it.part = k;  // = rt * chunks + c, the layout finalize_kernel reads
            it.pad[0] = it.pad[1] = it.pad[2] = 0;
            items[k] = it;
        }
        if (threadIdx.x == 0) {
            PairMeta m;
            m.a_row0 = 0;
            m.b_row0 = L.rt_n * kTile;
            m.na = na;
            m.nb = nb;
            m.nchunk = chunks;
            m.part_base = 0;
            m.col_base = 0;
            m.slot_off = 0;
            *meta = m;
            *counts = 0;
        }
        if (threadIdx.x < 16) ctl[threadIdx.x] = 0;
    }
    if (mutual) {
        unsigned long long *colbest = reinterpret_cast<unsigned long long *>(scratch + L.colbest);
        for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nb; k += gridDim.x * blockDim.x)
            colbest[k] = ~0ull;
    }
    float *tiled = reinterpret_cast<float *>(scratch + L.tiled);
    const uint32_t t = blockIdx.x >> 2;
    const int g = (int)(blockIdx.x & 3);
    if (t < L.rt_n)
        pack_group(d_a, na, tiled + (size_t)t * kTileFloats, t, g, sm);
    else
        pack_group(d_b, nb, tiled + (size_t)t * kTileFloats, t - L.rt_n, g, sm);
}

// Copies the match list to the caller's buffer (at most cap pairs) and writes
// the full count, or 0xffffffff if a bounded device wait gave up.
__global__ void single_copy_kernel(const unsigned char *scratch, SingleLayout L, slm_pair *out, uint32_t cap,
                                   uint32_t *d_count) {
    const uint2 *slots = reinterpret_cast<const uint2 *>(scratch + L.slots);
    const uint32_t n = *reinterpret_cast<const uint32_t *>(scratch + L.counts);
    const uint32_t err = reinterpret_cast<const uint32_t *>(scratch + L.ctl)[1];
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n && t < cap; t += gridDim.x * blockDim.x) {
        const uint2 v = slots[t];
        out[t].i = v.x;
        out[t].j = v.y;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *d_count = err ? 0xffffffffu : n;
}

slm_status na_fail(slm_status s, const std::string &m) {
    set_last_error(m.c_str());
    return s;
}

// Once per device, with that device current.
slm_status device_setup(int dev, DeviceSetup *out) {
    if (dev < 0 || dev >= kMaxDevices) return na_fail(SLM_NO_DEVICE, "device ordinal out of range");
    std::lock_guard<std::mutex> g(g_setup_mu);
    DeviceSetup &d = g_setup[dev];
    if (!d.ready) {
        int major = 0, minor = 0, sms = 0;
        if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
            cudaGetLastError();
            return na_fail(SLM_NO_DEVICE, "cannot query the current device");
        }
        if (!(major == 10 && minor == 3)) return na_fail(SLM_NO_DEVICE, "libslm is built for sm_103a");
        void *ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr) {
            cudaGetLastError();
            return na_fail(SLM_CUDA_ERROR, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
        }
        const cudaError_t ke = init_exact_kernels();
        if (ke != cudaSuccess) {
            cudaGetLastError();
            return na_fail(SLM_NO_DEVICE, std::string("kernels do not load on this device: ") + cudaGetErrorString(ke));
        }
        d.scratch = static_cast<unsigned char *>(ptr);
        d.sms = sms;
        d.ready = true;
    }
    *out = d;
    return SLM_OK;
}

}  // namespace

SingleLayout single_layout(uint32_t na, uint32_t nb, int sms, bool inputs) {
    SingleLayout L{};
    L.rt_n = (na + kTile - 1) / kTile;
    L.ct_n = (nb + kTile - 1) / kTile;
    const uint32_t want = (uint32_t)(sms > 0 ? sms : 1) * 4;
    uint32_t chunks = L.rt_n ? (want + L.rt_n - 1) / L.rt_n : 1;
    chunks = chunks > L.ct_n ? L.ct_n : chunks;
    chunks = chunks > kChunksMax ? kChunksMax : chunks;
    L.chunks = chunks < 1 ? 1 : chunks;
    const size_t items = (size_t)L.rt_n * L.chunks;
    size_t o = 0;
    L.tiled = o, o += align256(sizeof(float) * (size_t)kTileFloats * (L.rt_n + L.ct_n));
    L.items = o, o += align256(sizeof(Item) * items);
    L.parts = o, o += align256(sizeof(RowPart) * kTile * items);
    L.meta = o, o += align256(sizeof(PairMeta));
    L.colbest = o, o += align256(sizeof(unsigned long long) * (nb ? nb : 1));
    L.slots = o, o += align256(sizeof(uint2) * (na ? na : 1));
    L.counts = o, o += align256(sizeof(uint32_t));
    L.ctl = o, o += align256(sizeof(uint32_t) * 16);
    if (inputs) {  // row-major inputs, for callers whose inputs the device cannot read where they lie
        L.raw_a = o, o += align256(sizeof(float) * kDesc * (size_t)(na ? na : 1));
        L.raw_b = o, o += align256(sizeof(float) * kDesc * (size_t)(nb ? nb : 1));
    }
    L.bytes = o;
    return L;
}

// The exact FP32 match of one pair (prep -> exact_kernel -> finalize [-> copy])
// over a scratch block laid out by single_layout: no metadata from the host.
cudaError_t single_exact_enqueue(unsigned char *sc, const SingleLayout &L, const float *d_a, uint32_t na,
                                 const float *d_b, uint32_t nb, float ratio, int mutual, slm_pair *d_out,
                                 uint32_t cap, uint32_t *d_count, int sms, cudaStream_t s) {
    const uint32_t n_items = L.rt_n * L.chunks;
    float *tiled = reinterpret_cast<float *>(sc + L.tiled);
    single_prep_kernel<<<4 * (L.rt_n + L.ct_n), 256, 0, s>>>(sc, L, d_a, na, d_b, nb, mutual);
    ExactArgs a{};
    a.tiled = tiled;
    a.items = reinterpret_cast<const Item *>(sc + L.items);
    a.n_items = n_items;
    a.pairs = reinterpret_cast<const PairMeta *>(sc + L.meta);
    a.parts = reinterpret_cast<RowPart *>(sc + L.parts);
    a.colbest = reinterpret_cast<unsigned long long *>(sc + L.colbest);
    a.work = reinterpret_cast<uint32_t *>(sc + L.ctl);
    a.err = reinterpret_cast<uint32_t *>(sc + L.ctl) + 1;
    a.mutual = mutual ? 1 : 0;
    a.x2 = 1;
    launch_exact(a, (int)(n_items < (uint32_t)sms ? n_items : (uint32_t)sms), s);
    FinalizeArgs f{};
    f.pairs = a.pairs;
    f.npairs = 1;
    f.parts = a.parts;
    f.colbest = a.colbest;
    f.ratio2 = ratio * ratio;
    f.mutual = a.mutual;
    if (single_direct_output(d_out, cap, na)) {
        // room for every possible match: finalize writes the list and the
        // count (or the error mark) straight into the caller's buffers
        f.slots = reinterpret_cast<uint2 *>(d_out);
        f.counts = d_count;
        f.err = a.err;
        launch_finalize(f, s);
    } else {
        f.slots = reinterpret_cast<uint2 *>(sc + L.slots);
        f.counts = reinterpret_cast<uint32_t *>(sc + L.counts);
        launch_finalize(f, s);
        single_copy_kernel<<<16, 256, 0, s>>>(sc, L, d_out, cap, d_count);
    }
    return cudaGetLastError();
}

}  // namespace slm

using namespace slm;

extern "C" slm_status slm_ratio_match_device_noalloc(const float *d_a, uint32_t na, const float *d_b, uint32_t nb,
                                                     float ratio, int mutual, slm_pair *d_out, uint32_t cap,
                                                     uint32_t *d_count, void *stream) {
    if ((na && !d_a) || (nb && !d_b) || !d_count || (cap && !d_out))
        return na_fail(SLM_INVALID_ARG, "NULL argument");
    if (!(ratio == ratio) || ratio - ratio != 0.0f) return na_fail(SLM_INVALID_ARG, "ratio must be finite");
    if (na > kNaMax || nb > kNaMax)
        return na_fail(SLM_INVALID_ARG, "slm_ratio_match_device_noalloc handles at most " + std::to_string(kNaMax) +
                                            " descriptors per side (got na=" + std::to_string(na) +
                                            ", nb=" + std::to_string(nb) + ")");
    if ((reinterpret_cast<uintptr_t>(d_a) | reinterpret_cast<uintptr_t>(d_b)) & 15u)
        return na_fail(SLM_INVALID_ARG, "d_a and d_b must be 16-byte aligned");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return na_fail(SLM_NO_DEVICE, "no current CUDA device");
    }
    DeviceSetup ds;
    slm_status st = device_setup(dev, &ds);
    if (st != SLM_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (na == 0 || nb < 2) {  // matching.rs:160-166: nothing can pass the ratio test
        if (cudaMemsetAsync(d_count, 0, sizeof(uint32_t), s) != cudaSuccess) {
            cudaGetLastError();
            return na_fail(SLM_CUDA_ERROR, "cudaMemsetAsync(d_count) failed");
        }
        return SLM_OK;
    }
    const SingleLayout L = single_layout(na, nb, ds.sms, false);
    if (L.bytes > kNoAllocBytes) return na_fail(SLM_INTERNAL, "scratch layout exceeds the static array");
    const cudaError_t le = single_exact_enqueue(ds.scratch, L, d_a, na, d_b, nb, ratio, mutual, d_out, cap, d_count,
                                                ds.sms, s);
    if (le != cudaSuccess) return na_fail(SLM_CUDA_ERROR, std::string("launch failed: ") + cudaGetErrorString(le));
    return SLM_OK;
}
