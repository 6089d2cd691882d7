// lsgb_noalloc.cu -- lsgb_periodogram_noalloc: the mixed-form batch periodogram with
// every piece of device scratch it needs held in one fixed-size array compiled into
// liblsgb.so, so a call allocates no memory at all.
//
// Who needs it. The regular entry points grow engine-owned buffers with cudaMalloc
// when a batch is larger than any before it. Some callers cannot let that happen on
// their call path: a host framework whose own allocator owns the whole device-memory
// budget (a plugin that calls cudaMalloc behind its back breaks that accounting, or
// fails once the framework has reserved the memory), a latency-critical loop that
// cannot absorb the device-wide synchronization cudaMalloc/cudaFree may cause, and a
// service that must reach its full memory footprint at start-up and never grow
// afterwards. For them this entry point works inside a fixed reservation: the caller
// passes inputs and outputs, the library never allocates.
//
// The price: the array below is reserved on every GPU that loads liblsgb.so, from
// the first CUDA use of the library until the process exits, and a call is limited
// to the sizes it was compiled for (kNoAllocMax*).
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <algorithm>
#include <mutex>

#include "../../include/lsgb.h"
#include "lsgb_internal.h"

namespace lsgb {
void set_last_error(const char *msg);  // lsgb_engine.cpp
}

using namespace lsgb;

namespace {

// Size limits of one call.
constexpr uint32_t kNoAllocMaxRows = 131072;      // observations (all objects together)
constexpr uint32_t kNoAllocMaxObjects = 2048;     // objects
constexpr uint32_t kNoAllocMaxTileUnits = 262144; // objects x frequency tiles

// Layout of the scratch array (byte offsets, each 256-byte aligned).
constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kOffRec = 0;
constexpr size_t kOffObjs = align256(kOffRec + sizeof(ObsRec) * kNoAllocMaxRows);
constexpr size_t kOffOffsets = align256(kOffObjs + sizeof(ObjInfo) * kNoAllocMaxObjects);
constexpr size_t kOffPerm = align256(kOffOffsets + sizeof(uint64_t) * (kNoAllocMaxObjects + 1));
constexpr size_t kOffTileBest = align256(kOffPerm + sizeof(uint32_t) * kNoAllocMaxObjects);
constexpr size_t kOffCounter = align256(kOffTileBest + sizeof(TileBest) * kNoAllocMaxTileUnits);
constexpr size_t kScratchBytes = align256(kOffCounter + sizeof(uint32_t));  // ~8.3 MiB

// The scratch array. Its name is only a host-side handle: host code must never hand
// it to a kernel; the device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// The mixed-kernel shapes this entry point uses (both compiled in lsgb_kernels.cu).
constexpr MixedShape kShapeStd = {12, 256, 2, 1};
constexpr MixedShape kShapeGen = {8, 256, 2, 1};

// Per-device set-up state: the device address of g_noalloc_scratch.
constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char *g_dev_ptr[kMaxDevices] = {nullptr};

// Host staging of the per-object tables, also fixed-size (no heap use per call).
// Guarded by g_mu: calls from several host threads serialize their set-up.
ObjInfo g_h_objs[kNoAllocMaxObjects];
uint32_t g_h_perm[kNoAllocMaxObjects];

int fail(int code, const char *msg) {
    set_last_error(msg);
    return code;
}

int fail_cuda(const char *what, cudaError_t e) {
    char buf[256];
    snprintf(buf, sizeof(buf), "lsgb_periodogram_noalloc: %s failed: %s", what,
             cudaGetErrorString(e));
    set_last_error(buf);
    return LSGB_ERR_CUDA;
}

constexpr double kInv2PiHi = 0.15915494309189535;
constexpr double kInv2PiLo = -9.839338337591243e-18;

void two_prod(double a, double &hi, double &lo) {
    hi = a * kInv2PiHi;
    lo = fma(a, kInv2PiHi, -hi) + a * kInv2PiLo;
    const double s = hi + lo;
    lo = lo - (s - hi);
    hi = s;
}

}  // namespace

extern "C" LSGB_API int lsgb_periodogram_noalloc(int variant, int dtype, const void *t,
                                                 const void *y, const void *dy,
                                                 const uint64_t *offsets, uint32_t n_obj,
                                                 double fmin, double df, uint32_t n_freq,
                                                 int normalize, void *pgram, uint32_t *best_idx,
                                                 void *best_power, void *stream) {
    if (variant != LSGB_STANDARD && variant != LSGB_GENERALIZED)
        return fail(LSGB_ERR_INVALID, "lsgb_periodogram_noalloc: bad variant");
    if (dtype != LSGB_F32 && dtype != LSGB_F64)
        return fail(LSGB_ERR_INVALID, "lsgb_periodogram_noalloc: bad dtype");
    if (!offsets || n_obj == 0 || !t || !y || (variant == LSGB_GENERALIZED && !dy))
        return fail(LSGB_ERR_INVALID, "lsgb_periodogram_noalloc: NULL input or no objects");
    if (n_obj > kNoAllocMaxObjects)
        return fail(LSGB_ERR_INVALID,
                    "lsgb_periodogram_noalloc: more than 2048 objects (fixed scratch limit)");
    if (offsets[0] != 0) return fail(LSGB_ERR_INVALID, "lsgb_periodogram_noalloc: offsets[0] != 0");
    for (uint32_t o = 0; o < n_obj; ++o)
        if (offsets[o + 1] <= offsets[o])
            return fail(LSGB_ERR_INVALID, "lsgb_periodogram_noalloc: an object has no rows");
    const uint64_t rows = offsets[n_obj];
    if (rows > kNoAllocMaxRows)
        return fail(LSGB_ERR_INVALID,
                    "lsgb_periodogram_noalloc: more than 131072 observations (fixed scratch limit)");
    const MixedShape shape = variant == LSGB_STANDARD ? kShapeStd : kShapeGen;
    const uint32_t tile_freqs = (uint32_t)(shape.f * shape.nt);
    const uint64_t n_tiles = ((uint64_t)n_freq + tile_freqs - 1) / tile_freqs;
    const uint64_t units = n_tiles * n_obj;
    if (units > kNoAllocMaxTileUnits)
        return fail(LSGB_ERR_INVALID,
                    "lsgb_periodogram_noalloc: objects x frequency tiles exceeds 262144 "
                    "(fixed scratch limit; a tile is 3072 or 2048 frequencies)");
    if (n_freq == 0) return LSGB_OK;
    cudaStream_t st = (cudaStream_t)stream;

    std::lock_guard<std::mutex> lk(g_mu);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail_cuda("cudaGetDevice", e);
    if (dev < 0 || dev >= kMaxDevices)
        return fail(LSGB_ERR_INVALID, "lsgb_periodogram_noalloc: device index above 63");
    if (!g_dev_ptr[dev]) {
        // once per device, with that device current: resolve the array's device address
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return fail_cuda("cudaGetSymbolAddress", e);
        g_dev_ptr[dev] = (unsigned char *)p;
    }
    unsigned char *base = g_dev_ptr[dev];
    ObsRec *d_rec = (ObsRec *)(base + kOffRec);
    ObjInfo *d_objs = (ObjInfo *)(base + kOffObjs);
    uint64_t *d_offs = (uint64_t *)(base + kOffOffsets);
    uint32_t *d_perm = (uint32_t *)(base + kOffPerm);
    TileBest *d_tb = (TileBest *)(base + kOffTileBest);
    uint32_t *d_counter = (uint32_t *)(base + kOffCounter);

    uint32_t max_n = 0;
    for (uint32_t o = 0; o < n_obj; ++o) {
        ObjInfo ob{};
        ob.row0 = offsets[o];
        ob.n = (uint32_t)(offsets[o + 1] - offsets[o]);
        g_h_objs[o] = ob;
        g_h_perm[o] = o;
        max_n = std::max(max_n, ob.n);
    }
    std::sort(g_h_perm, g_h_perm + n_obj, [](uint32_t a, uint32_t b) {
        return g_h_objs[a].n != g_h_objs[b].n ? g_h_objs[a].n > g_h_objs[b].n : a < b;
    });
    // Everything the kernels read back is rewritten here: the scratch keeps the last
    // call's contents, and the queue counter must start at zero.
    if ((e = cudaMemcpyAsync(d_objs, g_h_objs, sizeof(ObjInfo) * n_obj, cudaMemcpyHostToDevice,
                             st)) != cudaSuccess)
        return fail_cuda("cudaMemcpyAsync(objects)", e);
    if ((e = cudaMemcpyAsync(d_offs, offsets, sizeof(uint64_t) * (n_obj + 1),
                             cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return fail_cuda("cudaMemcpyAsync(offsets)", e);
    if ((e = cudaMemcpyAsync(d_perm, g_h_perm, sizeof(uint32_t) * n_obj, cudaMemcpyHostToDevice,
                             st)) != cudaSuccess)
        return fail_cuda("cudaMemcpyAsync(order)", e);
    if ((e = cudaMemsetAsync(d_counter, 0, sizeof(uint32_t), st)) != cudaSuccess)
        return fail_cuda("cudaMemsetAsync(counter)", e);
    // the host tables are consumed once the copies above have run
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail_cuda("cudaStreamSynchronize", e);

    if ((e = launch_stats(variant, 1, dtype, normalize, t, y, dy, d_objs, n_obj, nullptr, st)) !=
        cudaSuccess)
        return fail_cuda("statistics kernel", e);
    GridTurns g;
    two_prod(fmin, g.f0_hi, g.f0_lo);
    two_prod(df, g.df_hi, g.df_lo);
    if ((e = launch_records(variant, dtype, t, y, dy, d_offs, n_obj, d_objs, rows, g, d_rec, 0u, st)) !=
        cudaSuccess)
        return fail_cuda("records kernel", e);
    // Shared memory as the engine sizes it: staged observations up to what keeps the
    // shape's CTAs per SM resident, and for objects longer than one chunk a second-level
    // sum area after them (the chunk sums are folded there, so no long FP32 sum forms).
    int smem_sm = 0;
    if ((e = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev)) !=
        cudaSuccess)
        return fail_cuda("cudaDeviceGetAttribute", e);
    const size_t per_cta = (size_t)smem_sm / (size_t)std::max(1, shape.minb) - 1024 - 256;
    const uint32_t rec_bytes = (uint32_t)mixed_rec_bytes(shape);
    size_t rec_budget = std::min<size_t>(kMixedSmemMax, per_cta);
    uint32_t chunk = (uint32_t)std::min<size_t>(max_n, rec_budget / rec_bytes);
    const bool fold = max_n > chunk;
    const size_t fold_bytes = fold ? mixed_fold_bytes(variant, shape) : 0;
    if (fold) {
        rec_budget = per_cta >= fold_bytes + 64 * (size_t)rec_bytes
                         ? std::min<size_t>(kMixedSmemMax, per_cta - fold_bytes)
                         : 64 * (size_t)rec_bytes;
        chunk = (uint32_t)std::min<size_t>(max_n, rec_budget / rec_bytes);
    }
    const size_t smem = (size_t)rec_bytes * chunk + fold_bytes;
    int occ = 0, sms = 0;
    if ((e = mixed_occupancy(variant, dtype, shape, smem, &occ)) != cudaSuccess)
        return fail_cuda("occupancy query", e);
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
        return fail_cuda("cudaDeviceGetAttribute", e);
    const bool want_best = best_idx || best_power;
    MixedArgs a{};
    a.rec = d_rec;
    a.objs = d_objs;
    a.perm = d_perm;
    a.n_obj = n_obj;
    a.n_tiles = (uint32_t)n_tiles;
    a.n_freq = n_freq;
    a.chunk = chunk;
    a.fold = fold ? 1u : 0u;
    a.counter = d_counter;
    a.pgram = pgram;
    a.tile_best = want_best ? d_tb : nullptr;
    a.top = 1u;
    const int grid = (int)std::min<uint64_t>((uint64_t)sms * (occ > 0 ? occ : 1), units);
    if ((e = launch_mixed(variant, dtype, shape, a, grid, smem, st)) != cudaSuccess)
        return fail_cuda("periodogram kernel", e);
    if (want_best &&
        (e = launch_best_reduce(dtype, d_tb, n_obj, (uint32_t)n_tiles, 1u, best_idx, best_power, st)) !=
            cudaSuccess)
        return fail_cuda("argmax kernel", e);
    return LSGB_OK;
}
