// lsgb_engine.cpp -- host side of the Lomb-Scargle engine and the lsgb_* C ABI.
//
// Replaces the reference's per-call host driver source/main.cu:1006-1280
// (batchGPULS) and :570-720 (GPULSOneObject): instead of cudaMalloc/cudaFree on
// every call, one OpenMP-free host thread, a synchronous kernel and a host argmax
// over the returned periodogram, an engine keeps grow-only device buffers, plans a
// size-ordered work queue of (object, frequency tile) units for one persistent
// kernel, and computes the per-object argmax on the device. The periodogram is
// written only when the caller passes a buffer for it.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/lsgb.h"
#include "lsgb_internal.h"

using namespace lsgb;

namespace {

thread_local std::string g_last_error;

int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

#define LSGB_CUDA(call)                                                                     \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess)                                                              \
            return fail(e_ == cudaErrorMemoryAllocation ? LSGB_ERR_NOMEM : LSGB_ERR_CUDA,   \
                        "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                        __LINE__);                                                          \
    } while (0)

struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        const size_t want = std::max<size_t>(bytes, 256);
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

// 1/(2 pi) as a double-double (hi + lo).
constexpr double kInv2PiHi = 0.15915494309189535;
constexpr double kInv2PiLo = -9.839338337591243e-18;

void two_prod(double a, double b_hi, double b_lo, double &hi, double &lo) {
    hi = a * b_hi;
    lo = std::fma(a, b_hi, -hi) + a * b_lo;
    const double s = hi + lo;  // renormalize
    lo = lo - (s - hi);
    hi = s;
}

}  // namespace

namespace lsgb {
// Lets other translation units of the library report through lsgb_last_error().
void set_last_error(const char *msg) { g_last_error = msg; }
}  // namespace lsgb

struct lsgb_engine {
    int device = 0;
    int sms = 0;
    cudaStream_t stream = nullptr;  // host-buffer API stream
    DevBuf objs, offs, perm, rec, tile_best, counter, keys;
    DevBuf in_t, in_y, in_dy, out_pg, out_idx, out_p;
    MixedShape shape[2] = {{12, 256, 2, 1, 0}, {8, 256, 2, 1, 0}};
    uint32_t last_kernels = 0;
    uint64_t last_units = 0;
    cudaEvent_t ev_main0 = nullptr, ev_main1 = nullptr;  // around the last main-kernel launch
    bool ev_valid = false;
    uint32_t reanchor = 0;  // mixed form: 0 = anchor at each thread's frequency run
};

extern "C" {

LSGB_API const char *lsgb_last_error(void) { return g_last_error.c_str(); }

LSGB_API const char *lsgb_version(void) { return "lsgb 0.1 (sm_103a)"; }

LSGB_API int lsgb_engine_create(int device, lsgb_engine **out) {
    if (!out) return fail(LSGB_ERR_INVALID, "lsgb_engine_create: out is NULL");
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0)
        return fail(LSGB_ERR_NODEVICE, "no CUDA device available (%s)",
                    e != cudaSuccess ? cudaGetErrorString(e) : "count 0");
    if (device < 0 || device >= count)
        return fail(LSGB_ERR_INVALID, "device %d out of range [0, %d)", device, count);
    LSGB_CUDA(cudaSetDevice(device));
    lsgb_engine *eng = new lsgb_engine();
    eng->device = device;
    cudaError_t e2 = cudaDeviceGetAttribute(&eng->sms, cudaDevAttrMultiProcessorCount, device);
    if (e2 == cudaSuccess) e2 = cudaStreamCreateWithFlags(&eng->stream, cudaStreamNonBlocking);
    if (e2 == cudaSuccess) e2 = eng->counter.ensure(256);
    if (e2 == cudaSuccess) e2 = cudaEventCreate(&eng->ev_main0);
    if (e2 == cudaSuccess) e2 = cudaEventCreate(&eng->ev_main1);
    if (e2 != cudaSuccess) {
        delete eng;
        return fail(LSGB_ERR_CUDA, "engine set-up failed: %s", cudaGetErrorString(e2));
    }
    *out = eng;
    return LSGB_OK;
}

LSGB_API void lsgb_engine_destroy(lsgb_engine *eng) {
    if (!eng) return;
    cudaSetDevice(eng->device);
    if (eng->stream) cudaStreamSynchronize(eng->stream);
    DevBuf *bufs[] = {&eng->objs,   &eng->offs,  &eng->perm,    &eng->rec,
                      &eng->tile_best, &eng->counter, &eng->keys, &eng->in_t, &eng->in_y,
                      &eng->in_dy,  &eng->out_pg, &eng->out_idx, &eng->out_p};
    for (DevBuf *b : bufs) b->release();
    if (eng->stream) cudaStreamDestroy(eng->stream);
    if (eng->ev_main0) cudaEventDestroy(eng->ev_main0);
    if (eng->ev_main1) cudaEventDestroy(eng->ev_main1);
    delete eng;
}

LSGB_API int lsgb_set_tuning(lsgb_engine *eng, int variant, int f, int nt, int minb, int x2,
                             int unroll) {
    if (!eng || (variant != 0 && variant != 1))
        return fail(LSGB_ERR_INVALID, "lsgb_set_tuning: bad engine or variant");
    MixedShape s = eng->shape[variant];
    if (f > 0) s.f = f;
    if (nt > 0) s.nt = nt;
    if (minb > 0) s.minb = minb;
    if (x2 >= 0) s.x2 = x2 ? 1 : 0;
    if (unroll >= 0) s.uj = unroll ? 1 : 0;
    int blocks = 0;
    if (mixed_occupancy(variant, LSGB_F32, s, 1024, &blocks) != cudaSuccess)
        return fail(LSGB_ERR_INVALID,
                    "mixed shape F=%d x %d threads (min %d CTAs/SM, packed %d, unroll %d) is not "
                    "compiled for variant %d", s.f, s.nt, s.minb, s.x2, s.uj, variant);
    eng->shape[variant] = s;
    return LSGB_OK;
}

LSGB_API int lsgb_mixed_shapes(int *out, int max_shapes) { return mixed_shapes(out, max_shapes); }

LSGB_API int lsgb_fp64_sincos_check(lsgb_engine *eng, uint32_t n, double scale, double *max_err) {
    if (!eng || !max_err) return fail(LSGB_ERR_INVALID, "lsgb_fp64_sincos_check: NULL argument");
    LSGB_CUDA(cudaSetDevice(eng->device));
    DevBuf d;
    LSGB_CUDA(d.ensure(sizeof(double)));
    LSGB_CUDA(cudaMemsetAsync(d.p, 0, sizeof(double), eng->stream));
    LSGB_CUDA(launch_sincos_check(n, 12345, scale, (double *)d.p, eng->stream));
    LSGB_CUDA(cudaMemcpyAsync(max_err, d.p, sizeof(double), cudaMemcpyDeviceToHost, eng->stream));
    LSGB_CUDA(cudaStreamSynchronize(eng->stream));
    d.release();
    return LSGB_OK;
}

LSGB_API int lsgb_set_reanchor(lsgb_engine *eng, uint32_t interval) {
    if (!eng) return fail(LSGB_ERR_INVALID, "lsgb_set_reanchor: engine is NULL");
    eng->reanchor = interval;
    return LSGB_OK;
}

LSGB_API int lsgb_get_tuning(lsgb_engine *eng, int variant, int *out6) {
    if (!eng || !out6 || (variant != 0 && variant != 1))
        return fail(LSGB_ERR_INVALID, "lsgb_get_tuning: bad argument");
    const MixedShape s = eng->shape[variant];
    out6[0] = variant;
    out6[1] = s.f;
    out6[2] = s.nt;
    out6[3] = s.minb;
    out6[4] = s.x2;
    out6[5] = s.uj;
    return LSGB_OK;
}

LSGB_API int lsgb_last_launch_info(lsgb_engine *eng, uint32_t *kernels, uint64_t *units) {
    if (!eng) return fail(LSGB_ERR_INVALID, "lsgb_last_launch_info: engine is NULL");
    if (kernels) *kernels = eng->last_kernels;
    if (units) *units = eng->last_units;
    return LSGB_OK;
}

LSGB_API int lsgb_last_kernel_time(lsgb_engine *eng, float *ms) {
    if (!eng || !ms) return fail(LSGB_ERR_INVALID, "lsgb_last_kernel_time: NULL argument");
    if (!eng->ev_valid) return fail(LSGB_ERR_INVALID, "no main kernel has been launched");
    LSGB_CUDA(cudaEventSynchronize(eng->ev_main1));
    LSGB_CUDA(cudaEventElapsedTime(ms, eng->ev_main0, eng->ev_main1));
    return LSGB_OK;
}

LSGB_API int lsgb_periodogram_device(lsgb_engine *eng, int variant, int precision, int dtype,
                                     const void *t, const void *y, const void *dy,
                                     const uint64_t *offsets, uint32_t n_obj, double fmin,
                                     double df, uint32_t n_freq, int normalize, void *pgram,
                                     uint32_t *best_idx, void *best_power, void *stream_) {
    if (!eng) return fail(LSGB_ERR_INVALID, "engine is NULL");
    if (variant != LSGB_STANDARD && variant != LSGB_GENERALIZED)
        return fail(LSGB_ERR_INVALID, "variant %d is not LSGB_STANDARD or LSGB_GENERALIZED", variant);
    if (precision != LSGB_PLAIN_FP64 && precision != LSGB_MIXED)
        return fail(LSGB_ERR_INVALID, "precision %d is not LSGB_PLAIN_FP64 or LSGB_MIXED", precision);
    if (dtype != LSGB_F32 && dtype != LSGB_F64)
        return fail(LSGB_ERR_INVALID, "dtype %d is not LSGB_F32 or LSGB_F64", dtype);
    if (n_obj == 0) return fail(LSGB_ERR_INVALID, "n_obj is 0");
    if (!offsets) return fail(LSGB_ERR_INVALID, "offsets is NULL");
    if (!t || !y) return fail(LSGB_ERR_INVALID, "t or y is NULL");
    if (variant == LSGB_GENERALIZED && !dy)
        return fail(LSGB_ERR_INVALID, "dy is NULL for the generalized variant");
    if (!std::isfinite(fmin) || !std::isfinite(df))
        return fail(LSGB_ERR_INVALID, "fmin/df must be finite");
    if (offsets[0] != 0) return fail(LSGB_ERR_INVALID, "offsets[0] must be 0");
    uint32_t max_n = 0;
    std::vector<ObjInfo> h_objs(n_obj);
    for (uint32_t o = 0; o < n_obj; ++o) {
        if (offsets[o + 1] <= offsets[o])
            return fail(LSGB_ERR_INVALID, "object %u has no observations (offsets must increase)", o);
        const uint64_t n = offsets[o + 1] - offsets[o];
        if (n > 0xffffffffull) return fail(LSGB_ERR_INVALID, "object %u has more than 2^32-1 rows", o);
        ObjInfo ob{};
        ob.row0 = offsets[o];
        ob.n = (uint32_t)n;
        h_objs[o] = ob;
        max_n = std::max<uint32_t>(max_n, (uint32_t)n);
    }
    eng->last_kernels = 0;
    eng->last_units = 0;
    if (n_freq == 0) return LSGB_OK;  // nothing to compute or write
    const uint64_t rows = offsets[n_obj];
    cudaStream_t st = (cudaStream_t)stream_;
    LSGB_CUDA(cudaSetDevice(eng->device));

    // Work order: largest objects first (longest-processing-time first), ties by index.
    std::vector<uint32_t> h_perm(n_obj);
    std::iota(h_perm.begin(), h_perm.end(), 0u);
    std::stable_sort(h_perm.begin(), h_perm.end(),
                     [&](uint32_t a, uint32_t b) { return h_objs[a].n > h_objs[b].n; });

    const bool mixed = precision == LSGB_MIXED;
    const MixedShape shape = eng->shape[variant];
    const uint32_t tile_freqs = mixed ? (uint32_t)(shape.f * shape.nt) : (uint32_t)kPlainThreads;
    const uint64_t n_tiles64 = (n_freq + (uint64_t)tile_freqs - 1) / tile_freqs;
    const uint64_t n_units64 = n_tiles64 * n_obj;
    if (n_units64 >= 0xffffffffull)
        return fail(LSGB_ERR_INVALID, "%llu work units exceed the 2^32 queue; split the batch",
                    (unsigned long long)n_units64);
    const uint32_t n_tiles = (uint32_t)n_tiles64;
    const bool want_best = best_idx || best_power;

    LSGB_CUDA(eng->objs.ensure(sizeof(ObjInfo) * n_obj));
    LSGB_CUDA(eng->offs.ensure(sizeof(uint64_t) * (n_obj + 1)));
    LSGB_CUDA(eng->perm.ensure(sizeof(uint32_t) * n_obj));
    if (want_best && !mixed) LSGB_CUDA(eng->tile_best.ensure(sizeof(TileBest) * n_units64));
    if (want_best && mixed) {
        LSGB_CUDA(eng->keys.ensure(sizeof(unsigned long long) * n_obj));
        LSGB_CUDA(cudaMemsetAsync(eng->keys.p, 0, sizeof(unsigned long long) * n_obj, st));
    }
    if (mixed) LSGB_CUDA(eng->rec.ensure(sizeof(ObsRec) * rows));
    LSGB_CUDA(cudaMemcpyAsync(eng->objs.p, h_objs.data(), sizeof(ObjInfo) * n_obj,
                              cudaMemcpyHostToDevice, st));
    LSGB_CUDA(cudaMemcpyAsync(eng->offs.p, offsets, sizeof(uint64_t) * (n_obj + 1),
                              cudaMemcpyHostToDevice, st));
    LSGB_CUDA(cudaMemcpyAsync(eng->perm.p, h_perm.data(), sizeof(uint32_t) * n_obj,
                              cudaMemcpyHostToDevice, st));
    LSGB_CUDA(cudaMemsetAsync(eng->counter.p, 0, sizeof(uint32_t), st));

    ObjInfo *d_objs = (ObjInfo *)eng->objs.p;
    uint32_t kernels = 0;
    LSGB_CUDA(launch_stats(variant, mixed ? 1 : 0, dtype, normalize, y, dy, d_objs, n_obj, st));
    ++kernels;
    if (mixed) {
        GridTurns g;
        two_prod(fmin, kInv2PiHi, kInv2PiLo, g.f0_hi, g.f0_lo);
        two_prod(df, kInv2PiHi, kInv2PiLo, g.df_hi, g.df_lo);
        LSGB_CUDA(launch_records(variant, dtype, t, y, dy, (const uint64_t *)eng->offs.p, n_obj,
                                 d_objs, rows, g, (ObsRec *)eng->rec.p, st));
        ++kernels;
        const uint32_t rec_bytes = (uint32_t)mixed_rec_bytes(shape);
        const uint32_t chunk = std::min<uint32_t>(max_n, kMixedSmemMax / rec_bytes);
        // objects longer than one chunk sum in two levels (chunk sums folded in smem)
        const bool fold = max_n > chunk;
        const size_t smem = (size_t)rec_bytes * chunk + (fold ? mixed_fold_bytes(variant, shape) : 0);
        int occ = 0;
        LSGB_CUDA(mixed_occupancy(variant, dtype, shape, smem, &occ));
        if (occ < 1) return fail(LSGB_ERR_CUDA, "mixed kernel does not fit on an SM (smem %zu)", smem);
        MixedArgs a{};
        a.rec = (const ObsRec *)eng->rec.p;
        a.objs = d_objs;
        a.perm = (const uint32_t *)eng->perm.p;
        a.n_obj = n_obj;
        a.n_tiles = n_tiles;
        a.n_freq = n_freq;
        a.chunk = chunk;
        a.counter = (uint32_t *)eng->counter.p;
        a.pgram = pgram;
        a.tile_best = nullptr;
        a.best_key = want_best ? (unsigned long long *)eng->keys.p : nullptr;
        a.reanchor = eng->reanchor;
        a.fold = fold ? 1u : 0u;
        const int grid = (int)std::min<uint64_t>((uint64_t)eng->sms * occ, n_units64);
        LSGB_CUDA(cudaEventRecord(eng->ev_main0, st));
        LSGB_CUDA(launch_mixed(variant, dtype, shape, a, grid, smem, st));
        LSGB_CUDA(cudaEventRecord(eng->ev_main1, st));
        eng->ev_valid = true;
        ++kernels;
    } else {
        const uint32_t chunk = std::min<uint32_t>(max_n, kPlainChunkMax);
        const size_t smem = sizeof(double) * chunk * (variant == LSGB_GENERALIZED ? 3 : 2);
        int occ = 0;
        LSGB_CUDA(plain_occupancy(variant, dtype, dtype, smem, &occ));
        if (occ < 1) return fail(LSGB_ERR_CUDA, "plain kernel does not fit on an SM (smem %zu)", smem);
        PlainArgs a{};
        a.t = t;
        a.y = y;
        a.dy = dy;
        a.objs = d_objs;
        a.perm = (const uint32_t *)eng->perm.p;
        a.n_obj = n_obj;
        a.n_tiles = n_tiles;
        a.n_freq = n_freq;
        a.chunk = chunk;
        a.fmin = fmin;
        a.df = df;
        a.counter = (uint32_t *)eng->counter.p;
        a.pgram = pgram;
        a.tile_best = want_best ? (TileBest *)eng->tile_best.p : nullptr;
        const int grid = (int)std::min<uint64_t>((uint64_t)eng->sms * occ, n_units64);
        LSGB_CUDA(cudaEventRecord(eng->ev_main0, st));
        LSGB_CUDA(launch_plain(variant, dtype, dtype, a, grid, smem, st));
        LSGB_CUDA(cudaEventRecord(eng->ev_main1, st));
        eng->ev_valid = true;
        ++kernels;
    }
    if (want_best && mixed) {
        LSGB_CUDA(launch_key_decode(dtype, (const unsigned long long *)eng->keys.p, n_obj, best_idx,
                                    best_power, st));
        ++kernels;
    } else if (want_best) {
        LSGB_CUDA(launch_best_reduce(dtype, (const TileBest *)eng->tile_best.p, n_obj, n_tiles,
                                     best_idx, best_power, st));
        ++kernels;
    }
    eng->last_kernels = kernels;
    eng->last_units = n_units64;
    return LSGB_OK;
}

LSGB_API int lsgb_periodogram_host(lsgb_engine *eng, int variant, int precision, int dtype,
                                   const void *t, const void *y, const void *dy,
                                   const uint64_t *offsets, uint32_t n_obj, double fmin, double df,
                                   uint32_t n_freq, int normalize, void *pgram, uint32_t *best_idx,
                                   void *best_power) {
    if (!eng) return fail(LSGB_ERR_INVALID, "engine is NULL");
    if (!offsets || n_obj == 0) return fail(LSGB_ERR_INVALID, "offsets is NULL or n_obj is 0");
    if (dtype != LSGB_F32 && dtype != LSGB_F64)
        return fail(LSGB_ERR_INVALID, "dtype %d is not LSGB_F32 or LSGB_F64", dtype);
    if (!t || !y || (variant == LSGB_GENERALIZED && !dy))
        return fail(LSGB_ERR_INVALID, "t, y (and dy for the generalized variant) must be non-NULL");
    const size_t es = dtype == LSGB_F32 ? 4 : 8;
    const uint64_t rows = offsets[n_obj];
    LSGB_CUDA(cudaSetDevice(eng->device));
    cudaStream_t st = eng->stream;
    LSGB_CUDA(eng->in_t.ensure(es * rows));
    LSGB_CUDA(eng->in_y.ensure(es * rows));
    LSGB_CUDA(cudaMemcpyAsync(eng->in_t.p, t, es * rows, cudaMemcpyHostToDevice, st));
    LSGB_CUDA(cudaMemcpyAsync(eng->in_y.p, y, es * rows, cudaMemcpyHostToDevice, st));
    const void *d_dy = nullptr;
    if (variant == LSGB_GENERALIZED) {
        LSGB_CUDA(eng->in_dy.ensure(es * rows));
        LSGB_CUDA(cudaMemcpyAsync(eng->in_dy.p, dy, es * rows, cudaMemcpyHostToDevice, st));
        d_dy = eng->in_dy.p;
    }
    void *d_pg = nullptr;
    uint32_t *d_idx = nullptr;
    void *d_p = nullptr;
    const uint64_t pg_elems = (uint64_t)n_obj * n_freq;
    if (pgram && pg_elems) {
        LSGB_CUDA(eng->out_pg.ensure(es * pg_elems));
        d_pg = eng->out_pg.p;
    }
    if (best_idx) {
        LSGB_CUDA(eng->out_idx.ensure(sizeof(uint32_t) * n_obj));
        d_idx = (uint32_t *)eng->out_idx.p;
    }
    if (best_power) {
        LSGB_CUDA(eng->out_p.ensure(es * n_obj));
        d_p = eng->out_p.p;
    }
    int rc = lsgb_periodogram_device(eng, variant, precision, dtype, eng->in_t.p, eng->in_y.p, d_dy,
                                     offsets, n_obj, fmin, df, n_freq, normalize, d_pg, d_idx, d_p,
                                     (void *)st);
    if (rc != LSGB_OK) {
        cudaStreamSynchronize(st);
        return rc;
    }
    if (n_freq == 0) {
        // nothing computed: report index 0 / power 0 as the reference's argmax would
        if (best_idx) memset(best_idx, 0, sizeof(uint32_t) * n_obj);
        if (best_power) memset(best_power, 0, es * n_obj);
        LSGB_CUDA(cudaStreamSynchronize(st));
        return LSGB_OK;
    }
    if (d_pg) LSGB_CUDA(cudaMemcpyAsync(pgram, d_pg, es * pg_elems, cudaMemcpyDeviceToHost, st));
    if (d_idx)
        LSGB_CUDA(cudaMemcpyAsync(best_idx, d_idx, sizeof(uint32_t) * n_obj, cudaMemcpyDeviceToHost, st));
    if (d_p) LSGB_CUDA(cudaMemcpyAsync(best_power, d_p, es * n_obj, cudaMemcpyDeviceToHost, st));
    LSGB_CUDA(cudaStreamSynchronize(st));
    return LSGB_OK;
}

}  // extern "C"
