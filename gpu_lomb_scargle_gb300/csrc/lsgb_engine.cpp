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

// ---- one batch: plan (host), tables (upload), kernels (enqueue) ----------------------

// Device buffers one batch needs besides the caller's arrays.
struct Workspace {
    DevBuf objs, offs, perm, rec, tile_best, counter, keys;
    DevBuf optab;  // tensor form: per-K-block left operands and steps (tensor_optab_bytes)
    DevBuf partial;  // tensor form with K slices: each unit's raw sums (tensor_partial_bytes)
    DevBuf kbobj;    // tensor form: the object of every K-block of the batch
    DevBuf key3;     // tensor form, top three: every (object, tile)'s warp triples
    // sticky status word of the call's kernels (kStatusTimeout: a bounded pipeline wait of
    // the tensor form ran out; kStatusBadInput: non-finite or invalid inputs); zeroed when
    // allocated and after it is reported
    DevBuf status;
    void release() {
        DevBuf *b[] = {&objs, &offs, &perm, &rec, &tile_best, &counter, &keys, &optab, &partial,
                       &kbobj, &key3, &status};
        for (DevBuf *x : b) x->release();
    }
};

// Everything about a batch decided on the host.
struct Batch {
    bool empty = false;  // n_freq == 0: nothing to compute
    int variant = 0, precision = 0, dtype = 0, normalize = 0;
    const void *t = nullptr, *y = nullptr, *dy = nullptr;
    void *pgram = nullptr, *best_power = nullptr;
    uint32_t *best_idx = nullptr;
    uint32_t n_obj = 0, n_freq = 0, n_tiles = 0, max_n = 0, chunk = 0;
    uint64_t rows = 0, units = 0;
    uint64_t total_kb = 0;  // tensor form: K-blocks of the batch (operand table entries)
    uint32_t ksplit = 1;    // tensor form: slices of every object's K-blocks (units = pairs x ksplit)
    double fmin = 0, df = 0;
    MixedShape shape{};
    uint32_t reanchor = 0;
    bool want_best = false, fold = false;
    uint32_t top = 1;  // best frequencies per object: 1 (argmax) or 3 (the top three)
    long long wait_cycles = 0;  // tensor form: bounded-wait limit (0: the kernel's default)
    size_t smem = 0;
    int grid = 0;
    uint32_t kernels = 0;
    std::vector<ObjInfo> objs;
    std::vector<uint32_t> perm;
    std::vector<uint64_t> offsets;
    std::vector<uint32_t> kbobj;  // tensor form: object of each K-block (the table's rows)
};

int plan_batch(Batch &b, int sms, const MixedShape *shapes, uint32_t reanchor, int variant,
               int precision, int dtype, const void *t, const void *y, const void *dy,
               const uint64_t *offsets, uint32_t n_obj, double fmin, double df, uint32_t n_freq,
               int normalize, void *pgram, uint32_t *best_idx, void *best_power,
               uint32_t top = 1) {
    if (top != 1 && top != 3) return fail(LSGB_ERR_INVALID, "top must be 1 or 3");
    b.top = top;
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
    b.objs.assign(n_obj, ObjInfo{});
    uint32_t max_n = 0;
    for (uint32_t o = 0; o < n_obj; ++o) {
        if (offsets[o + 1] <= offsets[o])
            return fail(LSGB_ERR_INVALID, "object %u has no observations (offsets must increase)", o);
        const uint64_t n = offsets[o + 1] - offsets[o];
        if (n > 0xffffffffull) return fail(LSGB_ERR_INVALID, "object %u has more than 2^32-1 rows", o);
        b.objs[o].row0 = offsets[o];
        b.objs[o].n = (uint32_t)n;
        max_n = std::max<uint32_t>(max_n, (uint32_t)n);
    }
    b.empty = n_freq == 0;
    if (b.empty) return LSGB_OK;  // nothing to compute or write
    b.variant = variant;
    b.precision = precision;
    b.dtype = dtype;
    b.normalize = normalize;
    b.t = t;
    b.y = y;
    b.dy = dy;
    b.pgram = pgram;
    b.best_idx = best_idx;
    b.best_power = best_power;
    b.n_obj = n_obj;
    b.n_freq = n_freq;
    b.fmin = fmin;
    b.df = df;
    b.max_n = max_n;
    b.rows = offsets[n_obj];
    b.offsets.assign(offsets, offsets + n_obj + 1);
    // Work order: largest objects first (longest-processing-time first), ties by index.
    b.perm.resize(n_obj);
    std::iota(b.perm.begin(), b.perm.end(), 0u);
    std::stable_sort(b.perm.begin(), b.perm.end(),
                     [&](uint32_t x, uint32_t z) { return b.objs[x].n > b.objs[z].n; });
    const bool mixed = precision == LSGB_MIXED;
    b.shape = shapes[variant];
    b.reanchor = mixed ? reanchor : 0;
    // the re-anchoring study is compiled for the consecutive-frequency packed loop only
    if (b.reanchor) b.shape = variant == LSGB_STANDARD ? MixedShape{12, 256, 2, 1, 0}
                                                       : MixedShape{8, 256, 2, 1, 0};
    const uint32_t tile_freqs = mixed ? (uint32_t)(b.shape.f * b.shape.nt) : (uint32_t)kPlainThreads;
    const uint64_t n_tiles64 = (n_freq + (uint64_t)tile_freqs - 1) / tile_freqs;
    b.units = n_tiles64 * n_obj;
    if (b.units >= 0xffffffffull)
        return fail(LSGB_ERR_INVALID, "%llu work units exceed the 2^32 queue; split the batch",
                    (unsigned long long)b.units);
    b.n_tiles = (uint32_t)n_tiles64;
    b.want_best = best_idx || best_power;
    int occ = 0;
    if (mixed && b.shape.x2 == 3) {
        // tensor form: one persistent CTA per SM with its own shared-memory ring
        if ((uint32_t)b.shape.f * (uint32_t)b.shape.nt != tensor_tile_freqs(variant))
            return fail(LSGB_ERR_INVALID, "tensor form: shape %dx%d is not compiled", b.shape.f,
                        b.shape.nt);
        b.chunk = 0;
        b.fold = false;
        b.smem = tensor_smem_bytes(variant);
        occ = 1;
        uint64_t kb = 0;
        for (uint32_t o = 0; o < n_obj; ++o) {
            b.objs[o].kb0 = (uint32_t)kb;
            kb += (b.objs[o].n + kTensorKBlock - 1) / kTensorKBlock;
        }
        if (kb >= 0xffffffffull) return fail(LSGB_ERR_INVALID, "batch too long for the tensor form");
        b.total_kb = kb;
        b.kbobj.resize(kb);
        for (uint32_t o = 0; o < n_obj; ++o) {
            const uint32_t nkb = (b.objs[o].n + kTensorKBlock - 1) / kTensorKBlock;
            std::fill_n(b.kbobj.begin() + b.objs[o].kb0, nkb, o);
        }
        // Fewer (object, tile) pairs than SMs: cut every object's K-blocks into slices so
        // that the units fill the SMs, each slice at least kMinSliceKB K-blocks long; a
        // finishing pass adds the slices' sums (one object of 3,555 observations and 1e5
        // frequencies: 13 pairs, 11 slices)
        b.ksplit = 1;
        const uint32_t min_nkb = (b.objs[b.perm.back()].n + kTensorKBlock - 1) / kTensorKBlock;
        if (b.units < (uint64_t)sms) {
            const uint64_t by_sms = (uint64_t)sms / b.units;
            const uint64_t by_len = min_nkb / kMinSliceKB;
            b.ksplit = (uint32_t)std::max<uint64_t>(1, std::min(by_sms, by_len));
        }
        b.units *= b.ksplit;
        // The tensor kernel walks its units statically (CTA c takes units c, c + grid, ...),
        // so the order is not for load balance but for overlap: largest and smallest objects
        // alternate, so that a CTA's short units (whose power pass outlasts their MMAs) fall
        // between long ones and the TMEM slots absorb them (0.4% at 999 objects).
        std::vector<uint32_t> alt;
        alt.reserve(n_obj);
        for (size_t lo = 0, hi = n_obj; lo < hi;) {
            alt.push_back(b.perm[lo++]);
            if (lo < hi) alt.push_back(b.perm[--hi]);
        }
        b.perm.swap(alt);
    } else if (mixed) {
        // Shared memory per CTA: at most what keeps the CTAs per SM that the shape's
        // register budget allows resident (less the per-CTA reservation and the static
        // variables), and at most kMixedSmemMax of staged records.
        int dev = 0, smem_sm = 0;
        LSGB_CUDA(cudaGetDevice(&dev));
        LSGB_CUDA(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
        const size_t per_cta = (size_t)smem_sm / (size_t)std::max(1, b.shape.minb) - 1024 - 256;
        const uint32_t rec_bytes = (uint32_t)mixed_rec_bytes(b.shape);
        size_t rec_budget = std::min<size_t>(kMixedSmemMax, per_cta);
        b.chunk = (uint32_t)std::min<size_t>(max_n, rec_budget / rec_bytes);
        // objects longer than one chunk sum in two levels (chunk sums folded in smem)
        b.fold = max_n > b.chunk;
        if (b.fold) {
            const size_t fb = mixed_fold_bytes(variant, b.shape);
            rec_budget = per_cta >= fb + 64 * (size_t)rec_bytes
                             ? std::min<size_t>(kMixedSmemMax, per_cta - fb)
                             : 64 * (size_t)rec_bytes;
            b.chunk = (uint32_t)std::min<size_t>(max_n, rec_budget / rec_bytes);
        }
        b.smem = (size_t)rec_bytes * b.chunk + (b.fold ? mixed_fold_bytes(variant, b.shape) : 0);
        LSGB_CUDA(mixed_occupancy(variant, dtype, b.shape, b.smem, &occ));
        if (occ < 1) return fail(LSGB_ERR_CUDA, "mixed kernel does not fit on an SM (smem %zu)", b.smem);
    } else {
        b.chunk = std::min<uint32_t>(max_n, kPlainChunkMax);
        b.smem = sizeof(double) * b.chunk * (variant == LSGB_GENERALIZED ? 3 : 2);
        LSGB_CUDA(plain_occupancy(variant, dtype, dtype, b.smem, &occ));
        if (occ < 1) return fail(LSGB_ERR_CUDA, "plain kernel does not fit on an SM (smem %zu)", b.smem);
    }
    b.grid = (int)std::min<uint64_t>((uint64_t)sms * occ, b.units);
    return LSGB_OK;
}

// Sizes the workspace and copies the per-object tables (stream-ordered).
int upload_tables(const Batch &b, Workspace &ws, cudaStream_t st) {
    const bool mixed = b.precision == LSGB_MIXED;
    LSGB_CUDA(ws.objs.ensure(sizeof(ObjInfo) * b.n_obj));
    LSGB_CUDA(ws.offs.ensure(sizeof(uint64_t) * (b.n_obj + 1)));
    LSGB_CUDA(ws.perm.ensure(sizeof(uint32_t) * b.n_obj));
    LSGB_CUDA(ws.counter.ensure(sizeof(uint32_t)));
    if (b.want_best && !mixed) LSGB_CUDA(ws.tile_best.ensure(sizeof(TileBest) * b.units * b.top));
    if (b.want_best && mixed)
        LSGB_CUDA(ws.keys.ensure(sizeof(unsigned long long) * b.n_obj * b.top));
    if (mixed) LSGB_CUDA(ws.rec.ensure(mixed_global_rec_bytes(b.shape) * b.rows));
    if (mixed && b.shape.x2 == 3) LSGB_CUDA(ws.optab.ensure(tensor_optab_bytes(b.variant, b.total_kb)));
    if (mixed && b.shape.x2 == 3 && b.ksplit > 1)
        LSGB_CUDA(ws.partial.ensure(tensor_partial_bytes(b.variant) * b.units));
    if (mixed && b.shape.x2 == 3 && b.ksplit <= 1 && b.top == 3 && b.want_best)
        LSGB_CUDA(ws.key3.ensure(tensor_tile_key3_bytes((uint64_t)b.n_obj * b.n_tiles)));
    if (!ws.status.p) {
        LSGB_CUDA(ws.status.ensure(sizeof(uint32_t)));
        LSGB_CUDA(cudaMemsetAsync(ws.status.p, 0, sizeof(uint32_t), st));
    }
    LSGB_CUDA(cudaMemcpyAsync(ws.objs.p, b.objs.data(), sizeof(ObjInfo) * b.n_obj,
                              cudaMemcpyHostToDevice, st));
    LSGB_CUDA(cudaMemcpyAsync(ws.offs.p, b.offsets.data(), sizeof(uint64_t) * (b.n_obj + 1),
                              cudaMemcpyHostToDevice, st));
    LSGB_CUDA(cudaMemcpyAsync(ws.perm.p, b.perm.data(), sizeof(uint32_t) * b.n_obj,
                              cudaMemcpyHostToDevice, st));
    if (mixed && b.shape.x2 == 3 && b.total_kb) {
        LSGB_CUDA(ws.kbobj.ensure(sizeof(uint32_t) * b.total_kb));
        LSGB_CUDA(cudaMemcpyAsync(ws.kbobj.p, b.kbobj.data(), sizeof(uint32_t) * b.total_kb,
                                  cudaMemcpyHostToDevice, st));
    }
    return LSGB_OK;
}

// The status a status word stands for (0: none).
int status_code(uint32_t v) {
    if (v & kStatusBadInput)
        return fail(LSGB_ERR_INVALID,
                    "invalid input: a non-finite time or magnitude, or (generalized variant) a "
                    "non-finite or non-positive dmag; the results of the call are invalid");
    if (v & kStatusTimeout)
        return fail(LSGB_ERR_CUDA,
                    "tensor-form kernel: a pipeline wait timed out; the results of the call are invalid");
    return LSGB_OK;
}

// Reports (and clears) what the call's kernels recorded in the status word. Call after the
// work that may have set it has completed.
int check_status(Workspace &ws) {
    if (!ws.status.p) return LSGB_OK;
    uint32_t v = 0;
    LSGB_CUDA(cudaMemcpy(&v, ws.status.p, sizeof(v), cudaMemcpyDeviceToHost));
    if (v == 0) return LSGB_OK;
    LSGB_CUDA(cudaMemset(ws.status.p, 0, sizeof(uint32_t)));
    return status_code(v);
}

// Queues on st a copy of the status word to host memory and then its reset, so that the
// caller learns, once st has reached this point, what the work before it recorded.
int status_async(Workspace &ws, uint32_t *host, cudaStream_t st) {
    if (!host) return fail(LSGB_ERR_INVALID, "status destination is NULL");
    if (!ws.status.p) {
        *host = 0;
        return LSGB_OK;
    }
    LSGB_CUDA(cudaMemcpyAsync(host, ws.status.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    LSGB_CUDA(cudaMemsetAsync(ws.status.p, 0, sizeof(uint32_t), st));
    return LSGB_OK;
}

// Records `ev` on `st`; while `st` is being captured the record becomes an event node
// of the graph (a plain record there would only mark a capture dependency).
cudaError_t record(cudaEvent_t ev, cudaStream_t st, bool capturing) {
    return capturing ? cudaEventRecordWithFlags(ev, st, cudaEventRecordExternal)
                     : cudaEventRecord(ev, st);
}

// The device work of a batch: memsets and kernels only, so it can be captured in a graph.
// ev0/ev1 (may be null) are recorded around the main kernel.
int enqueue_batch(Batch &b, Workspace &ws, cudaStream_t st, cudaEvent_t ev0, cudaEvent_t ev1,
                  bool capturing = false) {
    const bool mixed = b.precision == LSGB_MIXED;
    ObjInfo *d_objs = (ObjInfo *)ws.objs.p;
    uint32_t kernels = 0;
    // the statistics kernel also zeroes the queue counter and the best keys
    LSGB_CUDA(launch_stats(b.variant, mixed ? 1 : 0, b.dtype, b.normalize, b.t, b.y, b.dy, d_objs,
                           b.n_obj, (uint32_t *)ws.status.p, st,
                           b.want_best && mixed ? (unsigned long long *)ws.keys.p : nullptr, b.top,
                           (uint32_t *)ws.counter.p));
    ++kernels;
    if (mixed) {
        GridTurns g;
        two_prod(b.fmin, kInv2PiHi, kInv2PiLo, g.f0_hi, g.f0_lo);
        two_prod(b.df, kInv2PiHi, kInv2PiLo, g.df_hi, g.df_lo);
        LSGB_CUDA(launch_records(b.variant, b.dtype, b.t, b.y, b.dy, (const uint64_t *)ws.offs.p,
                                 b.n_obj, d_objs, b.rows, g, ws.rec.p,
                                 b.shape.x2 == 2 ? (uint32_t)b.shape.nt : 0u, st,
                                 /*rotation=*/b.shape.x2 != 3));
        ++kernels;
        MixedArgs a{};
        a.rec = ws.rec.p;
        a.steps = ws.optab.p;
        a.total_kb = (uint32_t)b.total_kb;
        a.optab = (const unsigned char *)ws.optab.p + b.total_kb * tensor_step_bytes(b.variant);
        a.objs = d_objs;
        a.perm = (const uint32_t *)ws.perm.p;
        a.n_obj = b.n_obj;
        a.n_tiles = b.n_tiles;
        a.n_freq = b.n_freq;
        a.chunk = b.chunk;
        a.counter = (uint32_t *)ws.counter.p;
        a.pgram = b.pgram;
        a.tile_best = nullptr;
        a.best_key = b.want_best ? (unsigned long long *)ws.keys.p : nullptr;
        a.reanchor = b.reanchor;
        a.fold = b.fold ? 1u : 0u;
        a.status = (uint32_t *)ws.status.p;
        a.top = b.top;
        a.wait_cycles = b.wait_cycles;
        a.ksplit = b.ksplit;
        a.kb_obj = (const uint32_t *)ws.kbobj.p;
        a.tile_key3 = (unsigned long long *)ws.key3.p;
        a.partial = b.ksplit > 1 ? (float *)ws.partial.p : nullptr;
        if (b.shape.x2 == 3) {
            LSGB_CUDA(launch_tensor_optab(b.variant, a, b.total_kb, st));
            ++kernels;
        }
        if (ev0) LSGB_CUDA(record(ev0, st, capturing));
        LSGB_CUDA(launch_mixed(b.variant, b.dtype, b.shape, a, b.grid, b.smem, st));
        if (ev1) LSGB_CUDA(record(ev1, st, capturing));
        ++kernels;
    } else {
        PlainArgs a{};
        a.t = b.t;
        a.y = b.y;
        a.dy = b.dy;
        a.objs = d_objs;
        a.perm = (const uint32_t *)ws.perm.p;
        a.n_obj = b.n_obj;
        a.n_tiles = b.n_tiles;
        a.n_freq = b.n_freq;
        a.chunk = b.chunk;
        a.fmin = b.fmin;
        a.df = b.df;
        a.counter = (uint32_t *)ws.counter.p;
        a.pgram = b.pgram;
        a.tile_best = b.want_best ? (TileBest *)ws.tile_best.p : nullptr;
        a.top = b.top;
        if (ev0) LSGB_CUDA(record(ev0, st, capturing));
        LSGB_CUDA(launch_plain(b.variant, b.dtype, b.dtype, a, b.grid, b.smem, st));
        if (ev1) LSGB_CUDA(record(ev1, st, capturing));
        ++kernels;
    }
    if (b.want_best && mixed) {
        LSGB_CUDA(launch_key_decode(b.dtype, (const unsigned long long *)ws.keys.p,
                                    b.n_obj * b.top, b.best_idx, b.best_power, st));
        ++kernels;
    } else if (b.want_best) {
        LSGB_CUDA(launch_best_reduce(b.dtype, (const TileBest *)ws.tile_best.p, b.n_obj, b.n_tiles,
                                     b.top, b.best_idx, b.best_power, st));
        ++kernels;
    }
    b.kernels = kernels;
    return LSGB_OK;
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
    cudaStream_t d2h = nullptr;     // host-buffer API: periodogram copies overlapping compute
    Workspace ws;
    DevBuf in_t, in_y, in_dy, out_pg, out_idx, out_p;
    // defaults measured fastest on the 999-object, 1e6-frequency batches: the tensor-core
    // form (lsgb_tensor.cu) for both variants
    MixedShape shape[2] = {{64, 128, 1, 3, 0}, {32, 128, 1, 3, 0}};
    uint32_t last_kernels = 0;
    uint64_t last_units = 0;
    cudaEvent_t ev_main0 = nullptr, ev_main1 = nullptr;  // around the last main-kernel launch
    bool ev_valid = false;
    uint32_t reanchor = 0;  // mixed form: 0 = anchor at each thread's frequency run
    long long wait_cycles = 0;  // lsgb_set_wait_limit
    uint32_t *h_status = nullptr;  // pinned: the status word, copied back with a call's results
};

// Ends a host-buffer call whose results are queued for copy on st: the status word is
// copied back on the same stream, so one synchronization brings both (a separate
// synchronous read would cost another round trip); then it is reported and cleared.
static int finish_host_call(lsgb_engine *eng, cudaStream_t st) {
    if (!eng->ws.status.p) {
        LSGB_CUDA(cudaStreamSynchronize(st));
        return LSGB_OK;
    }
    LSGB_CUDA(cudaMemcpyAsync(eng->h_status, eng->ws.status.p, sizeof(uint32_t),
                              cudaMemcpyDeviceToHost, st));
    LSGB_CUDA(cudaStreamSynchronize(st));
    const uint32_t v = *eng->h_status;
    if (v == 0) return LSGB_OK;
    LSGB_CUDA(cudaMemset(eng->ws.status.p, 0, sizeof(uint32_t)));
    return status_code(v);
}

// A batch whose device work is captured once in a CUDA graph and replayed.
struct lsgb_plan {
    int device = 0;
    Workspace ws;
    Batch b;
    cudaStream_t cap = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    bool launched = false;
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
    if (e2 == cudaSuccess) e2 = cudaStreamCreateWithFlags(&eng->d2h, cudaStreamNonBlocking);
    if (e2 == cudaSuccess) e2 = cudaEventCreate(&eng->ev_main0);
    if (e2 == cudaSuccess) e2 = cudaEventCreate(&eng->ev_main1);
    if (e2 == cudaSuccess) e2 = cudaHostAlloc((void **)&eng->h_status, sizeof(uint32_t), 0);
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
    eng->ws.release();
    DevBuf *bufs[] = {&eng->in_t, &eng->in_y, &eng->in_dy, &eng->out_pg, &eng->out_idx, &eng->out_p};
    for (DevBuf *b : bufs) b->release();
    if (eng->stream) cudaStreamDestroy(eng->stream);
    if (eng->d2h) cudaStreamDestroy(eng->d2h);
    if (eng->ev_main0) cudaEventDestroy(eng->ev_main0);
    if (eng->ev_main1) cudaEventDestroy(eng->ev_main1);
    if (eng->h_status) cudaFreeHost(eng->h_status);
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
    if (x2 >= 0) s.x2 = x2 > 3 ? -1 : x2;  // -1 matches no compiled shape
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
    return check_status(eng->ws);
}

// The device-buffer call with `top` (1 or 3) best frequencies per object: best_idx and
// best_power hold [n_obj x top] entries, best first.
static int periodogram_device(lsgb_engine *eng, int variant, int precision, int dtype,
                              const void *t, const void *y, const void *dy,
                              const uint64_t *offsets, uint32_t n_obj, double fmin, double df,
                              uint32_t n_freq, int normalize, void *pgram, uint32_t *best_idx,
                              void *best_power, void *stream_, uint32_t top) {
    if (!eng) return fail(LSGB_ERR_INVALID, "engine is NULL");
    eng->last_kernels = 0;
    eng->last_units = 0;
    cudaStream_t st = (cudaStream_t)stream_;
    LSGB_CUDA(cudaSetDevice(eng->device));
    Batch b;
    int rc = plan_batch(b, eng->sms, eng->shape, eng->reanchor, variant, precision, dtype, t, y, dy,
                        offsets, n_obj, fmin, df, n_freq, normalize, pgram, best_idx, best_power,
                        top);
    if (rc != LSGB_OK || b.empty) return rc;
    b.wait_cycles = eng->wait_cycles;
    rc = upload_tables(b, eng->ws, st);
    if (rc != LSGB_OK) return rc;
    rc = enqueue_batch(b, eng->ws, st, eng->ev_main0, eng->ev_main1);
    if (rc != LSGB_OK) return rc;
    eng->ev_valid = true;
    eng->last_kernels = b.kernels;
    eng->last_units = b.units;
    return LSGB_OK;
}

LSGB_API int lsgb_periodogram_device(lsgb_engine *eng, int variant, int precision, int dtype,
                                     const void *t, const void *y, const void *dy,
                                     const uint64_t *offsets, uint32_t n_obj, double fmin,
                                     double df, uint32_t n_freq, int normalize, void *pgram,
                                     uint32_t *best_idx, void *best_power, void *stream) {
    return periodogram_device(eng, variant, precision, dtype, t, y, dy, offsets, n_obj, fmin, df,
                              n_freq, normalize, pgram, best_idx, best_power, stream, 1u);
}

LSGB_API int lsgb_periodogram_top3_device(lsgb_engine *eng, int variant, int precision, int dtype,
                                          const void *t, const void *y, const void *dy,
                                          const uint64_t *offsets, uint32_t n_obj, double fmin,
                                          double df, uint32_t n_freq, int normalize, void *pgram,
                                          uint32_t *top_idx, void *top_power, void *stream) {
    return periodogram_device(eng, variant, precision, dtype, t, y, dy, offsets, n_obj, fmin, df,
                              n_freq, normalize, pgram, top_idx, top_power, stream, 3u);
}

LSGB_API void lsgb_plan_destroy(lsgb_plan *p) {
    if (!p) return;
    cudaSetDevice(p->device);
    if (p->cap) cudaStreamSynchronize(p->cap);
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    if (p->ev0) cudaEventDestroy(p->ev0);
    if (p->ev1) cudaEventDestroy(p->ev1);
    if (p->cap) cudaStreamDestroy(p->cap);
    p->ws.release();
    delete p;
}

LSGB_API int lsgb_plan_create(lsgb_engine *eng, int variant, int precision, int dtype,
                              const void *t, const void *y, const void *dy,
                              const uint64_t *offsets, uint32_t n_obj, double fmin, double df,
                              uint32_t n_freq, int normalize, void *pgram, uint32_t *best_idx,
                              void *best_power, lsgb_plan **out) {
    if (!eng || !out) return fail(LSGB_ERR_INVALID, "lsgb_plan_create: NULL engine or out");
    *out = nullptr;
    if (n_freq == 0) return fail(LSGB_ERR_INVALID, "lsgb_plan_create: n_freq is 0");
    LSGB_CUDA(cudaSetDevice(eng->device));
    lsgb_plan *p = new lsgb_plan();
    p->device = eng->device;
    int rc = plan_batch(p->b, eng->sms, eng->shape, eng->reanchor, variant, precision, dtype, t, y,
                        dy, offsets, n_obj, fmin, df, n_freq, normalize, pgram, best_idx,
                        best_power);
    cudaError_t e = cudaSuccess;
    p->b.wait_cycles = eng->wait_cycles;
    if (rc == LSGB_OK) {
        e = cudaStreamCreateWithFlags(&p->cap, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreate(&p->ev0);
        if (e == cudaSuccess) e = cudaEventCreate(&p->ev1);
        if (e != cudaSuccess) rc = fail(LSGB_ERR_CUDA, "plan set-up: %s", cudaGetErrorString(e));
    }
    if (rc == LSGB_OK) rc = upload_tables(p->b, p->ws, p->cap);
    if (rc == LSGB_OK && (e = cudaStreamSynchronize(p->cap)) != cudaSuccess)
        rc = fail(LSGB_ERR_CUDA, "plan upload: %s", cudaGetErrorString(e));
    if (rc == LSGB_OK) {
        // relaxed: the launch helpers set kernel attributes (not stream work) while capturing
        e = cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeRelaxed);
        if (e != cudaSuccess) rc = fail(LSGB_ERR_CUDA, "begin capture: %s", cudaGetErrorString(e));
        if (rc == LSGB_OK) {
            const int rc2 = enqueue_batch(p->b, p->ws, p->cap, p->ev0, p->ev1, true);
            e = cudaStreamEndCapture(p->cap, &p->graph);
            if (rc2 != LSGB_OK) rc = rc2;
            else if (e != cudaSuccess)
                rc = fail(LSGB_ERR_CUDA, "end capture: %s", cudaGetErrorString(e));
        }
    }
    if (rc == LSGB_OK && (e = cudaGraphInstantiate(&p->exec, p->graph, 0)) != cudaSuccess)
        rc = fail(LSGB_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
    if (rc != LSGB_OK) {
        lsgb_plan_destroy(p);
        return rc;
    }
    *out = p;
    return LSGB_OK;
}

LSGB_API int lsgb_plan_launch(lsgb_plan *p, void *stream) {
    if (!p) return fail(LSGB_ERR_INVALID, "lsgb_plan_launch: plan is NULL");
    LSGB_CUDA(cudaSetDevice(p->device));
    LSGB_CUDA(cudaGraphLaunch(p->exec, (cudaStream_t)stream));
    p->launched = true;
    return LSGB_OK;
}

LSGB_API int lsgb_plan_info(lsgb_plan *p, uint32_t *kernels, uint64_t *units, float *last_kernel_ms) {
    if (!p) return fail(LSGB_ERR_INVALID, "lsgb_plan_info: plan is NULL");
    if (kernels) *kernels = p->b.kernels;
    if (units) *units = p->b.units;
    if (last_kernel_ms) {
        if (!p->launched) return fail(LSGB_ERR_INVALID, "lsgb_plan_info: plan never launched");
        LSGB_CUDA(cudaEventSynchronize(p->ev1));
        LSGB_CUDA(cudaEventElapsedTime(last_kernel_ms, p->ev0, p->ev1));
        return check_status(p->ws);  // set by kernels that ran before ev1
    }
    return LSGB_OK;
}

LSGB_API int lsgb_plan_status_async(lsgb_plan *p, uint32_t *host_status, void *stream) {
    if (!p) return fail(LSGB_ERR_INVALID, "lsgb_plan_status_async: plan is NULL");
    LSGB_CUDA(cudaSetDevice(p->device));
    return status_async(p->ws, host_status, (cudaStream_t)stream);
}

LSGB_API int lsgb_status_async(lsgb_engine *eng, uint32_t *host_status, void *stream) {
    if (!eng) return fail(LSGB_ERR_INVALID, "lsgb_status_async: engine is NULL");
    LSGB_CUDA(cudaSetDevice(eng->device));
    return status_async(eng->ws, host_status, (cudaStream_t)stream);
}

LSGB_API int lsgb_set_wait_limit(lsgb_engine *eng, uint64_t cycles) {
    if (!eng) return fail(LSGB_ERR_INVALID, "lsgb_set_wait_limit: engine is NULL");
    if (cycles > (1ull << 40)) return fail(LSGB_ERR_INVALID, "lsgb_set_wait_limit: above 2^40 cycles");
    eng->wait_cycles = (long long)cycles;
    return LSGB_OK;
}

// The host-buffer call with `top` (1 or 3) best frequencies per object.
static int periodogram_host(lsgb_engine *eng, int variant, int precision, int dtype,
                            const void *t, const void *y, const void *dy, const uint64_t *offsets,
                            uint32_t n_obj, double fmin, double df, uint32_t n_freq, int normalize,
                            void *pgram, uint32_t *best_idx, void *best_power, uint32_t top) {
    if (!eng) return fail(LSGB_ERR_INVALID, "engine is NULL");
    if (top != 1 && top != 3) return fail(LSGB_ERR_INVALID, "top must be 1 or 3");
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
        LSGB_CUDA(eng->out_idx.ensure(sizeof(uint32_t) * n_obj * top));
        d_idx = (uint32_t *)eng->out_idx.p;
    }
    if (best_power) {
        LSGB_CUDA(eng->out_p.ensure(es * n_obj * top));
        d_p = eng->out_p.p;
    }
    // A large periodogram goes out in object chunks: every chunk's computation is queued
    // first, then each chunk is copied to the host on a second stream as soon as it is
    // done, so the copy of chunk c overlaps the computation of chunks c+1.. (the result
    // of an object does not depend on the batch it is computed in, unless a batch has fewer
    // (object, tile) pairs than SMs: the tensor form then sums K slices, in another order,
    // within the mixed form's tolerance).
    const size_t kChunkBytes = size_t(512) << 20;
    const uint32_t n_chunks =
        (d_pg && n_freq && es * pg_elems > kChunkBytes && n_obj >= 2)
            ? (uint32_t)std::min<uint64_t>({8ull, n_obj, (es * pg_elems + kChunkBytes - 1) / kChunkBytes})
            : 1u;
    if (n_chunks > 1) {
        std::vector<uint32_t> cut{0};
        for (uint32_t c = 1; c < n_chunks; ++c) {  // equal rows per chunk, at object boundaries
            const uint64_t target = rows * c / n_chunks;
            uint32_t o = (uint32_t)(std::lower_bound(offsets, offsets + n_obj + 1, target) - offsets);
            o = std::max<uint32_t>(o, cut.back() + 1);
            if (o < n_obj) cut.push_back(o);
        }
        cut.push_back(n_obj);
        // size the workspace for the whole batch up front: growing it between chunks would
        // free memory still in use by queued kernels (cudaFree synchronizes the device)
        {
            const uint64_t max_tiles = (n_freq + 255) / 256;  // the smallest tile of any form
            LSGB_CUDA(eng->ws.objs.ensure(sizeof(ObjInfo) * n_obj));
            LSGB_CUDA(eng->ws.offs.ensure(sizeof(uint64_t) * (n_obj + 1)));
            LSGB_CUDA(eng->ws.perm.ensure(sizeof(uint32_t) * n_obj));
            LSGB_CUDA(eng->ws.counter.ensure(sizeof(uint32_t)));
            LSGB_CUDA(eng->ws.keys.ensure(sizeof(unsigned long long) * n_obj * top));
            if (precision == LSGB_MIXED)
                LSGB_CUDA(eng->ws.rec.ensure(mixed_global_rec_bytes(eng->shape[variant]) * rows));
            if (precision == LSGB_MIXED && eng->shape[variant].x2 == 3) {
                const uint64_t kb = rows / kTensorKBlock + n_obj;  // K-blocks, at most
                LSGB_CUDA(eng->ws.optab.ensure(tensor_optab_bytes(variant, kb)));
                LSGB_CUDA(eng->ws.kbobj.ensure(sizeof(uint32_t) * kb));
                LSGB_CUDA(eng->ws.partial.ensure(tensor_partial_bytes(variant) * (size_t)eng->sms));
                if (top == 3 && (best_idx || best_power))
                    LSGB_CUDA(eng->ws.key3.ensure(tensor_tile_key3_bytes(
                        (uint64_t)n_obj * ((n_freq + tensor_tile_freqs(variant) - 1) /
                                           tensor_tile_freqs(variant)))));
            } else if (best_idx || best_power)
                LSGB_CUDA(eng->ws.tile_best.ensure(sizeof(TileBest) * max_tiles * n_obj * top));
        }
        std::vector<cudaEvent_t> ev(cut.size() - 1, nullptr);
        int rc = LSGB_OK;
        for (size_t c = 0; c + 1 < cut.size() && rc == LSGB_OK; ++c) {
            const uint32_t o0 = cut[c], o1 = cut[c + 1];
            const uint64_t r0 = offsets[o0];
            std::vector<uint64_t> offs_c(offsets + o0, offsets + o1 + 1);
            for (auto &v : offs_c) v -= r0;
            rc = periodogram_device(
                eng, variant, precision, dtype, (const char *)eng->in_t.p + es * r0,
                (const char *)eng->in_y.p + es * r0, d_dy ? (const char *)d_dy + es * r0 : nullptr,
                offs_c.data(), o1 - o0, fmin, df, n_freq, normalize,
                (char *)d_pg + es * (uint64_t)o0 * n_freq, d_idx ? d_idx + (uint64_t)o0 * top : nullptr,
                d_p ? (char *)d_p + es * o0 * top : nullptr, (void *)st, top);
            if (rc == LSGB_OK) {
                cudaError_t e = cudaEventCreateWithFlags(&ev[c], cudaEventDisableTiming);
                if (e == cudaSuccess) e = cudaEventRecord(ev[c], st);
                if (e != cudaSuccess) rc = fail(LSGB_ERR_CUDA, "chunk event: %s", cudaGetErrorString(e));
            }
        }
        for (size_t c = 0; c + 1 < cut.size() && rc == LSGB_OK; ++c) {
            const uint64_t off = es * (uint64_t)cut[c] * n_freq;
            const uint64_t bytes = es * (uint64_t)(cut[c + 1] - cut[c]) * n_freq;
            cudaError_t e = cudaStreamWaitEvent(eng->d2h, ev[c], 0);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync((char *)pgram + off, (const char *)d_pg + off, bytes,
                                    cudaMemcpyDeviceToHost, eng->d2h);
            if (e != cudaSuccess) rc = fail(LSGB_ERR_CUDA, "periodogram copy: %s", cudaGetErrorString(e));
        }
        cudaStreamSynchronize(st);
        cudaStreamSynchronize(eng->d2h);
        for (cudaEvent_t x : ev)
            if (x) cudaEventDestroy(x);
        if (rc != LSGB_OK) return rc;
        if (d_idx)
            LSGB_CUDA(cudaMemcpyAsync(best_idx, d_idx, sizeof(uint32_t) * n_obj * top,
                                      cudaMemcpyDeviceToHost, st));
        if (d_p)
            LSGB_CUDA(cudaMemcpyAsync(best_power, d_p, es * n_obj * top, cudaMemcpyDeviceToHost, st));
        return finish_host_call(eng, st);
    }
    int rc = periodogram_device(eng, variant, precision, dtype, eng->in_t.p, eng->in_y.p, d_dy,
                                offsets, n_obj, fmin, df, n_freq, normalize, d_pg, d_idx, d_p,
                                (void *)st, top);
    if (rc != LSGB_OK) {
        cudaStreamSynchronize(st);
        return rc;
    }
    if (n_freq == 0) {
        // nothing computed: report index 0 / power 0 as the reference's argmax would
        if (best_idx) memset(best_idx, 0, sizeof(uint32_t) * n_obj * top);
        if (best_power) memset(best_power, 0, es * n_obj * top);
        LSGB_CUDA(cudaStreamSynchronize(st));
        return LSGB_OK;
    }
    if (d_pg) LSGB_CUDA(cudaMemcpyAsync(pgram, d_pg, es * pg_elems, cudaMemcpyDeviceToHost, st));
    if (d_idx)
        LSGB_CUDA(cudaMemcpyAsync(best_idx, d_idx, sizeof(uint32_t) * n_obj * top,
                                  cudaMemcpyDeviceToHost, st));
    if (d_p) LSGB_CUDA(cudaMemcpyAsync(best_power, d_p, es * n_obj * top, cudaMemcpyDeviceToHost, st));
    return finish_host_call(eng, st);
}

LSGB_API int lsgb_periodogram_host(lsgb_engine *eng, int variant, int precision, int dtype,
                                   const void *t, const void *y, const void *dy,
                                   const uint64_t *offsets, uint32_t n_obj, double fmin, double df,
                                   uint32_t n_freq, int normalize, void *pgram, uint32_t *best_idx,
                                   void *best_power) {
    return periodogram_host(eng, variant, precision, dtype, t, y, dy, offsets, n_obj, fmin, df,
                            n_freq, normalize, pgram, best_idx, best_power, 1u);
}

LSGB_API int lsgb_periodogram_top3_host(lsgb_engine *eng, int variant, int precision, int dtype,
                                        const void *t, const void *y, const void *dy,
                                        const uint64_t *offsets, uint32_t n_obj, double fmin,
                                        double df, uint32_t n_freq, int normalize, void *pgram,
                                        uint32_t *top_idx, void *top_power) {
    return periodogram_host(eng, variant, precision, dtype, t, y, dy, offsets, n_obj, fmin, df,
                            n_freq, normalize, pgram, top_idx, top_power, 3u);
}

}  // extern "C"
