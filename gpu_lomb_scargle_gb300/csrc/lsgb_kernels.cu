// lsgb_kernels.cu -- sm_103a kernels of the Lomb-Scargle engine.
//
// The hot path of the reference is the (object, frequency) double loop of
// source/kernel.cu:484-631 (lombscargleBatch, standard L-S) and :368-477
// (lombscargleBatchError, generalized L-S), plus their single-object forms
// (:76-361). Here one persistent kernel per form walks a work queue of
// (object, frequency tile) units, largest objects first, stages the object's
// observations in shared memory, and fuses the power, the optional periodogram
// store and the per-tile argmax into the same pass.
//
// Two precision forms:
//  * plain FP64 (drop-in): sincos(omega_k * t_j) in FP64 for every pair and the
//    reference's tau / power formulas in FP64 (with FP64 atan2; the reference's
//    GPU double build silently uses FP32 atan2f, source/kernel.cu:228/:563, because
//    `#if DTYPE==float` compares two undefined identifiers);
//  * mixed: the phase of every (observation, frequency-run start) comes exactly
//    from a 64-bit fixed-point anchor (a + k*b mod 2^64 turns), its sine/cosine from
//    the SFU, and the next F-1 frequencies of the run by an FP32 angle-addition
//    recurrence (rotation by the observation's per-step cos/sin). tau never needs an
//    arctangent: the power is a closed rational function of the sums and
//    r = hypot(CC-SS, 2CS) (the tau-rotated formula of source/main.cu:1588-1598
//    expanded with the double-angle identities).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "lsgb_device.h"
#include "lsgb_internal.h"

namespace lsgb {

namespace {

constexpr double kTwoPiOver2p64 = 3.4061215800865545e-19;  // 2 pi / 2^64
constexpr double k2p64 = 18446744073709551616.0;

template <typename T>
__device__ __forceinline__ double ld_as_double(const void *p, uint64_t i) {
    return (double)__ldg(reinterpret_cast<const T *>(p) + i);
}

__device__ __forceinline__ double load_in(int dtype, const void *p, uint64_t i) {
    return dtype == 0 ? ld_as_double<float>(p, i) : ld_as_double<double>(p, i);
}

// Block-wide sum of doubles (blockDim.x a multiple of 32, <= 1024).
__device__ double block_sum(double v, double *s_red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) s_red[w] = v;
    __syncthreads();
    double r = 0.0;
    if (w == 0) {
        r = (l < (int)(blockDim.x >> 5)) ? s_red[l] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
        if (l == 0) s_red[0] = r;
    }
    __syncthreads();
    r = s_red[0];
    __syncthreads();
    return r;
}

// frac(x * t) as a 64-bit fixed-point fraction of a turn, x = x_hi + x_lo
// (double-double). Error below 2^-60 turns for |x t| < 2^40.
__device__ __forceinline__ uint64_t frac_turns_u64(double x_hi, double x_lo, double t) {
    const double p_hi = x_hi * t;
    const double p_lo = fma(x_hi, t, -p_hi) + x_lo * t;
    const double r_hi = p_hi - floor(p_hi);  // exact, in [0, 1)
    const uint64_t u = __double2ull_rz(r_hi * k2p64);
    const long long e = __double2ll_rn(p_lo * k2p64);
    return u + (uint64_t)e;
}

template <int NT, typename V>
__device__ __forceinline__ void block_best(V &bp, uint32_t &bk, V *s_p, uint32_t *s_k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const V op = __shfl_xor_sync(0xffffffffu, bp, o);
        const uint32_t ok = __shfl_xor_sync(0xffffffffu, bk, o);
        if (better(op, ok, bp, bk)) { bp = op; bk = ok; }
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) { s_p[w] = bp; s_k[w] = bk; }
    __syncthreads();
    if (w == 0) {
        bp = l < NT / 32 ? s_p[l] : V(0);
        bk = l < NT / 32 ? s_k[l] : 0xffffffffu;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const V op = __shfl_xor_sync(0xffffffffu, bp, o);
            const uint32_t ok = __shfl_xor_sync(0xffffffffu, bk, o);
            if (better(op, ok, bp, bk)) { bp = op; bk = ok; }
        }
    }
}

// ---------------------------------------------------------------------------
// Per-object statistics (FP64). One CTA per object.
//  standard: norm = 2 / (N * sigma^2), sigma^2 the population variance of y
//            (source/main.cu:1295-1317, :1335), or 1 without normalization.
//  generalized (mixed form only): weighted mean of y with w = 1/dy^2 and the
//            quantities the mixed kernel needs to undo the float rounding of
//            the stored weights.
// ---------------------------------------------------------------------------
// Block-wide maximum of non-negative doubles (blockDim.x a multiple of 32, <= 1024).
__device__ double block_max(double v, double *s_red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) s_red[w] = v;
    __syncthreads();
    double r = 0.0;
    if (w == 0) {
        r = (l < (int)(blockDim.x >> 5)) ? s_red[l] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r = fmax(r, __shfl_xor_sync(0xffffffffu, r, o));
        if (l == 0) s_red[0] = r;
    }
    __syncthreads();
    return s_red[0];
}

// The power of two 2^-e with m / 2^e in (1/2, 1] (1 for m == 0).
__device__ float pow2_scale(double m) {
    if (!(m > 0.0) || !isfinite(m)) return 1.0f;
    int e;
    frexp(m, &e);  // m = f 2^e, f in [1/2, 1)
    return (float)ldexp(1.0, -e);
}

__global__ void stats_kernel(int variant, int mixed, int dtype, int normalize, const void *t,
                             const void *y, const void *dy, ObjInfo *objs, uint32_t *status,
                             unsigned long long *keys, uint32_t top, uint32_t *counter) {
    __shared__ double s_red[32];
    if (keys && threadIdx.x < top) keys[(uint64_t)blockIdx.x * top + threadIdx.x] = 0ull;
    if (counter && blockIdx.x == 0 && threadIdx.x == 0) *counter = 0u;
    ObjInfo &ob = objs[blockIdx.x];
    const uint64_t r0 = ob.row0;
    const uint32_t n = ob.n;
    // Inputs the algorithm has no answer for: a non-finite time or magnitude, and for the
    // generalized variant a non-finite or non-positive dmag (weight 1/dmag^2). The
    // reference computes NaN or infinite powers from them; here the call reports them
    // (status bit 1, kStatusBadInput) and its results for that object mean nothing.
    // The loops below are unrolled so that a thread's loads are in flight together (one
    // object is one CTA, so its passes are latency-bound); each thread still accumulates its
    // rows i = tid, tid + blockDim, ... in order, so the sums do not change.
    if (variant == 0) {
        // pass 1: the input check, the sum and (mixed form) the largest |y| as a float
        bool bad = false;
        double s = 0.0, ym = 0.0;
#pragma unroll 4
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
            const double yi = load_in(dtype, y, r0 + i);
            if (status) bad |= !isfinite(load_in(dtype, t, r0 + i)) || !isfinite(yi);
            s += yi;
            ym = fmax(ym, fabs((double)(float)yi));
        }
        if (status && __syncthreads_or(bad) && threadIdx.x == 0) atomicOr(status, kStatusBadInput);
        const double mean = block_sum(s, s_red) / (n * 1.0);
        ym = mixed ? block_max(ym, s_red) : 0.0;
        // pass 2: the centred sum of squares
        double s2 = 0.0;
#pragma unroll 4
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
            const double d = load_in(dtype, y, r0 + i) - mean;
            s2 += d * d;
        }
        s2 = block_sum(s2, s_red);
        if (threadIdx.x == 0) {
            const double sigma = sqrt(s2 / (n * 1.0));
            ob.norm = normalize ? 2.0 / (n * (sigma * sigma)) : 1.0;
            ob.norm32 = (float)ob.norm;
            ob.tsc0 = pow2_scale(ym);
            ob.tsc1 = 1.0f;
        }
        return;
    }
    // generalized: pass 1, the input check and (mixed form) the weight sums
    bool bad = false;
    double w_s = 0.0, wy_s = 0.0;
#pragma unroll 4
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const double e = load_in(dtype, dy, r0 + i), yi = load_in(dtype, y, r0 + i);
        if (status)
            bad |= !isfinite(load_in(dtype, t, r0 + i)) || !isfinite(yi) || !(isfinite(e) && e > 0.0);
        if (mixed) {
            double w = 1.0 / e;
            w = w * w;
            w_s += w;
            wy_s += w * yi;
        }
    }
    if (status && __syncthreads_or(bad) && threadIdx.x == 0) atomicOr(status, kStatusBadInput);
    if (!mixed) {
        if (threadIdx.x == 0) {
            ob.norm = 1.0;
            ob.norm32 = 1.0f;
        }
        return;
    }
    const double W = block_sum(w_s, s_red);
    const double ym = block_sum(wy_s, s_red) / W;
    double wf_s = 0.0, yf_s = 0.0, yy_s = 0.0, m0 = 0.0, m1 = 0.0;
#pragma unroll 4
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        double w = 1.0 / load_in(dtype, dy, r0 + i);
        w = w * w;
        const double wn = w / W;
        const double yc = load_in(dtype, y, r0 + i) - ym;
        wf_s += (double)(float)wn;
        yf_s += (double)(float)(wn * yc);
        yy_s += wn * yc * yc;
        m0 = fmax(m0, (double)(float)wn);
        m1 = fmax(m1, fabs((double)(float)(wn * yc)));
    }
    const double wf = block_sum(wf_s, s_red);
    const double yf = block_sum(yf_s, s_red);
    const double yy = block_sum(yy_s, s_red);
    m0 = block_max(m0, s_red);
    m1 = block_max(m1, s_red);
    if (threadIdx.x == 0) {
        ob.wtot = W;
        ob.ymean = ym;
        ob.wsum_f = wf;
        ob.ybar_f = yf / wf;
        const double ybar = yf / wf;
        ob.norm = 1.0 / (yy - ybar * ybar);
        ob.norm32 = (float)ob.norm;
        ob.invw32 = (float)(1.0 / wf);
        ob.ybar32 = (float)ybar;
        ob.tsc0 = pow2_scale(m0);
        ob.tsc1 = pow2_scale(m1);
    }
}

// ---------------------------------------------------------------------------
// Observation records of the mixed kernel (FP64 set-up, once per row).
// ---------------------------------------------------------------------------
__global__ void records_kernel(int variant, int dtype, const void *t, const void *y,
                               const void *dy, const uint64_t *offsets, uint32_t n_obj,
                               const ObjInfo *objs, uint64_t rows, GridTurns g, void *rec,
                               uint32_t so_stride, int rotation) {
    for (uint64_t row = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; row < rows;
         row += (uint64_t)gridDim.x * blockDim.x) {
        const double td = load_in(dtype, t, row);
        const uint64_t a = frac_turns_u64(g.f0_hi, g.f0_lo, td);
        const uint64_t b = frac_turns_u64(g.df_hi, g.df_lo, td);
        // the step of the recurrence: one grid point, or so_stride of them (exact in the
        // fixed-point turns; the signed reading puts the angle in [-pi, pi))
        const uint64_t bs = b * (uint64_t)(so_stride ? so_stride : 1u);
        double sd = 0.0, cd = 0.0;  // (an FP64 sine/cosine: skipped for the tensor form)
        if (rotation) sincos((double)(long long)bs * kTwoPiOver2p64, &sd, &cd);
        ObsRec r;
        r.a_lo = (uint32_t)a;
        r.a_hi = (uint32_t)(a >> 32);
        r.b_lo = (uint32_t)b;
        r.b_hi = (uint32_t)(b >> 32);
        r.cd = (float)cd;
        r.sd = (float)sd;
        if (variant == 0) {
            r.v0 = (float)load_in(dtype, y, row);
            r.v1 = 0.0f;
        } else {
            // object of this row: last o with offsets[o] <= row
            uint32_t lo = 0, hi = n_obj;
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) >> 1;
                if (offsets[mid] <= row) lo = mid; else hi = mid;
            }
            const ObjInfo &ob = objs[lo];
            double w = 1.0 / load_in(dtype, dy, row);
            w = w * w;
            const double wn = w / ob.wtot;
            r.v0 = (float)wn;
            r.v1 = (float)(wn * (load_in(dtype, y, row) - ob.ymean));
        }
        if (!so_stride) {
            uint4 *d = reinterpret_cast<uint4 *>(static_cast<ObsRec *>(rec) + row);
            d[0] = make_uint4(r.a_lo, r.a_hi, r.b_lo, r.b_hi);
            reinterpret_cast<float4 *>(d)[1] = make_float4(r.v0, r.v1, r.cd, r.sd);
        } else {
            // the pair step phi = 2 so_stride grid points
            double s2, c2;
            sincos((double)(long long)(bs * 2u) * kTwoPiOver2p64, &s2, &c2);
            const float fc2 = (float)c2, fs2 = (float)s2, K = (float)(2.0 * c2);
            const uint32_t well = fabs(s2) >= kSecondOrderMinSin ? 1u : 0u;
            uint4 *d = static_cast<SoRec *>(rec)[row].q;
            d[0] = make_uint4(r.a_lo, r.a_hi, r.b_lo, r.b_hi);
            reinterpret_cast<float4 *>(d)[1] = make_float4(r.v0, r.v0, r.cd, r.sd);
            reinterpret_cast<float4 *>(d)[2] = make_float4(fc2, fc2, fs2, fs2);
            reinterpret_cast<float4 *>(d)[3] = make_float4(-fs2, -fs2, r.v1, r.v1);
            reinterpret_cast<float4 *>(d)[4] = make_float4(K, K, -K, -K);
            d[5] = make_uint4(__float_as_uint(-fc2), __float_as_uint(-fc2), well, 0u);
        }
    }
}

// ---------------------------------------------------------------------------
// Mixed kernel.
// ---------------------------------------------------------------------------

template <typename OutT>
__device__ __forceinline__ void store_out_d(void *pgram, uint64_t i, double p) {
    reinterpret_cast<OutT *>(pgram)[i] = (OutT)p;
}

// Shared-memory record of the packed (X2) loop, expanded from ObsRec at staging:
//   q0 = {a_lo, a_hi, b_lo, b_hi}
//   q1 = {v0, v0, cd, sd}            ({y,y} or {w,w}; the single step for the odd chain)
//   q2 = {cd2, cd2, sd2, sd2}        (the double step of both chains)
//   q3 = {-sd2, -sd2, v1, v1}        ({wy, wy} for the generalized variant)
// Each 64-bit half of q1..q3 is a ready-made packed operand. The second-order form
// (PK = 2) stages SoRec records (lsgb_internal.h) as they are.
constexpr int kX2RecBytes = 64;

// Accumulates one packed pair of frequencies: (cos, sin) pairs C, S with the weights V0
// (y, or w) and V1 (w y', generalized).
template <bool GEN, int NA, int NP>
__device__ __forceinline__ void accumulate_pair(uint64_t (&acc2)[NA][NP], int pp, uint64_t V0,
                                                uint64_t V1, uint64_t C, uint64_t S) {
    if (!GEN) {
        acc2[0][pp] = ffma2(V0, C, acc2[0][pp]);  // XC
        acc2[1][pp] = ffma2(V0, S, acc2[1][pp]);  // XS
        acc2[2][pp] = ffma2(C, C, acc2[2][pp]);   // CC
        acc2[3][pp] = ffma2(C, S, acc2[3][pp]);   // CS
    } else {
        const uint64_t WC = fmul2(V0, C);
        acc2[0][pp] = fadd2(acc2[0][pp], WC);     // C
        acc2[1][pp] = ffma2(V0, S, acc2[1][pp]);  // S
        acc2[2][pp] = ffma2(V1, C, acc2[2][pp]);  // YC
        acc2[3][pp] = ffma2(V1, S, acc2[3][pp]);  // YS
        acc2[4][pp] = ffma2(WC, C, acc2[4][pp]);  // CC
        acc2[5][pp] = ffma2(WC, S, acc2[5][pp]);  // CS
    }
}

// Mixed kernel, PK selects the inner loop:
//   0  scalar: F consecutive frequencies per thread, rotation steps;
//   1  packed f32x2: the same run as two interleaved chains (even / odd frequencies),
//      pair p = (k0 + 2p, k0 + 2p + 1), rotation steps of two grid points;
//   2  packed f32x2, strided: frequencies k0 + i NT (i < F), pair p = (k0 + 2p NT,
//      k0 + (2p+1) NT), steps of phi = 2 NT grid points by the second-order recurrence
//      x[p+1] = K x[p] - x[p-1], K = 2 cos phi, where it is well conditioned (SoRec).
// In form 2 the recurrence runs on sign-flipped values y[p] = sigma[p] x[p] with
// sigma = (+, +, -, -, +, +, ...), for which y[p+1] = (+-K) y[p] + y[p-1] needs no
// negation; the sums linear in (cos, sin) take the sign, the quadratic ones do not, and
// the epilogue flips it back. The rotation path of ill-conditioned observations produces
// the same signed values (by negated rotations where sigma changes).
template <int F, int NT, int MINB, bool GEN, int PK, int UJ, bool RA, typename OutT>
__global__ void __launch_bounds__(NT, MINB) mixed_kernel(MixedArgs a) {
    constexpr bool X2 = PK != 0;
    constexpr bool SO = PK == 2;
    static_assert(!(SO && RA), "re-anchoring applies to the consecutive-frequency forms");
    constexpr int RQ = SO ? 6 : (X2 ? 4 : 2);  // 16-byte quads per staged observation
    extern __shared__ __align__(16) unsigned char smem_raw[];
    uint4 *s_rec = reinterpret_cast<uint4 *>(smem_raw);  // RQ x uint4 per observation
    // second-level sums of objects longer than one staged chunk, private per thread:
    // s_fold[(q * F + f) * NT + tid]; present when a.fold != 0
    float *s_fold = reinterpret_cast<float *>(smem_raw + (size_t)a.chunk * (16 * RQ));
    __shared__ uint32_t s_unit;
    __shared__ float s_bp[NT / 32];
    __shared__ uint32_t s_bk[NT / 32];
    constexpr int NA = GEN ? 6 : 4;
    // frequency f of a thread is k0 + f * KS
    constexpr uint32_t KS = SO ? NT : 1;
    const uint32_t units = a.n_obj * a.n_tiles;

    for (;;) {
        if (threadIdx.x == 0) s_unit = atomicAdd(a.counter, 1u);
        __syncthreads();
        const uint32_t u = s_unit;
        if (u >= units) break;
        const uint32_t o = a.perm[u / a.n_tiles];
        const uint32_t tile = u - (u / a.n_tiles) * a.n_tiles;
        const uint64_t row0 = a.objs[o].row0;
        const uint32_t n = a.objs[o].n;
        const uint32_t k0 = tile * (uint32_t)(NT * F) + threadIdx.x * (uint32_t)(SO ? 1 : F);

        static_assert(!X2 || F % 2 == 0, "the packed loop needs an even F");
        constexpr int NP = X2 ? F / 2 : 1;
        float acc[NA][F];
        uint64_t acc2[NA][NP];
#pragma unroll
        for (int q = 0; q < NA; ++q) {
#pragma unroll
            for (int f = 0; f < F; ++f) acc[q][f] = 0.0f;
#pragma unroll
            for (int p = 0; p < NP; ++p) acc2[q][p] = 0ull;
        }

        const bool fold = a.fold && n > a.chunk;
        if (fold) {
#pragma unroll
            for (int q = 0; q < NA * F; ++q) s_fold[q * NT + threadIdx.x] = 0.0f;
        }
        for (uint32_t c0 = 0; c0 < n; c0 += a.chunk) {
            const uint32_t cnt = min(a.chunk, n - c0);
            if (SO) {
                const uint4 *src = reinterpret_cast<const SoRec *>(a.rec)[row0 + c0].q;
                for (uint32_t i = threadIdx.x; i < 6 * cnt; i += NT) s_rec[i] = __ldg(src + i);
            } else if (!X2) {
                const uint4 *src = reinterpret_cast<const uint4 *>(
                    static_cast<const ObsRec *>(a.rec) + row0 + c0);
                for (uint32_t i = threadIdx.x; i < 2 * cnt; i += NT) s_rec[i] = __ldg(src + i);
            } else {
                const uint4 *src = reinterpret_cast<const uint4 *>(
                    static_cast<const ObsRec *>(a.rec) + row0 + c0);
                for (uint32_t i = threadIdx.x; i < cnt; i += NT) {
                    const uint4 q0 = __ldg(src + 2 * i);
                    const uint4 qv = __ldg(src + 2 * i + 1);
                    const float v0 = __uint_as_float(qv.x), v1 = __uint_as_float(qv.y);
                    const float cd = __uint_as_float(qv.z), sd = __uint_as_float(qv.w);
                    const float cd2 = fmaf(cd, cd, -sd * sd), sd2 = 2.0f * cd * sd;
                    float4 *d = reinterpret_cast<float4 *>(s_rec) + 4 * i;
                    reinterpret_cast<uint4 *>(d)[0] = q0;
                    d[1] = make_float4(v0, v0, cd, sd);
                    d[2] = make_float4(cd2, cd2, sd2, sd2);
                    d[3] = make_float4(-sd2, -sd2, v1, v1);
                }
            }
            __syncthreads();
            // anchor: top 32 bits of a + ka*b (mod 2^64), as a signed turn count; ka is
            // the thread's first frequency, or with re-anchoring every R grid points the
            // R-aligned point below it. In the scalar loop the anchor of observation j+1 is
            // computed during observation j, off the critical path of its recurrence (the
            // packed loops measured faster without this).
            constexpr bool PIPE = !X2;
            const uint32_t adv = RA ? k0 % a.reanchor : 0u;
            const uint32_t ka = k0 - adv;
            auto anchor = [&](uint32_t jj, float &sa, float &ca) {
                const uint4 ab = s_rec[RQ * jj];
                const uint64_t p = (uint64_t)ka * ab.z + (((uint64_t)ab.y << 32) | ab.x);
                const uint32_t hi = (uint32_t)(p >> 32) + ka * ab.w;
                __sincosf((float)(int32_t)hi * kTwoPiOver2p32f, &sa, &ca);
            };
            float s_next = 0.0f, c_next = 0.0f;
            if (PIPE) anchor(0, s_next, c_next);
#pragma unroll UJ
            for (uint32_t j = 0; j < cnt; ++j) {
                float s, c;
                if (PIPE) {
                    s = s_next;
                    c = c_next;
                    anchor(min(j + 1, cnt - 1), s_next, c_next);
                } else {
                    anchor(j, s, c);
                }
                if (RA && adv) {
                    const float4 v = reinterpret_cast<const float4 *>(s_rec)[RQ * j + 1];
                    const float cd = v.z, sd = v.w;  // same place in both layouts
                    for (uint32_t q = 0; q < adv; ++q) {
                        const float cn = fmaf(c, cd, -s * sd);
                        s = fmaf(s, cd, c * sd);
                        c = cn;
                    }
                }
                if (!X2) {
                    const float4 v = reinterpret_cast<const float4 *>(s_rec)[2 * j + 1];
#pragma unroll
                    for (int f = 0; f < F; ++f) {
                        if (!GEN) {
                            acc[0][f] = fmaf(v.x, c, acc[0][f]);  // XC
                            acc[1][f] = fmaf(v.x, s, acc[1][f]);  // XS
                            acc[2][f] = fmaf(c, c, acc[2][f]);    // CC
                            acc[3][f] = fmaf(c, s, acc[3][f]);    // CS
                        } else {
                            const float wc = v.x * c;
                            acc[0][f] += wc;                       // C
                            acc[1][f] = fmaf(v.x, s, acc[1][f]);   // S
                            acc[2][f] = fmaf(v.y, c, acc[2][f]);   // YC
                            acc[3][f] = fmaf(v.y, s, acc[3][f]);   // YS
                            acc[4][f] = fmaf(wc, c, acc[4][f]);    // CC
                            acc[5][f] = fmaf(wc, s, acc[5][f]);    // CS
                        }
                        if (f + 1 < F) {
                            const float cn = fmaf(c, v.z, -s * v.w);
                            s = fmaf(s, v.z, c * v.w);
                            c = cn;
                        }
                    }
                } else {
                    const ulonglong2 *R = reinterpret_cast<const ulonglong2 *>(s_rec) + RQ * j;
                    const ulonglong2 q1 = R[1], q2 = R[2], q3 = R[3];
                    float cd, sd;
                    unpack2(q1.y, cd, sd);
                    const float c1 = fmaf(c, cd, -s * sd);  // odd lane: one step (or NT) ahead
                    const float s1 = fmaf(s, cd, c * sd);
                    uint64_t C = pack2(c, c1), S = pack2(s, s1);
                    const uint64_t V0 = q1.x, CD2 = q2.x, SD2 = q2.y, NSD2 = q3.x, V1 = q3.y;
                    if (!SO) {
#pragma unroll
                        for (int pp = 0; pp < NP; ++pp) {
                            accumulate_pair<GEN>(acc2, pp, V0, V1, C, S);
                            if (pp + 1 < NP) {
                                const uint64_t t1 = fmul2(S, NSD2);
                                const uint64_t t2 = fmul2(C, SD2);
                                C = ffma2(C, CD2, t1);
                                S = ffma2(S, CD2, t2);
                            }
                        }
                    } else {
                        accumulate_pair<GEN>(acc2, 0, V0, V1, C, S);
                        // pair 1 by a rotation (sigma[1] = sigma[0])
                        uint64_t Cp = C, Sp = S;
                        if (NP > 1) {
                            const uint64_t t1 = fmul2(S, NSD2);
                            const uint64_t t2 = fmul2(C, SD2);
                            C = ffma2(C, CD2, t1);
                            S = ffma2(S, CD2, t2);
                            accumulate_pair<GEN>(acc2, 1, V0, V1, C, S);
                        }
                        const ulonglong2 q5 = R[5];
                        if ((uint32_t)q5.y) {
                            // well conditioned: y[p] = A[p] y[p-1] + y[p-2], A[p] = -K for
                            // even p, +K for odd p
                            const ulonglong2 q4 = R[4];
#pragma unroll
                            for (int pp = 2; pp < NP; ++pp) {
                                const uint64_t A = (pp & 1) ? q4.x : q4.y;
                                const uint64_t Cn = ffma2(A, C, Cp);
                                const uint64_t Sn = ffma2(A, S, Sp);
                                Cp = C;
                                Sp = S;
                                C = Cn;
                                S = Sn;
                                accumulate_pair<GEN>(acc2, pp, V0, V1, C, S);
                            }
                        } else {
                            // rotation; negated where sigma changes sign (even p)
                            const uint64_t NCD2 = q5.x;
#pragma unroll
                            for (int pp = 2; pp < NP; ++pp) {
                                if (pp & 1) {
                                    const uint64_t t1 = fmul2(S, NSD2);
                                    const uint64_t t2 = fmul2(C, SD2);
                                    C = ffma2(C, CD2, t1);
                                    S = ffma2(S, CD2, t2);
                                } else {
                                    const uint64_t t1 = fmul2(S, SD2);
                                    const uint64_t t2 = fmul2(C, NSD2);
                                    C = ffma2(C, NCD2, t1);
                                    S = ffma2(S, NCD2, t2);
                                }
                                accumulate_pair<GEN>(acc2, pp, V0, V1, C, S);
                            }
                        }
                    }
                }
            }
            if (fold) {
                // fold this chunk's FP32 sums into the second level and restart them, so
                // rounding grows with sqrt(chunk) + sqrt(n / chunk) rather than sqrt(n)
#pragma unroll
                for (int q = 0; q < NA; ++q) {
                    if (X2) {
#pragma unroll
                        for (int pp = 0; pp < NP; ++pp) {
                            float lo, hi2;
                            unpack2(acc2[q][pp], lo, hi2);
                            s_fold[(q * F + 2 * pp) * NT + threadIdx.x] += lo;
                            s_fold[(q * F + 2 * pp + 1) * NT + threadIdx.x] += hi2;
                            acc2[q][pp] = 0ull;
                        }
                    } else {
#pragma unroll
                        for (int f = 0; f < F; ++f) {
                            s_fold[(q * F + f) * NT + threadIdx.x] += acc[q][f];
                            acc[q][f] = 0.0f;
                        }
                    }
                }
            }
            __syncthreads();
        }
        if (fold) {
#pragma unroll
            for (int q = 0; q < NA; ++q)
#pragma unroll
                for (int f = 0; f < F; ++f) acc[q][f] = s_fold[(q * F + f) * NT + threadIdx.x];
        } else if (X2) {
#pragma unroll
            for (int q = 0; q < NA; ++q)
#pragma unroll
                for (int pp = 0; pp < NP; ++pp) {
                    unpack2(acc2[q][pp], acc[q][2 * pp], acc[q][2 * pp + 1]);
                }
        }
        if (SO) {
            // undo sigma on the sums linear in (cos, sin): pairs 2, 3 (mod 4)
#pragma unroll
            for (int q = 0; q < (GEN ? 4 : 2); ++q)
#pragma unroll
                for (int f = 0; f < F; ++f)
                    if ((f >> 2) & 1) acc[q][f] = -acc[q][f];
        }

        // epilogue: power, optional store, thread-local first maximum (all FP32: the
        // FP64 pipe of this part is 1/64 of the FP32 rate)
        float bp = 0.0f;
        uint32_t bk = 0xffffffffu;
        if (tile == 0 && threadIdx.x == 0) bk = 0;  // the reference's (power 0, index 0) start
        const bool top3 = a.top == 3u && a.best_key;  // the three best, not the maximum
        // the object's current third key: whatever is not above it is dropped here
        const unsigned long long g3 =
            top3 ? *(volatile unsigned long long *)(a.best_key + 3ull * o + 2) : 0ull;
        Top3 t3;
        t3.seed(g3);
        const uint64_t out0 = (uint64_t)o * a.n_freq;
        const float nrm = a.objs[o].norm32;
        if (!GEN) {
            const float N = (float)n;
#pragma unroll
            for (int f = 0; f < F; ++f) {
                const uint32_t k = k0 + f * KS;
                const float P = std_power_f(N, acc[0][f], acc[1][f], acc[2][f], acc[3][f]) * nrm;
                if (k < a.n_freq) {
                    if (a.pgram) store_out<OutT>(a.pgram, out0 + k, P);
                    if (top3) t3.offer(P, k);
                    else if (P > bp) { bp = P; bk = k; }
                }
            }
        } else {
            const float invW = a.objs[o].invw32;
            const float ybar = a.objs[o].ybar32;
#pragma unroll
            for (int f = 0; f < F; ++f) {
                const uint32_t k = k0 + f * KS;
                const float P = gen_power_f(invW, ybar, acc[0][f], acc[1][f], acc[2][f], acc[3][f],
                                            acc[4][f], acc[5][f]) * nrm;
                if (k < a.n_freq) {
                    if (a.pgram) store_out<OutT>(a.pgram, out0 + k, P);
                    if (top3) t3.offer(P, k);
                    else if (P > bp) { bp = P; bk = k; }
                }
            }
        }
        if (top3) {
            // the warp's three best, then into the object's three slots; a warp none of whose
            // lanes beat the seed has nothing to insert
            if (__any_sync(0xffffffffu, t3.t0 > g3)) t3.warp_merge();
            if ((threadIdx.x & 31) == 0 && t3.t0 > g3) {
                unsigned long long *slots = a.best_key + 3ull * o;
                top3_insert(slots, t3.t0);
                top3_insert(slots, t3.t1);
                top3_insert(slots, t3.t2);
            }
        } else if (a.best_key) {
            // warp maximum, then one 64-bit atomicMax per warp: larger power wins, and on
            // equal power the larger ~index, i.e. the lower index (the first maximum)
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                const float op = __shfl_xor_sync(0xffffffffu, bp, off);
                const uint32_t ok = __shfl_xor_sync(0xffffffffu, bk, off);
                if (better(op, ok, bp, bk)) { bp = op; bk = ok; }
            }
            if ((threadIdx.x & 31) == 0 && bp > 0.0f)
                atomicMax(a.best_key + o,
                          ((unsigned long long)__float_as_uint(bp) << 32) | (unsigned long long)(~bk));
        } else if (a.tile_best) {
            block_best<NT, float>(bp, bk, s_bp, s_bk);
            if (threadIdx.x == 0) {
                TileBest tb;
                tb.p = (double)bp;
                tb.k = bk;
                tb.pad = 0;
                a.tile_best[(uint64_t)o * a.n_tiles + tile] = tb;
            }
            __syncthreads();
        }
    }
}


// ---------------------------------------------------------------------------
// FP64 sine and cosine for the plain kernel, written for the FP64 pipe of this part
// (1/64 of the FP32 rate), from published methods:
//  * Cody & Waite argument reduction (Software Manual for the Elementary Functions,
//    1980) modulo pi/64, with pi/64 as a double-double (FMA makes n*C1 exact enough for
//    |x| < 2^34 * pi/64) and the integer n obtained by the 1.5*2^52 rounding trick;
//  * a table of sin/cos(j pi/64), j = 0..127 (Tang's table-driven scheme), built per CTA
//    in shared memory with sincospi;
//  * Taylor polynomials on |r| <= pi/128: sin to r^7 (next term < 9e-21) and cos to r^6
//    (next term < 3.3e-18, under half an ulp of 1);
//  * sin(a+r) = sin a cos r + cos a sin r, cos(a+r) = cos a cos r - sin a sin r.
// About 16 FP64 operations against roughly twice that for the general-purpose
// sincos(). Arguments with |x| > 1e9 rad use sincos(). Checked against sincos() by
// lsgb_fp64_sincos_check.
// ---------------------------------------------------------------------------
constexpr double kPiOver64Hi = 0.04908738521234052;
constexpr double kPiOver64Lo = 1.9135106236677394e-18;
constexpr double k64OverPi = 20.371832715762604;
constexpr double kRoundMagic = 6755399441055744.0;  // 1.5 * 2^52

__device__ __forceinline__ void table_sincos(double x, const double2 *tab, double *s, double *c) {
    if (fabs(x) > 1.0e9) {
        sincos(x, s, c);
        return;
    }
    const double nm = fma(x, k64OverPi, kRoundMagic);
    const int j = __double2loint(nm) & 127;
    const double n = nm - kRoundMagic;
    const double r = fma(-n, kPiOver64Lo, fma(-n, kPiOver64Hi, x));
    const double r2 = r * r;
    const double sp = fma(r2, fma(r2, -0.0001984126984126984, 0.008333333333333333),
                          -0.16666666666666666);
    const double sr = fma(r * r2, sp, r);
    const double cr = fma(r2, fma(r2, fma(r2, -0.001388888888888889, 0.041666666666666664), -0.5),
                          1.0);
    const double2 t = tab[j];  // (sin, cos) of j pi/64
    *s = fma(t.x, cr, t.y * sr);
    *c = fma(t.y, cr, -(t.x * sr));
}

__device__ __forceinline__ void fill_sincos_table(double2 *tab) {
    for (int j = threadIdx.x; j < 128; j += blockDim.x) {
        double sj, cj;
        sincospi((double)j / 64.0, &sj, &cj);
        tab[j] = make_double2(sj, cj);
    }
}

__global__ void sincos_check_kernel(uint32_t n, uint64_t seed, double scale, double *max_err) {
    __shared__ double2 tab[128];
    fill_sincos_table(tab);
    __syncthreads();
    double worst = 0.0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        // a deterministic spread of arguments over [-scale, scale] (splitmix64 stream)
        uint64_t z = seed + 0x9e3779b97f4a7c15ull * (i + 1);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        z ^= z >> 31;
        const double x = ((double)(z >> 11) * 0x1.0p-53 * 2.0 - 1.0) * scale;
        double s1, c1, s2, c2;
        table_sincos(x, tab, &s1, &c1);
        sincos(x, &s2, &c2);
        worst = fmax(worst, fmax(fabs(s1 - s2), fabs(c1 - c2)));
    }
    for (int o = 16; o > 0; o >>= 1) worst = fmax(worst, __shfl_xor_sync(0xffffffffu, worst, o));
    if ((threadIdx.x & 31) == 0) {
        // non-negative doubles order like their bit patterns
        atomicMax(reinterpret_cast<unsigned long long *>(max_err), __double_as_longlong(worst));
    }
}

// ---------------------------------------------------------------------------
// Plain FP64 kernel: the reference's arithmetic, one frequency per thread.
// ---------------------------------------------------------------------------
template <int NT, bool GEN, typename InT, typename OutT>
__global__ void __launch_bounds__(NT) plain_kernel(PlainArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *s_t = reinterpret_cast<double *>(smem_raw);
    double *s_y = s_t + a.chunk;
    double *s_w = s_y + a.chunk;  // generalized only
    __shared__ uint32_t s_unit;
    __shared__ double s_bp[NT / 32];
    __shared__ uint32_t s_bk[NT / 32];
    __shared__ double s_bp3[3 * (NT / 32)];     // top-3 per warp (PlainArgs::top == 3)
    __shared__ uint32_t s_bk3[3 * (NT / 32)];
    __shared__ double2 s_tab[128];
    fill_sincos_table(s_tab);  // made visible by the first barrier of the unit loop
    const InT *T = reinterpret_cast<const InT *>(a.t);
    const InT *Y = reinterpret_cast<const InT *>(a.y);
    const InT *DY = reinterpret_cast<const InT *>(a.dy);
    const uint32_t units = a.n_obj * a.n_tiles;

    for (;;) {
        if (threadIdx.x == 0) s_unit = atomicAdd(a.counter, 1u);
        __syncthreads();
        const uint32_t u = s_unit;
        if (u >= units) break;
        const uint32_t o = a.perm[u / a.n_tiles];
        const uint32_t tile = u - (u / a.n_tiles) * a.n_tiles;
        const uint64_t row0 = a.objs[o].row0;
        const uint32_t n = a.objs[o].n;
        const uint32_t k = tile * (uint32_t)NT + threadIdx.x;
        // source/main.cu:1611 / source/kernel.cu:538: omega = minFreq + freqStep*k, with the
        // product rounded before the add as the reference's host code does (a fused
        // multiply-add would move omega by an ulp: 7e-8 rad of phase at t ~ 2.5e6 d)
        const double w = __dadd_rn(a.fmin, __dmul_rn(a.df, (double)k));
        double P;
        if (!GEN) {
            double xc = 0.0, xs = 0.0, cc = 0.0, ss = 0.0, cs = 0.0;
            for (uint32_t c0 = 0; c0 < n; c0 += a.chunk) {
                const uint32_t cnt = min(a.chunk, n - c0);
                for (uint32_t i = threadIdx.x; i < cnt; i += NT) {
                    s_t[i] = (double)T[row0 + c0 + i];
                    s_y[i] = (double)Y[row0 + c0 + i];
                }
                __syncthreads();
#pragma unroll 2
                for (uint32_t j = 0; j < cnt; ++j) {
                    double s, c;
                    table_sincos(w * s_t[j], s_tab, &s, &c);
                    const double yj = s_y[j];
                    xc += yj * c;
                    xs += yj * s;
                    cc += c * c;
                    ss += s * s;
                    cs += c * s;
                }
                __syncthreads();
            }
            // source/main.cu:1588-1598
            const double tau = atan2(2.0 * cs, cc - ss) / (2.0 * w);
            double s_tau, c_tau;
            sincos(w * tau, &s_tau, &c_tau);
            const double c_tau2 = c_tau * c_tau, s_tau2 = s_tau * s_tau;
            const double cs_tau = 2.0 * c_tau * s_tau;
            const double f1 = c_tau * xc + s_tau * xs;
            const double f2 = c_tau * xs - s_tau * xc;
            P = 0.5 * ((f1 * f1) / (c_tau2 * cc + cs_tau * cs + s_tau2 * ss) +
                       (f2 * f2) / (c_tau2 * ss - cs_tau * cs + s_tau2 * cc));
            P *= a.objs[o].norm;
        } else {
            // source/main.cu:1701-1777 (two passes over the observations)
            double wsum = 0.0, S = 0.0, C = 0.0, S2 = 0.0, C2 = 0.0;
            const bool one_chunk = n <= a.chunk;
            for (int pass = 0; pass < 2; ++pass) {
                double tau = 0.0;
                if (pass == 1) {
                    S2 /= wsum;
                    C2 /= wsum;
                    S /= wsum;
                    C /= wsum;
                    S2 -= (2.0 * S * C);
                    C2 -= (C * C - S * S);
                    tau = 0.5 * atan2(S2, C2) / w;
                }
                double Y_ = 0.0, YY = 0.0, Ct = 0.0, St = 0.0, YCt = 0.0, YSt = 0.0, CCt = 0.0,
                       SSt = 0.0;
                for (uint32_t c0 = 0; c0 < n; c0 += a.chunk) {
                    const uint32_t cnt = min(a.chunk, n - c0);
                    if (!(one_chunk && pass == 1)) {
                        for (uint32_t i = threadIdx.x; i < cnt; i += NT) {
                            s_t[i] = (double)T[row0 + c0 + i];
                            s_y[i] = (double)Y[row0 + c0 + i];
                            double wi = 1.0 / (double)DY[row0 + c0 + i];
                            s_w[i] = wi * wi;
                        }
                        __syncthreads();
                    }
                    if (pass == 0) {
#pragma unroll 2
                        for (uint32_t j = 0; j < cnt; ++j) {
                            const double wj = s_w[j];
                            double s, c;
                            table_sincos(w * s_t[j], s_tab, &s, &c);
                            wsum += wj;
                            S += wj * s;
                            C += wj * c;
                            S2 += 2.0 * wj * s * c;
                            C2 += wj - 2.0 * wj * s * s;
                        }
                    } else {
#pragma unroll 2
                        for (uint32_t j = 0; j < cnt; ++j) {
                            const double wj = s_w[j], yj = s_y[j];
                            double s, c;
                            table_sincos(w * (s_t[j] - tau), s_tab, &s, &c);
                            Y_ += wj * yj;
                            YY += wj * yj * yj;
                            Ct += wj * c;
                            St += wj * s;
                            YCt += wj * yj * c;
                            YSt += wj * yj * s;
                            CCt += wj * c * c;
                            SSt += wj * s * s;
                        }
                    }
                    if (!(one_chunk && pass == 0)) __syncthreads();
                }
                if (pass == 1) {
                    Y_ /= wsum;
                    YY /= wsum;
                    Ct /= wsum;
                    St /= wsum;
                    YCt /= wsum;
                    YSt /= wsum;
                    CCt /= wsum;
                    SSt /= wsum;
                    YCt -= Y_ * Ct;
                    YSt -= Y_ * St;
                    CCt -= Ct * Ct;
                    SSt -= St * St;
                    YY -= Y_ * Y_;
                    P = (YCt * YCt / CCt + YSt * YSt / SSt) / YY;
                }
            }
        }
        double bp = 0.0;
        uint32_t bk = 0xffffffffu;
        if (tile == 0 && threadIdx.x == 0) bk = 0;
        double Pr = 0.0;
        if (k < a.n_freq) {
            if (a.pgram) store_out_d<OutT>(a.pgram, (uint64_t)o * a.n_freq + k, P);
            Pr = (double)(OutT)P;  // compare in the output precision
            if (Pr > bp) { bp = Pr; bk = k; }
        }
        if (a.tile_best && a.top == 3u) {
            // the tile's three best: per warp, then warp 0 over the warps' triples (constant
            // indices throughout, so that the triples stay in registers)
            Top3PK<double> t3;
            if (k < a.n_freq) t3.offer(Pr, k);
            t3.warp_merge();
            const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
            if (l == 0) {
#pragma unroll
                for (int r = 0; r < 3; ++r) { s_bp3[w * 3 + r] = t3.p[r]; s_bk3[w * 3 + r] = t3.k[r]; }
            }
            __syncthreads();
            if (w == 0) {
                Top3PK<double> m;
                if (l < NT / 32)
#pragma unroll
                    for (int r = 0; r < 3; ++r) m.offer(s_bp3[l * 3 + r], s_bk3[l * 3 + r]);
                m.warp_merge();
                if (l == 0) {
#pragma unroll
                    for (int r = 0; r < 3; ++r) {
                        TileBest tb;
                        tb.p = m.p[r];
                        tb.k = m.k[r];
                        tb.pad = 0;
                        a.tile_best[((uint64_t)o * a.n_tiles + tile) * 3u + (uint32_t)r] = tb;
                    }
                }
            }
        } else if (a.tile_best) {
            block_best<NT, double>(bp, bk, s_bp, s_bk);
            if (threadIdx.x == 0) {
                TileBest tb;
                tb.p = bp;
                tb.k = bk;
                tb.pad = 0;
                a.tile_best[(uint64_t)o * a.n_tiles + tile] = tb;
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Per-object argmax over the tile results, tiles in frequency order, first
// maximum wins; one warp per object.
// ---------------------------------------------------------------------------
template <typename OutT>
__global__ void best_reduce_kernel(const TileBest *tb, uint32_t n_obj, uint32_t n_tiles,
                                   uint32_t *best_idx, OutT *best_power) {
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= n_obj) return;
    double bp = 0.0;
    uint32_t bk = 0xffffffffu;
    for (uint32_t i = lane; i < n_tiles; i += 32) {
        const TileBest x = tb[(uint64_t)warp * n_tiles + i];
        if (better(x.p, x.k, bp, bk)) { bp = x.p; bk = x.k; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double op = __shfl_xor_sync(0xffffffffu, bp, o);
        const uint32_t ok = __shfl_xor_sync(0xffffffffu, bk, o);
        if (better(op, ok, bp, bk)) { bp = op; bk = ok; }
    }
    if (lane == 0) {
        if (best_idx) best_idx[warp] = bk == 0xffffffffu ? 0u : bk;
        if (best_power) best_power[warp] = (OutT)bp;
    }
}

// The same for the tiles' top-3 triples: the object's three best (power, lowest index)
// pairs, best first, (0, 0) where fewer than three positive powers exist.
template <typename OutT>
__global__ void best3_reduce_kernel(const TileBest *tb, uint32_t n_obj, uint32_t n_tiles,
                                    uint32_t *best_idx, OutT *best_power) {
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= n_obj) return;
    Top3PK<double> t3;
    for (uint32_t i = lane; i < n_tiles * 3u; i += 32) {
        const TileBest x = tb[(uint64_t)warp * n_tiles * 3u + i];
        t3.offer(x.p, x.k);
    }
    t3.warp_merge();
    if (lane == 0) {
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            const bool none = t3.k[r] == 0xffffffffu;
            if (best_idx) best_idx[3ull * warp + r] = none ? 0u : t3.k[r];
            if (best_power) best_power[3ull * warp + r] = none ? OutT(0) : (OutT)t3.p[r];
        }
    }
}

template <typename OutT>
__global__ void key_decode_kernel(const unsigned long long *keys, uint32_t n_obj, uint32_t *best_idx,
                                  OutT *best_power) {
    const uint32_t o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= n_obj) return;
    const unsigned long long k = keys[o];
    if (best_idx) best_idx[o] = k ? ~(uint32_t)k : 0u;
    if (best_power) best_power[o] = (OutT)__uint_as_float((uint32_t)(k >> 32));
}

template <int F, int NT, int MINB, bool GEN, int PK, int UJ, bool RA>
cudaError_t launch_mixed_t(int dtype, const MixedArgs &a, int grid, size_t smem, cudaStream_t st) {
    if (dtype == 0) {
        auto k = mixed_kernel<F, NT, MINB, GEN, PK, UJ, RA, float>;
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k<<<grid, NT, smem, st>>>(a);
    } else {
        auto k = mixed_kernel<F, NT, MINB, GEN, PK, UJ, RA, double>;
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k<<<grid, NT, smem, st>>>(a);
    }
    return cudaGetLastError();
}

template <int F, int NT, int MINB, bool GEN, int PK, int UJ, bool RA>
cudaError_t occ_mixed_t(int dtype, size_t smem, int *blocks) {
    cudaError_t e;
    if (dtype == 0) {
        auto k = mixed_kernel<F, NT, MINB, GEN, PK, UJ, RA, float>;
        e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k, NT, smem);
    } else {
        auto k = mixed_kernel<F, NT, MINB, GEN, PK, UJ, RA, double>;
        e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k, NT, smem);
    }
    return e;
}

// The compiled mixed shapes: (frequencies per thread, threads, min CTAs per SM for
// the register budget, generalized?, inner loop form (0 scalar, 1 packed rotation,
// 2 packed second-order), observations per iteration, re-anchoring study variant?).
// Study variants are chosen by lsgb_set_reanchor, not listed as tuning shapes.
#define LSGB_MIXED_SHAPES(X)            \
    X(16, 256, 2, false, 0, 1, false)   \
    X(8, 256, 3, false, 0, 1, false)    \
    X(12, 256, 2, false, 1, 1, false)   \
    X(12, 128, 4, false, 1, 1, false)   \
    X(10, 256, 2, false, 1, 1, false)   \
    X(8, 256, 3, false, 1, 1, false)    \
    X(12, 256, 2, false, 2, 1, false)   \
    X(16, 256, 2, false, 2, 1, false)   \
    X(8, 256, 3, false, 2, 1, false)    \
    X(10, 256, 3, false, 2, 1, false)   \
    X(12, 256, 2, true, 0, 1, false)    \
    X(8, 256, 2, true, 1, 1, false)     \
    X(8, 128, 4, true, 1, 1, false)     \
    X(10, 256, 2, true, 1, 1, false)    \
    X(8, 256, 2, true, 2, 1, false)     \
    X(6, 256, 3, true, 2, 1, false)     \
    X(10, 256, 2, true, 2, 1, false)    \
    X(12, 256, 2, false, 1, 1, true)    \
    X(8, 256, 2, true, 1, 1, true)

}  // namespace

cudaError_t launch_stats(int variant, int mixed, int dtype, int normalize, const void *t,
                         const void *y, const void *dy, ObjInfo *objs, uint32_t n_obj,
                         uint32_t *status, cudaStream_t st, unsigned long long *keys,
                         uint32_t top, uint32_t *counter) {
    if (n_obj == 0) return cudaSuccess;
    stats_kernel<<<n_obj, 256, 0, st>>>(variant, mixed, dtype, normalize, t, y, dy, objs, status,
                                        keys, top, counter);
    return cudaGetLastError();
}

cudaError_t launch_records(int variant, int dtype, const void *t, const void *y, const void *dy,
                           const uint64_t *offsets, uint32_t n_obj, const ObjInfo *objs,
                           uint64_t rows, GridTurns g, void *rec, uint32_t so_stride,
                           cudaStream_t st, bool rotation) {
    if (rows == 0) return cudaSuccess;
    const uint64_t blocks64 = (rows + 255) / 256;
    const int blocks = (int)(blocks64 < 65535ull * 16 ? blocks64 : 65535ull * 16);
    records_kernel<<<blocks, 256, 0, st>>>(variant, dtype, t, y, dy, offsets, n_obj, objs, rows, g,
                                           rec, so_stride, rotation || so_stride ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_mixed(int variant, int dtype, MixedShape shape, const MixedArgs &a, int grid,
                         size_t smem, cudaStream_t st) {
    if (shape.x2 == 3) {
        if ((uint32_t)shape.f * (uint32_t)shape.nt != tensor_tile_freqs(variant) || shape.minb != 1 ||
            shape.uj || a.reanchor)
            return cudaErrorInvalidValue;
        return launch_tensor(variant, dtype, a, grid, st);
    }
#define X(F_, NT_, MB_, G_, PK_, UJ_, RA_)                                           \
    if (shape.f == F_ && shape.nt == NT_ && shape.minb == MB_ && (variant == 1) == G_ && \
        shape.x2 == PK_ && (shape.uj ? 2 : 1) == UJ_ && (a.reanchor != 0) == RA_)        \
        return launch_mixed_t<F_, NT_, MB_, G_, PK_, UJ_, RA_>(dtype, a, grid, smem, st);
    LSGB_MIXED_SHAPES(X)
#undef X
    return cudaErrorInvalidValue;
}

int mixed_shapes(int *out, int max_shapes) {
    int n = 0;
#define X(F_, NT_, MB_, G_, PK_, UJ_, RA_)       \
    if (RA_) {                                   \
    } else if (out && n < max_shapes) {          \
        out[6 * n + 0] = G_ ? 1 : 0;             \
        out[6 * n + 1] = F_;                     \
        out[6 * n + 2] = NT_;                    \
        out[6 * n + 3] = MB_;                    \
        out[6 * n + 4] = PK_;                    \
        out[6 * n + 5] = UJ_ == 2 ? 1 : 0;       \
    }                                            \
    n += RA_ ? 0 : 1;
    LSGB_MIXED_SHAPES(X)
#undef X
    // the tensor-core form of each variant: (coarse steps per unit, 128 fine steps)
    for (int v = 0; v < 2; ++v) {
        if (out && n < max_shapes) {
            out[6 * n + 0] = v;
            out[6 * n + 1] = (int)(tensor_tile_freqs(v) / 128u);
            out[6 * n + 2] = 128;
            out[6 * n + 3] = 1;
            out[6 * n + 4] = 3;
            out[6 * n + 5] = 0;
        }
        ++n;
    }
    return n;
}

cudaError_t mixed_occupancy(int variant, int dtype, MixedShape shape, size_t smem, int *blocks) {
    if (shape.x2 == 3) {
        if ((uint32_t)shape.f * (uint32_t)shape.nt != tensor_tile_freqs(variant) || shape.minb != 1 ||
            shape.uj)
            return cudaErrorInvalidValue;
        *blocks = 1;
        return cudaSuccess;
    }
#define X(F_, NT_, MB_, G_, PK_, UJ_, RA_)                                           \
    if (shape.f == F_ && shape.nt == NT_ && shape.minb == MB_ && (variant == 1) == G_ && \
        shape.x2 == PK_ && (shape.uj ? 2 : 1) == UJ_ && !RA_)                            \
        return occ_mixed_t<F_, NT_, MB_, G_, PK_, UJ_, RA_>(dtype, smem, blocks);
    LSGB_MIXED_SHAPES(X)
#undef X
    return cudaErrorInvalidValue;
}

namespace {
template <bool GEN, typename InT, typename OutT>
cudaError_t plain_t(const PlainArgs &a, int grid, size_t smem, cudaStream_t st, int *occ) {
    auto k = plain_kernel<kPlainThreads, GEN, InT, OutT>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if (occ) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, k, kPlainThreads, smem);
    k<<<grid, kPlainThreads, smem, st>>>(a);
    return cudaGetLastError();
}
template <bool GEN>
cudaError_t plain_dispatch(int in_dtype, int out_dtype, const PlainArgs &a, int grid, size_t smem,
                           cudaStream_t st, int *occ) {
    if (in_dtype == 0 && out_dtype == 0) return plain_t<GEN, float, float>(a, grid, smem, st, occ);
    if (in_dtype == 0 && out_dtype == 1) return plain_t<GEN, float, double>(a, grid, smem, st, occ);
    if (in_dtype == 1 && out_dtype == 0) return plain_t<GEN, double, float>(a, grid, smem, st, occ);
    return plain_t<GEN, double, double>(a, grid, smem, st, occ);
}
}  // namespace

cudaError_t launch_plain(int variant, int in_dtype, int out_dtype, const PlainArgs &a, int grid,
                         size_t smem, cudaStream_t st) {
    return variant == 0 ? plain_dispatch<false>(in_dtype, out_dtype, a, grid, smem, st, nullptr)
                        : plain_dispatch<true>(in_dtype, out_dtype, a, grid, smem, st, nullptr);
}

cudaError_t plain_occupancy(int variant, int in_dtype, int out_dtype, size_t smem, int *blocks) {
    PlainArgs dummy{};
    return variant == 0 ? plain_dispatch<false>(in_dtype, out_dtype, dummy, 0, smem, 0, blocks)
                        : plain_dispatch<true>(in_dtype, out_dtype, dummy, 0, smem, 0, blocks);
}

cudaError_t launch_sincos_check(uint32_t n, uint64_t seed, double scale, double *max_err,
                                cudaStream_t st) {
    sincos_check_kernel<<<256, 256, 0, st>>>(n, seed, scale, max_err);
    return cudaGetLastError();
}

cudaError_t launch_key_decode(int dtype, const unsigned long long *keys, uint32_t n_obj,
                              uint32_t *best_idx, void *best_power, cudaStream_t st) {
    if (n_obj == 0) return cudaSuccess;
    const int blocks = (int)((n_obj + 255) / 256);
    if (dtype == 0)
        key_decode_kernel<float><<<blocks, 256, 0, st>>>(keys, n_obj, best_idx, (float *)best_power);
    else
        key_decode_kernel<double><<<blocks, 256, 0, st>>>(keys, n_obj, best_idx, (double *)best_power);
    return cudaGetLastError();
}

cudaError_t launch_best_reduce(int dtype, const TileBest *tb, uint32_t n_obj, uint32_t n_tiles,
                               uint32_t top, uint32_t *best_idx, void *best_power, cudaStream_t st) {
    if (n_obj == 0) return cudaSuccess;
    const int threads = 256;
    const int blocks = (int)((n_obj * 32ull + threads - 1) / threads);
    if (top == 3u) {
        if (dtype == 0)
            best3_reduce_kernel<float><<<blocks, threads, 0, st>>>(tb, n_obj, n_tiles, best_idx,
                                                                   (float *)best_power);
        else
            best3_reduce_kernel<double><<<blocks, threads, 0, st>>>(tb, n_obj, n_tiles, best_idx,
                                                                    (double *)best_power);
        return cudaGetLastError();
    }
    if (top != 1u) return cudaErrorInvalidValue;
    if (dtype == 0)
        best_reduce_kernel<float><<<blocks, threads, 0, st>>>(tb, n_obj, n_tiles, best_idx,
                                                              (float *)best_power);
    else
        best_reduce_kernel<double><<<blocks, threads, 0, st>>>(tb, n_obj, n_tiles, best_idx,
                                                               (double *)best_power);
    return cudaGetLastError();
}

}  // namespace lsgb
