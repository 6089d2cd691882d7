// lsgb_device.h -- device helpers shared by the CUDA-core kernels (lsgb_kernels.cu) and
// the tensor-core kernel (lsgb_tensor.cu). Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace lsgb {
namespace {

constexpr float kTwoPiOver2p32f = 1.4629180792671596e-09f;  // 2 pi / 2^32

// Packed FP32 pairs (Blackwell f32x2): one instruction issues two FP32 lanes' work.
__device__ __forceinline__ uint64_t ffma2(uint64_t a, uint64_t b, uint64_t c) {
    uint64_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ uint64_t fmul2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t fadd2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t fsub2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t pack2(float lo, float hi) {
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void unpack2(uint64_t v, float &lo, float &hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}

// (power, index) ordering of the reference's argmax (source/main.cu:1545-1563):
// larger power wins, equal power -> lower index (the first maximum).
template <typename V>
__device__ __forceinline__ bool better(V p1, uint32_t k1, V p2, uint32_t k2) {
    return p1 > p2 || (p1 == p2 && k1 < k2);
}

// ---- the three best frequencies of an object (source/main.cu:1165-1219) ----
// The reference scans the periodogram three times from (power 0, index 0), each scan
// taking the first strictly larger power at an index the earlier scans did not take. So
// its result is the three largest (power, lowest index) pairs among the positive powers,
// in that order, padded with (0, index 0). With a positive FP32 power the key
// (power bits << 32 | ~index) orders pairs that way as one unsigned integer (0: none).
__device__ __forceinline__ unsigned long long rank_key(float p, uint32_t k) {
    return ((unsigned long long)__float_as_uint(p) << 32) | (unsigned long long)(~k);
}

// A thread's or warp's three largest keys, t0 > t1 > t2 (0 = empty).
struct Top3 {
    unsigned long long t0 = 0ull, t1 = 0ull, t2 = 0ull;
    float floor2 = 0.0f;  // the power of t2: a smaller power can never enter
    // Starts from a known lower bound g (the object's current third key, which only grows):
    // keys not above g could never be inserted and are not kept. The triple then holds
    // copies of g below the keys that beat it; g itself is never offered again.
    __device__ __forceinline__ void seed(unsigned long long g) {
        t0 = t1 = t2 = g;
        floor2 = __uint_as_float((uint32_t)(g >> 32));
    }
    // Offers a key (keys offered to one Top3 are distinct).
    __device__ __forceinline__ void offer(unsigned long long x) {
        if (x > t2) {
            if (x > t1) {
                t2 = t1;
                if (x > t0) { t1 = t0; t0 = x; }
                else t1 = x;
            } else {
                t2 = x;
            }
            floor2 = __uint_as_float((uint32_t)(t2 >> 32));
        }
    }
    // Offers a positive power at frequency index k; one float compare for the powers below
    // the current third (an equal power may still enter, with a lower index).
    __device__ __forceinline__ void offer(float p, uint32_t k) {
        if (p > 0.0f && p >= floor2) offer(rank_key(p, k));
    }
    // Offers n powers p[i] at indices k0 + i * step behind one branch on their maximum,
    // which after the first few is almost always below the floor.
    template <int n>
    __device__ __forceinline__ void offer_run(const float (&p)[n], uint32_t k0, uint32_t step) {
        float m = p[0];
#pragma unroll
        for (int i = 1; i < n; ++i) m = fmaxf(m, p[i]);
        if (m > 0.0f && m >= floor2) {
#pragma unroll
            for (int i = 0; i < n; ++i) offer(p[i], k0 + step * (uint32_t)i);
        }
    }
    // Merges the three keys of every lane of the (converged) warp into every lane. The
    // butterfly pairs disjoint groups of lanes, so the keys merged are always distinct.
    __device__ __forceinline__ void warp_merge() {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const unsigned long long u0 = __shfl_xor_sync(0xffffffffu, t0, off);
            const unsigned long long u1 = __shfl_xor_sync(0xffffffffu, t1, off);
            const unsigned long long u2 = __shfl_xor_sync(0xffffffffu, t2, off);
            if (u0) offer(u0);
            if (u1) offer(u1);
            if (u2) offer(u2);
        }
    }
};

// Inserts key x into an object's global top three slots s[0] > s[1] > s[2] (zero-
// initialized). Each level keeps the larger of what it holds and what arrives and passes
// the smaller on: level 0 ends with the largest key ever inserted, level 1 with the
// largest of the rest, and so on, whatever the interleaving of concurrent inserts. Keys
// not above the current third slot are skipped with one plain load (slots only grow).
__device__ __forceinline__ void top3_insert(unsigned long long *s, unsigned long long x) {
    if (x == 0ull || x <= *(volatile unsigned long long *)(s + 2)) return;
#pragma unroll
    for (int i = 0; i < 3 && x != 0ull; ++i) {
        const unsigned long long old = atomicMax(s + i, x);
        x = old < x ? old : x;
    }
}

// The same for (power, index) pairs of any type (the FP64 form keeps per-tile triples).
template <typename V>
struct Top3PK {
    V p[3] = {V(0), V(0), V(0)};
    uint32_t k[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu};  // 0xffffffff: empty
    // Offers a pair; only positive powers count (the reference's scans start at 0).
    __device__ __forceinline__ void offer(V q, uint32_t j) {
        if (j == 0xffffffffu || !(q > V(0)) || !better(q, j, p[2], k[2])) return;
        if (better(q, j, p[1], k[1])) {
            p[2] = p[1]; k[2] = k[1];
            if (better(q, j, p[0], k[0])) { p[1] = p[0]; k[1] = k[0]; p[0] = q; k[0] = j; }
            else { p[1] = q; k[1] = j; }
        } else {
            p[2] = q; k[2] = j;
        }
    }
    __device__ __forceinline__ void warp_merge() {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            V q[3];
            uint32_t j[3];
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                q[r] = __shfl_xor_sync(0xffffffffu, p[r], off);
                j[r] = __shfl_xor_sync(0xffffffffu, k[r], off);
            }
#pragma unroll
            for (int r = 0; r < 3; ++r) offer(q[r], j[r]);
        }
    }
};

// Standard L-S power from the sums of one frequency (N observations):
//   P = 1/2 [ (Q+U)/(N+r) + (Q-U)/(N-r) ],  Q = XC^2+XS^2,
//   U = [ (CC-SS)(XC^2-XS^2) + 4 CS XC XS ] / r,  r = hypot(CC-SS, 2 CS),
// which is source/main.cu:1588-1598 with cos/sin(2 omega tau) = (CC-SS, 2CS)/r.
// N - r is evaluated as 4 (CC SS - CS^2)/(N + r) to avoid cancellation, so with
// d1 = N + r, d4 = 4 (CC SS - CS^2) and t = 1/(d1 d4):
//   P = 1/2 [ (Q+U) (d4 t) + (Q-U) d1 (d1 t) ],
// the factors d4 t = 1/d1 and d1 t = 1/(N - r) formed before they meet Q, U. Two SFU
// operations: one reciprocal square root (1/r, and r = h/sqrt(h)) and one reciprocal.
__device__ __forceinline__ float std_power_f(float N, float xc, float xs, float cc, float cs) {
    const float ss = N - cc;
    const float D = cc - ss;
    const float E = 2.0f * cs;
    const float h = fmaf(D, D, E * E);
    const float ir = h > 0.0f ? rsqrtf(h) : 0.0f;  // 1/r
    const float r = h * ir;
    const float xc2 = xc * xc, xs2 = xs * xs;
    const float Q = xc2 + xs2;
    const float V = xc2 - xs2;
    const float U = h > 0.0f ? fmaf(D, V, 2.0f * E * xc * xs) * ir : V;
    const float d1 = N + r;
    const float d4 = 4.0f * fmaf(cc, ss, -cs * cs);
    const float t = __fdividef(1.0f, d1 * d4);
    return 0.5f * fmaf(Q + U, d4 * t, (Q - U) * (d1 * (d1 * t)));
}

// Twice the standard power from the raw sums XC, XS (of v e^{i theta}) and C2, S2 (of
// e^{2 i theta}) of N observations, N2 = N^2. With cc = (N + C2)/2, ss = (N - C2)/2 and
// cs = S2/2 the quantities of std_power_f reduce to D = C2, E = S2 and
// d4 = 4 (cc ss - cs^2) = N^2 - (C2^2 + S2^2) = N^2 - h.
__device__ __forceinline__ float std_power2_sums(float N, float N2, float xc, float xs,
                                                 float c2, float s2) {
    const float h = fmaf(c2, c2, s2 * s2);
    const float ir = h > 0.0f ? rsqrtf(h) : 0.0f;  // 1/r
    const float r = h * ir;
    const float xc2 = xc * xc;
    const float Q = fmaf(xs, xs, xc2);
    const float V = fmaf(-xs, xs, xc2);
    const float xs2 = xs + xs;
    const float U = h > 0.0f ? fmaf(c2, V, (s2 * xc) * xs2) * ir : V;
    const float d1 = N + r;
    const float d4 = N2 - h;
    const float t = __fdividef(1.0f, d1 * d4);
    return fmaf(Q + U, d4 * t, (Q - U) * (d1 * (d1 * t)));
}

// std_power2_sums for two frequencies at once, every argument a packed f32x2 pair (NN and
// NN2 hold N and N^2 twice): the arithmetic in packed instructions, the reciprocal square
// root and the reciprocal per lane.
__device__ __forceinline__ uint64_t std_power2_sums2(uint64_t NN, uint64_t NN2, uint64_t xc,
                                                     uint64_t xs, uint64_t c2, uint64_t s2) {
    const uint64_t h = ffma2(c2, c2, fmul2(s2, s2));
    float h0, h1;
    unpack2(h, h0, h1);
    // 1/r where h > 0; where h = 0, U = V (weight z = 1 on V)
    const uint64_t ir = pack2(h0 > 0.0f ? rsqrtf(h0) : 0.0f, h1 > 0.0f ? rsqrtf(h1) : 0.0f);
    const uint64_t z = pack2(h0 > 0.0f ? 0.0f : 1.0f, h1 > 0.0f ? 0.0f : 1.0f);
    const uint64_t r = fmul2(h, ir);
    const uint64_t xc2 = fmul2(xc, xc), xs2 = fmul2(xs, xs);
    const uint64_t Q = fadd2(xc2, xs2), V = fsub2(xc2, xs2);
    const uint64_t u0 = ffma2(c2, V, fmul2(fmul2(s2, xc), fadd2(xs, xs)));
    const uint64_t U = ffma2(V, z, fmul2(u0, ir));
    const uint64_t d1 = fadd2(NN, r);
    const uint64_t d4 = fsub2(NN2, h);
    float e0, e1;
    unpack2(fmul2(d1, d4), e0, e1);
    const uint64_t t = pack2(__fdividef(1.0f, e0), __fdividef(1.0f, e1));
    return ffma2(fadd2(Q, U), fmul2(d4, t), fmul2(fsub2(Q, U), fmul2(d1, fmul2(d1, t))));
}

// Generalized power from weight-normalized sums: cb, sb = C/W, S/W; yc, ys the centered
// YC/W - ybar cb, YS/W - ybar sb; c2, s2 = C2/W, S2/W (sums of w e^{2 i theta}). The
// covariances of gen_power_f reduce to D = vcc - vss = c2 - cb^2 + sb^2,
// E = 2 vcs = s2 - 2 cb sb, T = vcc + vss = 1 - cb^2 - sb^2 and
// d4 = 4 (vcc vss - vcs^2) = T^2 - (D^2 + E^2).
__device__ __forceinline__ float gen_power_sums(float cb, float sb, float yc, float ys, float c2,
                                                float s2) {
    const float cb2 = cb * cb, sb2 = sb * sb;
    const float D = (c2 - cb2) + sb2;
    const float m = cb * sb;
    const float E = fmaf(-2.0f, m, s2);
    const float T = (1.0f - cb2) - sb2;
    const float h = fmaf(D, D, E * E);
    const float ir = h > 0.0f ? rsqrtf(h) : 0.0f;  // 1/r
    const float r = h * ir;
    const float yc2 = yc * yc;
    const float Q = fmaf(ys, ys, yc2);
    const float V = fmaf(-ys, ys, yc2);
    const float ys2 = ys + ys;
    const float U = h > 0.0f ? fmaf(D, V, (E * yc) * ys2) * ir : V;
    const float d1 = T + r;
    const float d4 = fmaf(T, T, -h);
    const float t = __fdividef(1.0f, d1 * d4);
    return fmaf(Q + U, d4 * t, (Q - U) * (d1 * (d1 * t)));
}

// gen_power_sums for two frequencies at once (packed f32x2 pairs).
__device__ __forceinline__ uint64_t gen_power_sums2(uint64_t cb, uint64_t sb, uint64_t yc,
                                                    uint64_t ys, uint64_t c2, uint64_t s2) {
    const uint64_t one = pack2(1.0f, 1.0f), m2 = pack2(-2.0f, -2.0f);
    const uint64_t cb2 = fmul2(cb, cb), sb2 = fmul2(sb, sb);
    const uint64_t D = fadd2(fsub2(c2, cb2), sb2);
    const uint64_t E = ffma2(m2, fmul2(cb, sb), s2);
    const uint64_t T = fsub2(fsub2(one, cb2), sb2);
    const uint64_t h = ffma2(D, D, fmul2(E, E));
    float h0, h1;
    unpack2(h, h0, h1);
    // 1/r where h > 0; where h = 0, U = V (weight z = 1 on V)
    const uint64_t ir = pack2(h0 > 0.0f ? rsqrtf(h0) : 0.0f, h1 > 0.0f ? rsqrtf(h1) : 0.0f);
    const uint64_t z = pack2(h0 > 0.0f ? 0.0f : 1.0f, h1 > 0.0f ? 0.0f : 1.0f);
    const uint64_t r = fmul2(h, ir);
    const uint64_t yc2 = fmul2(yc, yc), ys2 = fmul2(ys, ys);
    const uint64_t Q = fadd2(yc2, ys2), V = fsub2(yc2, ys2);
    const uint64_t u0 = ffma2(D, V, fmul2(fmul2(E, yc), fadd2(ys, ys)));
    const uint64_t U = ffma2(V, z, fmul2(u0, ir));
    const uint64_t d1 = fadd2(T, r);
    const uint64_t d4 = fsub2(fmul2(T, T), h);
    float e0, e1;
    unpack2(fmul2(d1, d4), e0, e1);
    const uint64_t t = pack2(__fdividef(1.0f, e0), __fdividef(1.0f, e1));
    return ffma2(fadd2(Q, U), fmul2(d4, t), fmul2(fsub2(Q, U), fmul2(d1, fmul2(d1, t))));
}

// Generalized (floating-mean) power from weighted sums with total weight W:
// the same closed form applied to the weighted covariances, which is
// source/main.cu:1728-1776 with the second pass expressed by rotating the
// first-pass sums by omega*tau.
__device__ __forceinline__ float gen_power_f(float invW, float ybar, float C, float S, float YC,
                                             float YS, float CC, float CS) {
    const float cb = C * invW, sb = S * invW;
    const float cc = CC * invW, cs = CS * invW;
    const float ss = 1.0f - cc;
    const float yc = fmaf(-ybar, cb, YC * invW);
    const float ys = fmaf(-ybar, sb, YS * invW);
    const float vcc = fmaf(-cb, cb, cc);
    const float vss = fmaf(-sb, sb, ss);
    const float vcs = fmaf(-cb, sb, cs);
    const float D = vcc - vss, E = 2.0f * vcs, T = vcc + vss;
    const float h = fmaf(D, D, E * E);
    const float ir = h > 0.0f ? rsqrtf(h) : 0.0f;  // 1/r
    const float r = h * ir;
    const float yc2 = yc * yc, ys2 = ys * ys;
    const float Q = yc2 + ys2, V = yc2 - ys2;
    const float U = h > 0.0f ? fmaf(D, V, 2.0f * E * yc * ys) * ir : V;
    const float d1 = T + r;
    const float d4 = 4.0f * fmaf(vcc, vss, -vcs * vcs);
    const float t = __fdividef(1.0f, d1 * d4);
    return fmaf(Q + U, d4 * t, (Q - U) * (d1 * (d1 * t)));
}

template <typename OutT>
__device__ __forceinline__ void store_out(void *pgram, uint64_t i, float p) {
    reinterpret_cast<OutT *>(pgram)[i] = (OutT)p;
}
}  // namespace
}  // namespace lsgb
