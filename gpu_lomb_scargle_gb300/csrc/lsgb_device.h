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
