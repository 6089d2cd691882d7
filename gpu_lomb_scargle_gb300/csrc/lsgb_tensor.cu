// lsgb_tensor.cu -- the tensor-core form of the mixed periodogram (sm_103a: tcgen05, TMEM).
//
// The sums of the hot loop (source/kernel.cu:484-631 standard, :368-477 generalized) are
// recast as small complex matrix products. Within one work unit (object o, frequencies
// k = kT + p + 128 m, p < 128, m < NM) the phase of observation j is
//   theta_jk = alpha_jp + m beta_j,  alpha_jp = (fmin + (kT + p) df) t_j,  beta_j = 128 df t_j,
// so with A[p][j] = v_j exp(i alpha_jp) and B[m][j] = exp(i m beta_j)
//   sum_j v_j exp(i theta_jk) = (A B^T)[p][m],
// and the squared terms follow from the doubled angle, cos^2 = (1 + cos 2theta) / 2,
// cos sin = sin 2theta / 2, with A2 = exp(2i alpha), B2 = exp(2i m beta). Both angles
// come from the exact 64-bit fixed-point phases of ObsRec (a + k b mod 2^64 turns).
//
// Each complex product is two real MMAs with N = 2 NM: [XC | XS] = Ar [Br | Bi]^T +
// Ai [-Bi | Br]^T, the right factors being two overlapping row windows of
// Z = [-Bi; Br; Bi]. FP32 accuracy on the TF32 tensor cores comes from the split
// x = hi + lo (hi = x rounded to TF32, lo = x - hi): a b ~ ah bh + ah bl + al bh
// (the dropped al bl is below 2^-21 relative).
//
// One persistent CTA per SM, warp-specialized:
//   warps 0-3   epilogue: read the accumulators from TMEM (warp w owns lanes 32w..),
//               power per frequency, periodogram store, per-object maximum;
//   warp 4      TMEM allocation and the MMA issuer (one thread);
//   warps 5-12  producers: the split operands of 8 observations (one K-block) per stage
//               of a shared-memory ring, in the K-major no-swizzle layout.
// Shared-memory stages and the two TMEM accumulator buffers are handed over with
// mbarriers. Every wait is bounded: on a timeout the kernel records an error in
// MixedArgs::status, lets its issued MMAs drain, frees its TMEM and returns.
#include <cuda_runtime.h>
#include <stdint.h>

#include "lsgb_device.h"
#include "lsgb_internal.h"

namespace lsgb {

namespace {

constexpr int kTP = 128;        // fine frequency offsets p: A rows, TMEM lanes
constexpr int kTK = 8;          // observations per K-block (the TF32 MMA depth)
constexpr int kStages = 3;      // shared-memory ring depth
constexpr int kThreads = 416;   // 13 warps
constexpr int kProducerThreads = 256;
constexpr int kEpilogueThreads = 128;
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kBufCols = 256;  // TMEM columns of one accumulator buffer
constexpr long long kWaitCycles = 1ll << 32;  // ~2 s at 2 GHz

// Per-variant geometry.
template <bool GEN>
struct TGeo {
    static constexpr int NM = GEN ? 32 : 64;       // coarse frequency steps m per unit
    static constexpr int N = 2 * NM;               // MMA N: [real | imaginary]
    static constexpr int NAG = GEN ? 3 : 2;        // A groups: v e^ia (, v1 e^ia), e^2ia
    static constexpr int A_BYTES = kTP * kTK * 4;  // one 128 x 8 TF32 matrix
    static constexpr int Z_ROWS = 3 * NM;
    static constexpr int Z_BYTES = Z_ROWS * kTK * 4;
    // stage: A matrices (group g, part re/im, hi/lo) then Z matrices (angle 1/2, hi/lo)
    static constexpr int A_OFF = 0;
    static constexpr int Z_OFF = NAG * 4 * A_BYTES;
    static constexpr int STAGE = ((Z_OFF + 4 * Z_BYTES) + 1023) / 1024 * 1024;
    static constexpr int TILE = kTP * NM;          // frequencies per unit
};

// Byte offset of element (row r, column k < 8) of a K-major, no-swizzle operand:
// 8-row x 16-byte core matrices, the two K halves 128 bytes apart (LBO), row groups
// 256 bytes apart (SBO).
__device__ __forceinline__ uint32_t kmaj_off(uint32_t r, uint32_t k) {
    return (r & 7u) * 16u + (r >> 3) * 256u + (k & 3u) * 4u + (k >> 2) * 128u;
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor (tcgen05): start address, LBO, SBO in 16-byte units,
// descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)(128u >> 4) << 16) |
           ((uint64_t)(256u >> 4) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::tf32, FP32 accumulator, K-major A and B.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void split_tf32(float x, uint32_t &hi, uint32_t &lo) {
    uint32_t h;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(x));
    hi = h;
    lo = __float_as_uint(x - __uint_as_float(h));
}

__device__ __forceinline__ void mbar_init(uint64_t *b, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count));
}
__device__ __forceinline__ void mbar_arrive(uint64_t *b) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t *b, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; "
        "selp.u32 %0, 1, 0, p; }"
        : "=r"(done)
        : "r"(smem_u32(b)), "r"(parity)
        : "memory");
    return done != 0;
}

// Waits for the phase of `parity` of barrier b. Returns false (and raises the CTA's
// abort flag and the launch's status) on a timeout or when another role aborted.
__device__ __noinline__ bool mbar_wait(uint64_t *b, uint32_t parity, volatile uint32_t *abort,
                                       uint32_t *status) {
    if (mbar_test(b, parity)) return true;
    const long long t0 = clock64();
    for (uint32_t it = 1;; ++it) {
        if (mbar_test(b, parity)) return true;
        if ((it & 255u) == 0) {
            if (*abort) return false;
            if (clock64() - t0 > kWaitCycles) {
                *abort = 1u;
                if (status) atomicOr(status, 1u);
                return false;
            }
        }
    }
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{ .reg .pred p; setp.ne.b32 p, %4, 0; "
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p; }" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t *b) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(b))
                 : "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

// 16 consecutive accumulator columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
        "%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_wait_ld() {
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Phase of fixed-point turn count x as (sin, cos) on the SFU.
__device__ __forceinline__ void turn_sincos(uint32_t hi, float &s, float &c) {
    __sincosf((float)(int32_t)hi * kTwoPiOver2p32f, &s, &c);
}

struct UnitInfo {
    uint32_t o, tile, n;
    uint64_t row0;
};

__device__ __forceinline__ UnitInfo unit_info(const MixedArgs &a, uint32_t u) {
    UnitInfo w;
    const uint32_t oi = u / a.n_tiles;
    w.o = a.perm[oi];
    w.tile = u - oi * a.n_tiles;
    w.row0 = a.objs[w.o].row0;
    w.n = a.objs[w.o].n;
    return w;
}

template <bool GEN, typename OutT>
__global__ void __launch_bounds__(kThreads, 1) tensor_kernel(MixedArgs a) {
    using G = TGeo<GEN>;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // 1024-byte aligned ring of stages
    unsigned char *ring = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    __shared__ __align__(8) uint64_t full_bar[kStages], empty_bar[kStages];
    __shared__ __align__(8) uint64_t accf_bar[2], acce_bar[2], drain_bar;
    __shared__ uint32_t s_tmem;
    __shared__ volatile uint32_t s_abort;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t units = a.n_obj * a.n_tiles;

    if (tid == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&full_bar[s], kProducerThreads);
            mbar_init(&empty_bar[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&accf_bar[b], 1);
            mbar_init(&acce_bar[b], kEpilogueThreads);
        }
        mbar_init(&drain_bar, 1);
        s_abort = 0u;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 4) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&s_tmem)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = s_tmem;

    if (warp >= 5) {
        // ---------------- producers ----------------
        const uint32_t pt = (uint32_t)tid - 160u;
        const uint32_t p = pt >> 1, h = pt & 1u;  // A: row p, observations 4h..4h+3
        // B: std: m = pt / 4, observations 2(pt % 4) + {0, 1}; gen: m = pt / 8, obs pt % 8
        const uint32_t bm = GEN ? (pt >> 3) : (pt >> 2);
        const uint32_t bj0 = GEN ? (pt & 7u) : 2u * (pt & 3u);
        constexpr int BJ = GEN ? 1 : 2;
        uint32_t g = 0;
        for (uint32_t u = blockIdx.x; u < units && !s_abort; u += gridDim.x) {
            const UnitInfo w = unit_info(a, u);
            const uint32_t kT = w.tile * (uint32_t)G::TILE;
            const uint32_t nkb = (w.n + kTK - 1) / kTK;
            const ObsRec *rec = static_cast<const ObsRec *>(a.rec) + w.row0;
            for (uint32_t kb = 0; kb < nkb; ++kb, ++g) {
                const uint32_t s = g % kStages, use = g / kStages;
                if (!mbar_wait(&empty_bar[s], (use & 1u) ^ 1u, &s_abort, a.status)) break;
                unsigned char *st = ring + (size_t)s * G::STAGE;
                // A operands: row p, four observations
                {
                    float ar[4], ai[4], a3r[4], a3i[4], a2r[4], a2i[4];
                    const uint32_t ka = kT + p;
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const uint32_t j = kb * kTK + 4u * h + (uint32_t)q;
                        const bool valid = j < w.n;
                        const uint4 r0 = __ldg(reinterpret_cast<const uint4 *>(rec + (valid ? j : w.n - 1)));
                        const float4 r1 =
                            __ldg(reinterpret_cast<const float4 *>(rec + (valid ? j : w.n - 1)) + 1);
                        const uint64_t ph = (uint64_t)ka * r0.z + (((uint64_t)r0.y << 32) | r0.x);
                        const uint32_t hi = (uint32_t)(ph >> 32) + ka * r0.w;
                        float sn, cs;
                        turn_sincos(hi, sn, cs);
                        const float v0 = valid ? r1.x : 0.0f;
                        ar[q] = v0 * cs;
                        ai[q] = v0 * sn;
                        if (GEN) {
                            const float v1 = valid ? r1.y : 0.0f;
                            a3r[q] = v1 * cs;
                            a3i[q] = v1 * sn;
                            // weighted doubled angle: w cos 2t, w sin 2t
                            a2r[q] = v0 * fmaf(cs, cs, -sn * sn);
                            a2i[q] = v0 * (2.0f * cs * sn);
                        } else {
                            a2r[q] = valid ? fmaf(cs, cs, -sn * sn) : 0.0f;
                            a2i[q] = valid ? 2.0f * cs * sn : 0.0f;
                        }
                    }
                    const uint32_t off = kmaj_off(p, 4u * h);
                    auto put4 = [&](int mat, const float (&x)[4]) {
                        uint32_t hi[4], lo[4];
#pragma unroll
                        for (int q = 0; q < 4; ++q) split_tf32(x[q], hi[q], lo[q]);
                        unsigned char *base = st + G::A_OFF + (size_t)mat * G::A_BYTES + off;
                        *reinterpret_cast<uint4 *>(base) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
                        *reinterpret_cast<uint4 *>(base + G::A_BYTES) =
                            make_uint4(lo[0], lo[1], lo[2], lo[3]);
                    };
                    // matrix order: group g: (re hi, re lo, im hi, im lo) at 4g..4g+3
                    put4(0, ar);
                    put4(2, ai);
                    if (GEN) {
                        put4(4, a3r);
                        put4(6, a3i);
                        put4(8, a2r);
                        put4(10, a2i);
                    } else {
                        put4(4, a2r);
                        put4(6, a2i);
                    }
                }
                // Z operands: Z = [-Bi; Br; Bi] for angle m beta and 2 m beta
                {
                    float cr[BJ], si[BJ], c2[BJ], s2[BJ];
                    const uint32_t kb128 = 128u * bm;
#pragma unroll
                    for (int q = 0; q < BJ; ++q) {
                        const uint32_t j = kb * kTK + bj0 + (uint32_t)q;
                        const uint4 r0 =
                            __ldg(reinterpret_cast<const uint4 *>(rec + (j < w.n ? j : w.n - 1)));
                        const uint64_t ph = (uint64_t)kb128 * r0.z;
                        const uint32_t hi = (uint32_t)(ph >> 32) + kb128 * r0.w;
                        float sn, cs;
                        turn_sincos(hi, sn, cs);
                        cr[q] = cs;
                        si[q] = sn;
                        c2[q] = fmaf(cs, cs, -sn * sn);
                        s2[q] = 2.0f * cs * sn;
                    }
                    auto putz = [&](int zmat, uint32_t row, const float *x, bool neg) {
                        unsigned char *base =
                            st + G::Z_OFF + (size_t)zmat * G::Z_BYTES + kmaj_off(row, bj0);
                        uint32_t hi[BJ], lo[BJ];
#pragma unroll
                        for (int q = 0; q < BJ; ++q) split_tf32(neg ? -x[q] : x[q], hi[q], lo[q]);
                        if (BJ == 2) {
                            *reinterpret_cast<uint2 *>(base) = make_uint2(hi[0], hi[BJ - 1]);
                            *reinterpret_cast<uint2 *>(base + G::Z_BYTES) = make_uint2(lo[0], lo[BJ - 1]);
                        } else {
                            *reinterpret_cast<uint32_t *>(base) = hi[0];
                            *reinterpret_cast<uint32_t *>(base + G::Z_BYTES) = lo[0];
                        }
                    };
                    constexpr uint32_t NM = G::NM;
                    // angle m beta: Z matrices 0 (hi), 1 (lo); 2 m beta: 2 (hi), 3 (lo)
                    putz(0, bm, si, true);
                    putz(0, NM + bm, cr, false);
                    putz(0, 2 * NM + bm, si, false);
                    putz(2, bm, s2, true);
                    putz(2, NM + bm, c2, false);
                    putz(2, 2 * NM + bm, s2, false);
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                mbar_arrive(&full_bar[s]);
            }
        }
    } else if (warp == 4) {
        // ---------------- MMA issuer ----------------
        if (lane == 0) {
            constexpr uint32_t idesc = idesc_tf32(kTP, G::N);
            uint32_t g = 0, lu = 0;
            bool ok = true;
            for (uint32_t u = blockIdx.x; u < units && ok; u += gridDim.x, ++lu) {
                const UnitInfo w = unit_info(a, u);
                const uint32_t nkb = (w.n + kTK - 1) / kTK;
                const uint32_t buf = lu & 1u, ub = lu >> 1;
                if (!mbar_wait(&acce_bar[buf], (ub & 1u) ^ 1u, &s_abort, a.status)) break;
                tc_fence_after();
                const uint32_t d0 = tmem + buf * kBufCols;
                for (uint32_t kb = 0; kb < nkb; ++kb, ++g) {
                    const uint32_t s = g % kStages, use = g / kStages;
                    if (!mbar_wait(&full_bar[s], use & 1u, &s_abort, a.status)) { ok = false; break; }
                    tc_fence_after();
                    const uint32_t sb = smem_u32(ring + (size_t)s * G::STAGE);
                    auto adesc = [&](int mat) { return sdesc(sb + G::A_OFF + mat * G::A_BYTES); };
                    // right factors: [Br; Bi] = Z rows NM.., [-Bi; Br] = Z rows 0..
                    auto zdesc = [&](int zmat, int row0) {
                        return sdesc(sb + G::Z_OFF + zmat * G::Z_BYTES + row0 * 32);
                    };
                    const uint32_t acc0 = kb > 0 ? 1u : 0u;
                    // one complex product: D += A_g (re, im) x Z_z, split-TF32
                    auto cplx = [&](uint32_t d, int ga, int zz) {
                        const uint64_t arh = adesc(4 * ga + 0), arl = adesc(4 * ga + 1);
                        const uint64_t aih = adesc(4 * ga + 2), ail = adesc(4 * ga + 3);
                        const uint64_t bh = zdesc(zz, G::NM), bl = zdesc(zz + 1, G::NM);
                        const uint64_t nh = zdesc(zz, 0), nl = zdesc(zz + 1, 0);
                        mma_tf32(d, arh, bh, idesc, acc0);
                        mma_tf32(d, arh, bl, idesc, 1u);
                        mma_tf32(d, arl, bh, idesc, 1u);
                        mma_tf32(d, aih, nh, idesc, 1u);
                        mma_tf32(d, aih, nl, idesc, 1u);
                        mma_tf32(d, ail, nh, idesc, 1u);
                    };
                    if (GEN) {
                        cplx(d0 + 0, 0, 0);                    // [C | S]
                        cplx(d0 + (uint32_t)G::N, 1, 0);       // [YC | YS]
                        cplx(d0 + 2u * (uint32_t)G::N, 2, 2);  // [C2 | S2]
                    } else {
                        cplx(d0 + 0, 0, 0);                    // [XC | XS]
                        cplx(d0 + (uint32_t)G::N, 1, 2);       // [C2 | S2]
                    }
                    mma_commit(&empty_bar[s]);
                }
                if (!ok) break;
                mma_commit(&accf_bar[buf]);
            }
            // every issued MMA has completed before TMEM is released
            mma_commit(&drain_bar);
            const long long t0 = clock64();
            while (!mbar_test(&drain_bar, 0u) && clock64() - t0 < kWaitCycles) {
            }
        }
        __syncwarp();
    } else {
        // ---------------- epilogue (warps 0-3: TMEM lanes 32 warp ..) ----------------
        const uint32_t pl = (uint32_t)warp * 32u + (uint32_t)lane;
        const uint32_t lane_base = ((uint32_t)warp * 32u) << 16;
        uint32_t lu = 0;
        for (uint32_t u = blockIdx.x; u < units; u += gridDim.x, ++lu) {
            const UnitInfo w = unit_info(a, u);
            const uint32_t buf = lu & 1u, ub = lu >> 1;
            if (!mbar_wait(&accf_bar[buf], ub & 1u, &s_abort, a.status)) break;
            tc_fence_after();
            const uint32_t d0 = tmem + lane_base + buf * kBufCols;
            const uint32_t kT = w.tile * (uint32_t)G::TILE;
            const ObjInfo &ob = a.objs[w.o];
            const float nrm = ob.norm32;
            const uint64_t out0 = (uint64_t)w.o * a.n_freq;
            float bp = 0.0f;
            uint32_t bk = 0xffffffffu;
            if (w.tile == 0 && pl == 0) bk = 0;  // the reference's (power 0, index 0) start
#pragma unroll 1
            for (int m0 = 0; m0 < G::NM; m0 += 16) {
                float re[16], im[16], r2[16], i2[16];
                float yr[16], yi[16];
                tmem_ld16(d0 + (uint32_t)m0, re);
                tmem_ld16(d0 + (uint32_t)(G::NM + m0), im);
                if (GEN) {
                    tmem_ld16(d0 + (uint32_t)(G::N + m0), yr);
                    tmem_ld16(d0 + (uint32_t)(G::N + G::NM + m0), yi);
                    tmem_ld16(d0 + (uint32_t)(2 * G::N + m0), r2);
                    tmem_ld16(d0 + (uint32_t)(2 * G::N + G::NM + m0), i2);
                } else {
                    tmem_ld16(d0 + (uint32_t)(G::N + m0), r2);
                    tmem_ld16(d0 + (uint32_t)(G::N + G::NM + m0), i2);
                }
                tmem_wait_ld();
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    const uint32_t k = kT + pl + (uint32_t)kTP * (uint32_t)(m0 + i);
                    float P;
                    if (GEN) {
                        // CC = (W + sum w cos 2t) / 2, CS = sum w sin 2t / 2, W = wsum_f
                        const float W = __fdividef(1.0f, ob.invw32);
                        P = gen_power_f(ob.invw32, ob.ybar32, re[i], im[i], yr[i], yi[i],
                                        0.5f * (W + r2[i]), 0.5f * i2[i]) *
                            nrm;
                    } else {
                        const float N = (float)w.n;
                        P = std_power_f(N, re[i], im[i], 0.5f * (N + r2[i]), 0.5f * i2[i]) * nrm;
                    }
                    if (k < a.n_freq) {
                        if (a.pgram) store_out<OutT>(a.pgram, out0 + k, P);
                        if (better(P, k, bp, bk)) { bp = P; bk = k; }
                    }
                }
            }
            tc_fence_before();
            mbar_arrive(&acce_bar[buf]);
            if (a.best_key) {
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) {
                    const float op = __shfl_xor_sync(0xffffffffu, bp, off);
                    const uint32_t ok = __shfl_xor_sync(0xffffffffu, bk, off);
                    if (better(op, ok, bp, bk)) { bp = op; bk = ok; }
                }
                if (lane == 0 && bp > 0.0f)
                    atomicMax(a.best_key + w.o,
                              ((unsigned long long)__float_as_uint(bp) << 32) |
                                  (unsigned long long)(~bk));
            }
        }
    }

    tc_fence_before();
    __syncthreads();
    if (warp == 4) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(kTmemCols)
                     : "memory");
    }
}

template <bool GEN>
size_t tensor_smem() {
    return (size_t)kStages * TGeo<GEN>::STAGE + 1024;
}

template <bool GEN, typename OutT>
cudaError_t launch_t(const MixedArgs &a, int grid, cudaStream_t st) {
    auto k = tensor_kernel<GEN, OutT>;
    const size_t smem = tensor_smem<GEN>();
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<grid, kThreads, smem, st>>>(a);
    return cudaGetLastError();
}

}  // namespace

uint32_t tensor_tile_freqs(int variant) {
    return variant ? (uint32_t)TGeo<true>::TILE : (uint32_t)TGeo<false>::TILE;
}

size_t tensor_smem_bytes(int variant) { return variant ? tensor_smem<true>() : tensor_smem<false>(); }

cudaError_t launch_tensor(int variant, int dtype, const MixedArgs &a, int grid, cudaStream_t st) {
    if (variant == 0) return dtype == 0 ? launch_t<false, float>(a, grid, st) : launch_t<false, double>(a, grid, st);
    return dtype == 0 ? launch_t<true, float>(a, grid, st) : launch_t<true, double>(a, grid, st);
}

}  // namespace lsgb
