// lsgb_tensor.cu -- the tensor-core form of the mixed periodogram (sm_103a: tcgen05, TMEM,
// bulk copies).
//
// The sums of the hot loop (source/kernel.cu:484-631 standard, :368-477 generalized) are
// recast as small complex matrix products. Within one work unit (object o, frequencies
// k = kT + p + 128 m, p < 128, m < NM) the phase of observation j is
//   theta_jk = alpha_jp + gamma_jm,  alpha_jp = a_j + p b_j,  gamma_jm = (kT + 128 m) b_j
// (a_j, b_j: the exact 64-bit fixed-point phase of ObsRec, a + k b mod 2^64 turns), so
// with A[p][j] = v_j exp(i alpha_jp) and B[m][j] = exp(i gamma_jm)
//   sum_j v_j exp(i theta_jk) = (A B^T)[p][m],
// and the squared terms follow from the doubled angle, cos^2 = (1 + cos 2theta) / 2,
// cos sin = sin 2theta / 2, with A2 = exp(2i alpha) (times v for the generalized variant)
// and B2 = exp(2i gamma). A does not depend on the frequency tile: it is computed once per
// batch into the operand table (agen_kernel) and bulk-copied into every stage, so the
// kernel's producers compute only the NM x 16 entries of B per K-block.
//
// Each complex product is two real MMAs with N = 2 NM: [Re | Im] = Ar [Br | Bi]^T +
// Ai [-Bi | Br]^T, the right factors being two overlapping row windows of
// Z = [-Bi; Br; Bi]. FP32 accuracy on the FP16 tensor cores comes from the split
// x = hi + lo (hi: x rounded to 11 significant bits, lo = x - hi rounded to FP16),
// a b ~ ah bh + ah bl + al bh: every operand is a cosine or sine, times a weight scaled
// into [-1, 1] by a power of two per object (ObjInfo::tsc0/tsc1) on the A side, so hi + lo
// carries x to about 2^-24 (lo may be subnormal, whose absolute spacing is 2^-24).
//
// The tensor cores round their FP32 accumulations toward zero, which makes the error of
// a long accumulation grow linearly with its length. So a unit's observations are summed
// in passes of kPassKB K-blocks. TMEM holds four slots of accumulators: a phase's first
// pass accumulates into a free slot, which then holds that phase's running sum; each later
// pass accumulates into another free slot, which the epilogue warps fold into the running
// sum with round-to-nearest adds and free at once; after the last pass of a unit they
// compute the powers from the two running sums and free their slots (SlotRing).
//
// One persistent CTA per SM, warp-specialized:
//   warps 0-3   fold and epilogue, one warp per TMEM lane quarter (warp w may access lanes
//               32 (w % 4) ..): power per frequency, periodogram store, per-object maximum;
//   warp 4      TMEM allocation and the MMA issuer (the whole warp runs the loop, one
//               elected lane issues);
//   warp 5      operand loader (one thread): bulk copies of a stage's A matrices from the
//               operand table, and L2 prefetches of the table ahead;
//   warps 6-13  producers: the split FP16 Z matrices of a stage's K-blocks, K-major without
//               swizzle, one sine/cosine per entry, from the K-blocks' frequency steps (read
//               from global memory one stage ahead); warps 6-9 build a stage's first K-block,
//               warps 10-13 its second. They start as soon as the stage is free, in parallel
//               with its bulk copy.
// All hand-offs use mbarriers. Every wait is bounded (MixedArgs::wait_cycles, by default
// about 2 s): on a timeout the kernel records kStatusTimeout in MixedArgs::status, lets its
// issued MMAs drain and its bulk copies land, frees its TMEM and returns.
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "lsgb_device.h"
#include "lsgb_internal.h"

namespace lsgb {

namespace {

constexpr int kTP = 128;        // fine frequency offsets p: A rows, TMEM lanes
constexpr int kTK = 16;         // observations per K-block (the FP16 MMA depth)
constexpr int kPassKB = 8;      // K-blocks accumulated in TMEM before an FP32 fold
constexpr int kLoaderWarp = 5;
constexpr int kProducerWarp0 = 6;
// 14 warps in all, at most 4 per SM sub-partition, so up to 128 registers per thread:
// kEpiPerQuarter epilogue warps per TMEM lane quarter. 1: warps 0-3 and 8 producer warps;
// 2: warps 0-3 and the four after 4 producer warps (the producers then fall behind the
// MMA warp: 2-3% slower)
constexpr int kEpiPerQuarter = 1;
constexpr int kProducerWarps = kEpiPerQuarter == 2 ? 4 : 8;
constexpr int kEpilogueWarp1 = kProducerWarp0 + kProducerWarps;  // second epilogue group
constexpr int kThreads = 32 * (kEpilogueWarp1 + (kEpiPerQuarter == 2 ? 4 : 0));
constexpr int kEpilogueThreads = 128 * kEpiPerQuarter;
constexpr uint32_t kPrefetchKB = 32;   // operand-table K-blocks prefetched into L2 ahead
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kSlots = 4;       // TMEM accumulator slots
constexpr uint32_t kSlotCols = 128;  // TMEM columns of one slot
// Default limit of a bounded wait (MixedArgs::wait_cycles overrides it for the pipeline
// waits); the final waits for the CTA's own MMAs in flight always use it.
constexpr long long kWaitCycles = 1ll << 32;  // ~2 s at 2 GHz
constexpr long long kAbortCopyCycles = 1ll << 21;  // ~1 ms: in-flight copies after an abort

// Per-variant geometry.
template <bool GEN>
struct TGeo {
    static constexpr int NM = GEN ? 32 : 64;       // coarse frequency steps m per unit
    // right-operand groups of phase 0: standard 1 (the weight v0 is on the A side);
    // generalized 2, B1 = v0 e^{i gamma} and B2 = v1 e^{i gamma} against one unweighted A
    static constexpr int G0 = GEN ? 2 : 1;
    static constexpr int N0 = 2 * G0 * NM;         // phase-0 MMA N: [Re groups | Im groups]
    static constexpr int N1 = 2 * NM;              // phase-1 MMA N: [Re | Im]
    static constexpr int W0 = N0;                  // phase-0 accumulator columns
    static constexpr int W1 = N1;                  // phase-1 accumulator columns
    static constexpr int A_BYTES = kTP * kTK * 2;  // one 128 x 16 FP16 matrix
    static constexpr int Z_ROWS = 3 * G0 * NM;     // [-Bi; Br; Bi], each G rows blocks of NM
    static constexpr int Z_BYTES = Z_ROWS * kTK * 2;
    // stage: KPS consecutive K-blocks of one phase, so that the MMA warp waits and
    // commits once per 6 KPS MMAs: their A matrices (re/im, hi/lo; AKB bytes each), then
    // their Z matrices (hi, lo; ZKB bytes each)
    static constexpr int KPS = 2;
    static constexpr int AKB = 4 * A_BYTES;
    static constexpr int ZKB = 2 * Z_BYTES;
    static constexpr int Z_OFF = KPS * AKB;
    static constexpr int STAGE = (Z_OFF + KPS * ZKB + 1023) / 1024 * 1024;
    static constexpr int STAGES = 4;
    static constexpr int TILE = kTP * NM;          // frequencies per unit
    static_assert(kPassKB % KPS == 0, "passes cover whole stages");
    // operand table: phase-major, [phase][K-block of the batch], AKB bytes each, so a
    // stage's K-blocks are one contiguous bulk copy
    // bytes per observation of the steps array: b (standard), b and the two scaled
    // weights (generalized)
    static constexpr int SB = GEN ? 16 : 8;
    static_assert(W0 <= (int)kSlotCols && W1 <= (int)kSlotCols, "TMEM slot too narrow");
    static_assert(kSlots * kSlotCols == kTmemCols, "TMEM layout");
    static_assert(NM % 32 == 0 && kProducerWarps % KPS == 0, "producer mapping");
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Byte offset of element (row r, column k < 16) of a K-major, no-swizzle FP16 operand:
// 8-row x 16-byte core matrices, the two K halves 128 bytes apart (LBO), row groups
// 256 bytes apart (SBO).
__device__ __forceinline__ uint32_t kmaj_off(uint32_t r, uint32_t k) {
    return (r & 7u) * 16u + (r >> 3) * 256u + (k & 7u) * 2u + (k >> 3) * 128u;
}

// Shared-memory matrix descriptor (tcgen05): start address, LBO, SBO in 16-byte units,
// descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)(128u >> 4) << 16) |
           ((uint64_t)(256u >> 4) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16 with FP16 A and B, FP32 accumulator, K-major.
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N) {
    return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Split of an FP32 value (|x| <= 1) into hi with 11 significant bits (exact in FP16 down to
// 2^-14) and lo = x - hi (exact in FP32; its FP16 rounding costs at most 2^-25 absolute):
// hi is x rounded to nearest at the 11th significant bit, by an integer add and mask on its
// bit pattern (a carry into the exponent gives the next power of two, still exact).
__device__ __forceinline__ void vsplit(float x, float &hi, float &lo) {
    hi = __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
    lo = __fsub_rn(x, hi);
}

// Split of two FP32 values x (|x| <= 1, packed f32x2) into FP16 pairs hi = x rounded to
// FP16 and lo = x - hi rounded to FP16 (the subtraction exact in FP32): the accuracy of
// vsplit, with one conversion instruction per pair.
__device__ __forceinline__ void split2(uint64_t x, uint32_t &hi, uint32_t &lo) {
    float a, b;
    unpack2(x, a, b);
    const __half2 h = __floats2half2_rn(a, b);
    const float2 hf = __half22float2(h);
    float ra, rb;
    unpack2(fsub2(x, pack2(hf.x, hf.y)), ra, rb);
    hi = *reinterpret_cast<const uint32_t *>(&h);
    const __half2 l = __floats2half2_rn(ra, rb);
    lo = *reinterpret_cast<const uint32_t *>(&l);
}

// Two FP32 values as one packed FP16 pair (first value in the low half).
__device__ __forceinline__ uint32_t pack_h2(float a, float b) {
    const __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<const uint32_t *>(&h);
}

__device__ __forceinline__ void mbar_init(uint64_t *b, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count));
}
__device__ __forceinline__ void mbar_arrive(uint64_t *b) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)),
                 "r"(bytes)
                 : "memory");
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

// Non-blocking test of the phase of `parity` of barrier b.
__device__ __forceinline__ bool mbar_test_now(uint64_t *b, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{ .reg .pred p; mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2; "
        "selp.u32 %0, 1, 0, p; }"
        : "=r"(done)
        : "r"(smem_u32(b)), "r"(parity)
        : "memory");
    return done != 0;
}

// Waits for the phase of `parity` of barrier b for at most `limit` cycles. Returns false
// (and raises the CTA's abort flag and the launch's status) on a timeout or when another
// role aborted. With the default limit it polls with try_wait (which may suspend the thread
// until the phase completes) and looks at the clock and the abort flag every 256 polls; a
// shorter limit (lsgb_set_wait_limit, for tests) polls without suspending and looks every
// time, so that it is kept to the cycle.
__device__ __noinline__ bool mbar_wait_slow(uint64_t *b, uint32_t parity,
                                            volatile uint32_t *abort, uint32_t *status,
                                            long long limit) {
    const long long t0 = clock64();
    const bool exact = limit < kWaitCycles;
    for (uint32_t it = 1;; ++it) {
        if (exact ? mbar_test_now(b, parity) : mbar_test(b, parity)) return true;
        if (exact || (it & 255u) == 0) {
            if (*abort) return false;
            if (clock64() - t0 > limit) {
                *abort = 1u;
                if (status) atomicOr(status, kStatusTimeout);
                return false;
            }
        }
    }
}
// The completed case inline (one try_wait), the polling loop out of line; a shorter limit
// goes straight to the loop's non-blocking polls.
__device__ __forceinline__ bool mbar_wait(uint64_t *b, uint32_t parity, volatile uint32_t *abort,
                                          uint32_t *status, long long limit) {
    return (limit >= kWaitCycles && mbar_test(b, parity)) ||
           mbar_wait_slow(b, parity, abort, status, limit);
}

__device__ __forceinline__ void bulk_prefetch_l2(const void *src, uint32_t bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(__cvta_generic_to_global(src)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, uint32_t bytes,
                                              uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(__cvta_generic_to_global(src)), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// One complex product's six split-FP16 MMAs into d: a[0..3] = (re hi, re lo, im hi, im lo),
// b[0..3] = (window [Br; Bi] hi, lo, window [-Bi; Br] hi, lo); the first MMA overwrites d
// unless `accumulate`. The two MMAs that share an A matrix read it once: the first fills
// the A collector buffer, the second takes it from there. Called by a whole converged warp:
// elect.sync picks the one lane that issues, so the warp's loop stays uniform and its
// descriptors need no per-lane moves.
__device__ __forceinline__ void mma_cplx6(uint32_t d, const uint64_t (&a)[4],
                                          const uint64_t (&b)[4], uint32_t idesc,
                                          uint32_t accumulate) {
    asm volatile(
        "{ .reg .pred p0, pt, e; elect.sync _|e, 0xffffffff;\n\t"
        "setp.ne.b32 p0, %9, 0; setp.eq.b32 pt, %9, %9;\n\t"
        "@e tcgen05.mma.cta_group::1.kind::f16.collector::a::fill [%0], %1, %5, %10, p0;\n\t"
        "@e tcgen05.mma.cta_group::1.kind::f16.collector::a::lastuse [%0], %1, %6, %10, pt;\n\t"
        "@e tcgen05.mma.cta_group::1.kind::f16 [%0], %2, %5, %10, pt;\n\t"
        "@e tcgen05.mma.cta_group::1.kind::f16.collector::a::fill [%0], %3, %7, %10, pt;\n\t"
        "@e tcgen05.mma.cta_group::1.kind::f16.collector::a::lastuse [%0], %3, %8, %10, pt;\n\t"
        "@e tcgen05.mma.cta_group::1.kind::f16 [%0], %4, %7, %10, pt; }" ::"r"(d),
        "l"(a[0]), "l"(a[1]), "l"(a[2]), "l"(a[3]), "l"(b[0]), "l"(b[1]), "l"(b[2]), "l"(b[3]),
        "r"(accumulate), "r"(idesc)
        : "memory");
}
// Arrives on b once every MMA issued so far has completed (whole converged warp, one lane
// commits).
__device__ __forceinline__ void mma_commit(uint64_t *b) {
    asm volatile(
        "{ .reg .pred e; elect.sync _|e, 0xffffffff;\n\t"
        "@e tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0]; }" ::"r"(
            smem_u32(b))
        : "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

// 8 consecutive accumulator columns of this thread's TMEM lane (asynchronous until
// tmem_wait_ld).
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&r)[8]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
                   "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
}
// 16 consecutive accumulator columns (asynchronous until tmem_wait_ld).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t *r) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
        "%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t *v) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,"
        "%13,%14,%15,%16};" ::"r"(taddr),
        "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]),
        "r"(v[8]), "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]),
        "r"(v[15])
        : "memory");
}
// 32 consecutive accumulator columns (asynchronous until tmem_wait_ld).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
        "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
          "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
          "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_st32(uint32_t taddr, const uint32_t (&v)[32]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,"
        "%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(
            taddr),
        "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]),
        "r"(v[8]), "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]),
        "r"(v[15]), "r"(v[16]), "r"(v[17]), "r"(v[18]), "r"(v[19]), "r"(v[20]), "r"(v[21]),
        "r"(v[22]), "r"(v[23]), "r"(v[24]), "r"(v[25]), "r"(v[26]), "r"(v[27]), "r"(v[28]),
        "r"(v[29]), "r"(v[30]), "r"(v[31])
        : "memory");
}
__device__ __forceinline__ void tmem_wait_ld() {
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_wait_st() {
    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

// Sine and cosine of a 32-bit fixed-point turn count, on the SFU.
__device__ __forceinline__ void turn_sincos(uint32_t hi, float &s, float &c) {
    __sincosf((float)(int32_t)hi * kTwoPiOver2p32f, &s, &c);
}

// Work units: (object, frequency tile) pairs q in queue order, each cut into S = ksplit
// slices of its object's K-blocks when SPLIT (a batch with fewer pairs than SMs); unit
// u = q S + s sums slice s of the object's nkb K-blocks: nkb / S of them, one more for the
// first nkb % S slices. Without SPLIT, unit u is pair u.
template <bool SPLIT>
__device__ __forceinline__ uint32_t ksplit_of(const MixedArgs &a) {
    return SPLIT ? a.ksplit : 1u;
}

struct UnitInfo {
    uint32_t o, tile, n, nkb, kb0;  // n: the object's observations; nkb, kb0: the slice's
    uint32_t u;
    uint64_t row0;
};

template <bool SPLIT>
__device__ __forceinline__ UnitInfo unit_info_of(const MixedArgs &a, uint32_t u, uint32_t o) {
    UnitInfo w;
    w.o = o;
    w.u = u;
    w.row0 = a.objs[o].row0;
    w.n = a.objs[o].n;
    w.kb0 = a.objs[o].kb0;
    w.nkb = (w.n + kTK - 1) / kTK;
    if (!SPLIT) {
        w.tile = u % a.n_tiles;
    } else {
        const uint32_t S = a.ksplit;
        const uint32_t q = u / S, s = u - q * S;
        w.tile = q % a.n_tiles;
        const uint32_t len = w.nkb / S, extra = w.nkb - len * S;
        w.kb0 += len * s + min(s, extra);
        w.nkb = len + (s < extra ? 1u : 0u);
    }
    return w;
}

// The object of unit u.
template <bool SPLIT>
__device__ __forceinline__ uint32_t unit_obj(const MixedArgs &a, uint32_t u) {
    return a.perm[SPLIT ? u / (a.n_tiles * a.ksplit) : u / a.n_tiles];
}

// A CTA's walk over its units b, b + g, b + 2g, ... (b = blockIdx.x, g = gridDim.x) with
// loads issued one unit ahead: next(u) returns unit u's information, loaded during the
// previous call, then issues the object loads of unit u + g (whose object index was read
// one call earlier still) and the object index of unit u + 2g. No role then waits on the
// perm -> objs load chain at a unit boundary.
template <bool SPLIT>
struct UnitWalk {
    UnitInfo nxt;
    uint32_t o1;  // object of the unit after the one in nxt
    __device__ __forceinline__ UnitWalk(const MixedArgs &a, uint32_t units) {
        const uint32_t b = blockIdx.x, g = gridDim.x;
        if (b < units) nxt = unit_info_of<SPLIT>(a, b, unit_obj<SPLIT>(a, b));
        o1 = b + g < units ? unit_obj<SPLIT>(a, b + g) : 0u;
    }
    __device__ __forceinline__ UnitInfo next(const MixedArgs &a, uint32_t u, uint32_t units) {
        const UnitInfo cur = nxt;
        const uint32_t u1 = u + gridDim.x, u2 = u1 + gridDim.x;
        if (u1 < units) nxt = unit_info_of<SPLIT>(a, u1, o1);
        o1 = u2 < units ? unit_obj<SPLIT>(a, u2) : 0u;
        return cur;
    }
};

// Which TMEM slot each pass accumulates into. Free slots are handed out in the order they
// were freed: pop() for every pass in order; a phase's first pass keeps its slot as the
// running sum, a later pass's slot is pushed back once the epilogue has folded it, and the
// unit's two running-sum slots are pushed back after its power pass. The MMA warp and the
// epilogue warps run this same bookkeeping over the same sequence of passes, so they agree
// on every pass's slot without exchanging it. At most two slots are held across a pass
// boundary (the running sums), so a pop always finds one; the slot's barriers alternate
// between its full and empty phases, whose parity is the count of its uses so far.
struct SlotRing {
    uint32_t q = 0xE4u;  // queued free slots, 2 bits each, head in the low bits: 0, 1, 2, 3
    uint32_t n = kSlots;
    uint32_t par = 0u;   // bit s: parity of slot s's uses before the current one
    __device__ __forceinline__ uint32_t pop(uint32_t &parity) {
        const uint32_t s = q & 3u;
        q >>= 2;
        --n;
        parity = (par >> s) & 1u;
        par ^= 1u << s;
        return s;
    }
    __device__ __forceinline__ void push(uint32_t s) {
        q |= s << (2u * n);
        ++n;
    }
};

// The powers of two frequencies (packed pairs) from their raw sums in TMEM order, standard
// (XC, XS, C2, S2) and generalized (C, S, YC, YS, C2, S2), with the object's scales.
template <bool GEN>
struct SumPower {
    uint64_t NN, NN2, FA, FB, S0, S1, NYB, NRM;
    __device__ __forceinline__ SumPower(float nrm, float tsc0, float tsc1, float invw, float ybar,
                                        uint32_t n) {
        const float us0 = 1.0f / tsc0, us1 = 1.0f / tsc1;  // powers of two
        // standard: P = (2P of the raw sums) us0 (us0 nrm / 2), the scale applied in two
        // steps so that us0^2 never forms; generalized: weight-normalized sums
        const float fa = us0, fb = 0.5f * nrm * us0;
        const float s0 = us0 * invw, s1 = us1 * invw;
        const float Nf = (float)n, N2 = Nf * Nf;
        NN = pack2(Nf, Nf);
        NN2 = pack2(N2, N2);
        FA = pack2(fa, fa);
        FB = pack2(fb, fb);
        S0 = pack2(s0, s0);
        S1 = pack2(s1, s1);
        NYB = pack2(-ybar, -ybar);
        NRM = pack2(nrm, nrm);
    }
    __device__ __forceinline__ uint64_t operator()(uint64_t q0, uint64_t q1, uint64_t q2,
                                                   uint64_t q3, uint64_t q4, uint64_t q5) const {
        if (GEN) {
            const uint64_t cb = fmul2(q0, S0), sb = fmul2(q1, S0);
            return fmul2(gen_power_sums2(cb, sb, ffma2(NYB, cb, fmul2(q2, S1)),
                                         ffma2(NYB, sb, fmul2(q3, S1)), fmul2(q4, S0),
                                         fmul2(q5, S0)),
                         NRM);
        }
        return fmul2(fmul2(std_power2_sums2(NN, NN2, q0, q1, q2, q3), FA), FB);
    }
};

// SPLIT: the batch is K-sliced (the epilogue stores raw sums); TOP3: the three best
// frequencies of each object instead of the maximum (launched with a.best_key set).
template <bool GEN, typename OutT, bool SPLIT, bool TOP3>
__global__ void __launch_bounds__(kThreads, 1) tensor_kernel(MixedArgs a) {
    using G = TGeo<GEN>;
    constexpr int S = G::STAGES;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *ring = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    // full: the stage's A matrices have landed (the loader's arrival and bytes) and its Z
    // matrix is written (the producers' arrivals); empty: its MMAs have completed (the
    // loader and the producers wait for it)
    __shared__ __align__(8) uint64_t full_bar[S], empty_bar[S];
    // sfull: a pass's MMAs into the slot have completed; sempty: the epilogue has folded the
    // slot or, for a running sum, finished the unit's power pass
    __shared__ __align__(8) uint64_t sfull_bar[kSlots], sempty_bar[kSlots], drain_bar;
    __shared__ uint32_t s_tmem;
    __shared__ volatile uint32_t s_abort;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t units = a.n_obj * a.n_tiles * ksplit_of<SPLIT>(a);
    const long long lim = a.wait_cycles > 0 ? a.wait_cycles : kWaitCycles;  // pipeline waits

    if (tid == 0) {
        for (int s = 0; s < S; ++s) {
            mbar_init(&full_bar[s], kProducerWarps + 1);  // one arrival per producer warp
            mbar_init(&empty_bar[s], 1);
        }
        for (uint32_t b = 0; b < kSlots; ++b) {
            mbar_init(&sfull_bar[b], 1);
            mbar_init(&sempty_bar[b], kEpilogueThreads / 32);  // one arrival per warp
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

    // Every role walks the same sequence: units b, b + grid, ...; in each unit phase 0
    // (exp(i theta) sums) then phase 1 (exp(2i theta) sums), each over the unit's nkb
    // K-blocks, cut into passes of kPassKB K-blocks.
    if (warp >= kProducerWarp0 && warp < kEpilogueWarp1) {
        // ---------------- producers ----------------
        // Z entry (m, j): B = exp(i (kT + 128 m) b_j) (phase 0) or its square (phase 1).
        // The producer warps come in KPS groups, group hk building K-block hk of every stage.
        // A thread owns row m and the JPT observations j0.. of its K-block: one 2 JPT-byte
        // store per row kind (-Bi, Br, Bi) and half (hi, lo). The lanes of a quarter-warp
        // own 8 consecutive rows of one core matrix, so the stores have no bank conflicts.
        constexpr uint32_t GW = (uint32_t)kProducerWarps / (uint32_t)G::KPS;  // warps a group
        constexpr uint32_t JPT = (uint32_t)G::NM * kTK / (32u * GW);
        constexpr uint32_t JS = kTK / JPT;
        static_assert(JPT == 4 || JPT == 8, "producer mapping");
        const uint32_t pw = (uint32_t)(warp - kProducerWarp0);
        const uint32_t hk = pw / GW;
        // quarter-warp c of the group: observation slice c % JS, row group c / JS
        const uint32_t c = ((uint32_t)lane >> 3) + 4u * (pw % GW);
        const uint32_t m = 8u * (c / JS) + ((uint32_t)lane & 7u);
        const uint32_t j0 = JPT * (c % JS);
        // group g of G: rows g NM + m (-Bi), (G + g) NM + m (Br), (2G + g) NM + m (Bi) of the
        // hi matrix; lo is Z_BYTES further
        const uint32_t zo = (uint32_t)G::Z_OFF + hk * (uint32_t)G::ZKB + kmaj_off(m, j0);
        constexpr uint32_t kRowNM = (uint32_t)G::NM * 32u;  // kmaj_off(r + NM) - kmaj_off(r)
        uint32_t g = 0;
        UnitWalk<SPLIT> walk(a, units);
        // the steps (and weights) of the group's K-block of the next stage, loaded one stage
        // ahead (only for K-blocks that exist)
        constexpr uint32_t NQ4 = JPT * (uint32_t)G::SB / 16u;  // uint4 per thread and stage
        const uint4 *steps = static_cast<const uint4 *>(a.steps);
        uint4 nb[NQ4];
        auto load_b = [&](uint32_t kbg) {
#pragma unroll
            for (uint32_t h = 0; h < NQ4; ++h)
                nb[h] = __ldg(steps + (kbg * kTK + j0) * (uint32_t)G::SB / 16u + h);
        };
        if (blockIdx.x < units && hk < walk.nxt.nkb) load_b(walk.nxt.kb0 + hk);
        // the warp's lanes leave together: the abort flag as lane 0 reads it, and every
        // wait's outcome voted over the warp
        for (uint32_t u = blockIdx.x; u < units && __shfl_sync(0xffffffffu, s_abort, 0) == 0u;
             u += gridDim.x) {
            const UnitInfo w = walk.next(a, u, units);
            const uint32_t k = w.tile * (uint32_t)G::TILE + 128u * m;
            const uint32_t nsp = (w.nkb + (uint32_t)G::KPS - 1u) / (uint32_t)G::KPS;  // a phase
            bool ok = true;
            for (uint32_t st = 0; st < 2u * nsp; ++st) {
                const bool ph1 = st >= nsp;
                const uint32_t kb = (ph1 ? st - nsp : st) * (uint32_t)G::KPS + hk;
                const bool mine = kb < w.nkb;
                uint4 cb[NQ4];
#pragma unroll
                for (uint32_t h = 0; h < NQ4; ++h) cb[h] = nb[h];
                // the group's K-block of the next stage: this unit's, or the next unit's first
                {
                    const uint32_t st1 = st + 1u;
                    if (st1 < 2u * nsp) {
                        const uint32_t kb1 = (st1 >= nsp ? st1 - nsp : st1) * (uint32_t)G::KPS + hk;
                        if (kb1 < w.nkb) load_b(w.kb0 + kb1);
                    } else if (u + gridDim.x < units && hk < walk.nxt.nkb) {
                        load_b(walk.nxt.kb0 + hk);
                    }
                }
                const uint32_t s = g % S, us = g / S;
                if (!__all_sync(0xffffffffu,
                                mbar_wait(&empty_bar[s], (us & 1u) ^ 1u, &s_abort, a.status, lim))) {
                    ok = false;
                    break;
                }
                if (mine) {
                    unsigned char *zh = ring + (size_t)s * G::STAGE + zo;
                    auto put = [&](unsigned char *dst, const uint32_t (&v)[JPT / 2]) {
                        if constexpr (JPT == 8)
                            *reinterpret_cast<uint4 *>(dst) = make_uint4(v[0], v[1], v[2], v[3]);
                        else
                            *reinterpret_cast<uint2 *>(dst) = make_uint2(v[0], v[1]);
                    };
                    // the observations in pairs (j, j + 1): cos / sin of k b_j (or of twice
                    // it), times the group weights, split and packed as FP16 pairs
                    const uint32_t ng = (GEN && !ph1) ? 2u : 1u;
                    uint32_t pch[2][JPT / 2], pcl[2][JPT / 2], psh[2][JPT / 2], psl[2][JPT / 2];
#pragma unroll
                    for (uint32_t h = 0; h < JPT / 2; ++h) {
                        uint32_t bl[2], bh[2];
                        float wt[2][2];  // [observation][group]
                        if constexpr (GEN) {
                            const uint4 q0 = cb[2 * h], q1 = cb[2 * h + 1];
                            bl[0] = q0.x; bh[0] = q0.y; bl[1] = q1.x; bh[1] = q1.y;
                            wt[0][0] = __uint_as_float(q0.z); wt[0][1] = __uint_as_float(q0.w);
                            wt[1][0] = __uint_as_float(q1.z); wt[1][1] = __uint_as_float(q1.w);
                        } else {
                            bl[0] = cb[h].x; bh[0] = cb[h].y; bl[1] = cb[h].z; bh[1] = cb[h].w;
                            wt[0][0] = wt[0][1] = wt[1][0] = wt[1][1] = 1.0f;
                        }
                        float sn[2], cs[2];
#pragma unroll
                        for (int q = 0; q < 2; ++q) {
                            // hi 32 bits of k b mod 2^64: (k b_lo) >> 32 plus k b_hi
                            const uint32_t t32 = __umulhi(k, bl[q]) + k * bh[q];
                            // phase 1: the doubled angle is the doubled turn count (mod 2^32)
                            turn_sincos(ph1 ? t32 << 1 : t32, sn[q], cs[q]);
                        }
                        // the two observations as packed pairs
                        const uint64_t C = pack2(cs[0], cs[1]), Sn = pack2(sn[0], sn[1]);
#pragma unroll
                        for (int gi = 0; gi < (GEN ? 2 : 1); ++gi) {
                            if (gi >= (int)ng) break;  // phase 1 has one group
                            uint64_t Cg = C, Sg = Sn;
                            if (GEN) {
                                const uint64_t W = pack2(wt[0][gi], wt[1][gi]);
                                Cg = fmul2(C, W);
                                Sg = fmul2(Sn, W);
                            }
                            split2(Cg, pch[gi][h], pcl[gi][h]);
                            split2(Sg, psh[gi][h], psl[gi][h]);
                        }
                    }
#pragma unroll
                    for (uint32_t gi = 0; gi < (GEN ? 2u : 1u); ++gi) {
                        if (gi >= ng) break;
                        // -x = (-hi) + (-lo) exactly: the sign bits of both FP16 halves flipped
                        uint32_t nsh[JPT / 2], nsl[JPT / 2];
#pragma unroll
                        for (uint32_t h = 0; h < JPT / 2; ++h) {
                            nsh[h] = psh[gi][h] ^ 0x80008000u;
                            nsl[h] = psl[gi][h] ^ 0x80008000u;
                        }
                        unsigned char *zg = zh + gi * kRowNM;
                        put(zg, nsh);
                        put(zg + G::Z_BYTES, nsl);
                        put(zg + ng * kRowNM, pch[gi]);
                        put(zg + ng * kRowNM + G::Z_BYTES, pcl[gi]);
                        put(zg + 2u * ng * kRowNM, psh[gi]);
                        put(zg + 2u * ng * kRowNM + G::Z_BYTES, psl[gi]);
                    }
                }
                // generic-proxy stores -> the MMA's async-proxy reads; then one arrival for
                // the warp (also when the stage has no K-block for its group), after all its
                // lanes have fenced
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncwarp();
                if (lane == 0) mbar_arrive(&full_bar[s]);
                ++g;
            }
            if (!ok) break;
        }
    } else if (warp == kLoaderWarp) {
        // ---------------- operand loader ----------------
        if (lane == 0) {
            const unsigned char *tab = static_cast<const unsigned char *>(a.optab);
            uint32_t g = 0;
            UnitWalk<SPLIT> walk(a, units);
            const uint64_t tph = (uint64_t)a.total_kb * G::AKB;  // phase stride of the table
            auto prefetch = [&](uint32_t kbg, uint32_t n) {  // K-blocks kbg.. of both phases
                bulk_prefetch_l2(tab + (uint64_t)kbg * G::AKB, n * (uint32_t)G::AKB);
                bulk_prefetch_l2(tab + tph + (uint64_t)kbg * G::AKB, n * (uint32_t)G::AKB);
            };
            if (blockIdx.x < units) prefetch(walk.nxt.kb0, min(walk.nxt.nkb, kPrefetchKB));
            for (uint32_t u = blockIdx.x; u < units && !s_abort; u += gridDim.x) {
                const UnitInfo w = walk.next(a, u, units);
                // L2: the next unit's first K-blocks now, this unit's further ones as the
                // phase-0 pass reaches them
                if (u + gridDim.x < units) prefetch(walk.nxt.kb0, min(walk.nxt.nkb, kPrefetchKB));
                bool ok = true;
                for (uint32_t ph = 0; ph < 2u && ok; ++ph) {
                    for (uint32_t kb = 0; kb < w.nkb; kb += G::KPS, ++g) {
                        const uint32_t s = g % S, us = g / S;
                        const uint32_t cnt = min((uint32_t)G::KPS, w.nkb - kb);
                        if (!ph && kb + kPrefetchKB < w.nkb)
                            prefetch(w.kb0 + kb + kPrefetchKB, min(cnt, w.nkb - kb - kPrefetchKB));
                        if (!mbar_wait(&empty_bar[s], (us & 1u) ^ 1u, &s_abort, a.status, lim)) {
                            ok = false;
                            break;
                        }
                        const uint32_t bytes = cnt * (uint32_t)G::AKB;
                        mbar_expect_tx(&full_bar[s], bytes);
                        bulk_copy_g2s(ring + (size_t)s * G::STAGE,
                                      tab + ph * tph + (uint64_t)(w.kb0 + kb) * G::AKB, bytes,
                                      &full_bar[s]);
                    }
                }
                if (!ok) break;
            }
        }
        __syncwarp();
    } else if (warp == 4) {
        // ---------------- MMA issuer ----------------
        // The whole warp walks the loop (every value in it is warp-uniform and every wait
        // ends in a vote); one elected lane issues the MMAs and commits.
        {
            constexpr uint32_t idesc0 = idesc_f16(kTP, G::N0), idesc1 = idesc_f16(kTP, G::N1);
            // descriptors: the upper 32 bits are the same for every operand; the address
            // field of the lower ones is linear in the shared address (16-byte units; shared
            // addresses stay below 2^18, so the 14-bit field never carries)
            const uint64_t sdb = sdesc(smem_u32(ring));
            const uint32_t dhi = (uint32_t)(sdb >> 32), dlo0 = (uint32_t)sdb;
            auto dsc = [&](uint32_t lo, uint32_t off) -> uint64_t {
                return ((uint64_t)dhi << 32) | (uint64_t)(lo + (off >> 4));
            };
            uint32_t s = 0, sph = 0;  // stage slot and its phase parity
            uint32_t dlo = dlo0;      // lower descriptor half of slot s
            bool ok = true;
            SlotRing ring;
            uint32_t rsum[2] = {0u, 0u};  // the unit's running-sum slots
            UnitWalk<SPLIT> walk(a, units);
            for (uint32_t u = blockIdx.x; u < units && ok; u += gridDim.x) {
                const UnitInfo w = walk.next(a, u, units);  // nkb >= 1: no slice is empty
                for (uint32_t ph = 0; ph < 2 && ok; ++ph) {
                    for (uint32_t kb0 = 0; kb0 < w.nkb && ok; kb0 += kPassKB) {
                        uint32_t sp;
                        const uint32_t slot = ring.pop(sp);
                        if (!__all_sync(0xffffffffu, mbar_wait(&sempty_bar[slot], sp ^ 1u,
                                                               &s_abort, a.status, lim))) {
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                        const uint32_t d0 = tmem + slot * kSlotCols;
                        const uint32_t kb1 = min(w.nkb, kb0 + (uint32_t)kPassKB);
                        // windows of Z = [-Bi; Br; Bi] (blocks of G NM rows): [Br; Bi] at
                        // row G NM, [-Bi; Br] at row 0
                        const uint32_t gnm = ph ? 1u : (uint32_t)G::G0;
                        const uint32_t wre = gnm * (uint32_t)G::NM * 32u;
                        const uint32_t idesc = ph ? idesc1 : idesc0;
                        for (uint32_t kb = kb0; kb < kb1; kb += G::KPS) {  // one stage
                            if (!__all_sync(0xffffffffu,
                                            mbar_wait(&full_bar[s], sph, &s_abort, a.status, lim))) {
                                ok = false;
                                break;
                            }
                            tc_fence_after();
                            const uint32_t cnt = min((uint32_t)G::KPS, kb1 - kb);
                            for (uint32_t kbi = 0; kbi < cnt; ++kbi) {
                                const uint32_t acc0 = kb + kbi > kb0 ? 1u : 0u;
                                const uint32_t ao = kbi * (uint32_t)G::AKB;
                                const uint32_t zo = (uint32_t)G::Z_OFF + kbi * (uint32_t)G::ZKB;
                                const uint64_t bd[4] = {dsc(dlo, zo + wre),
                                                        dsc(dlo, zo + wre + G::Z_BYTES),
                                                        dsc(dlo, zo), dsc(dlo, zo + G::Z_BYTES)};
                                // one complex product: D += A (re, im) x Z window, split
                                // FP16: [XC | XS], [C C' | S S'] (generalized phase 0), or
                                // [C2 | S2]
                                const uint64_t ad[4] = {dsc(dlo, ao), dsc(dlo, ao + G::A_BYTES),
                                                        dsc(dlo, ao + 2 * G::A_BYTES),
                                                        dsc(dlo, ao + 3 * G::A_BYTES)};
                                mma_cplx6(d0, ad, bd, idesc, acc0);
                            }
                            mma_commit(&empty_bar[s]);
                            if (++s == (uint32_t)S) {
                                s = 0;
                                sph ^= 1u;
                                dlo = dlo0;
                            } else {
                                dlo += (uint32_t)G::STAGE >> 4;
                            }
                        }
                        if (ok) mma_commit(&sfull_bar[slot]);
                        // the epilogue's side of the bookkeeping
                        if (kb0 == 0) rsum[ph] = slot;
                        else ring.push(slot);
                    }
                }
                ring.push(rsum[0]);
                ring.push(rsum[1]);
            }
            // every issued MMA has completed before TMEM is released
            mma_commit(&drain_bar);
            const long long t0 = clock64();
            while (!mbar_test(&drain_bar, 0u) && clock64() - t0 < kWaitCycles) {
            }
        }
        __syncwarp();
    } else {
        // ---------------- fold and epilogue ----------------
        // warp w may access TMEM lanes 32 (w % 4) ..; with two warps per lane quarter they
        // split the coarse steps: warp half eh owns m in [eh SPAN, (eh+1) SPAN), i.e. the same
        // part of every NM-column quantity block, in the folds and in the power pass, so a
        // warp only ever reads running sums it wrote itself
        const uint32_t eq = (uint32_t)warp & 3u;
        const uint32_t eh = (kEpiPerQuarter == 2 && warp >= kEpilogueWarp1) ? 1u : 0u;
        // columns of each NM-column quantity block this warp folds and reads: SPAN from eh SPAN
        constexpr uint32_t SPAN = (uint32_t)G::NM / (uint32_t)kEpiPerQuarter;
        const uint32_t pl = eq * 32u + (uint32_t)lane;
        const uint32_t lane_base = (eq * 32u) << 16;
        bool ok = true;
        SlotRing ring;
        UnitWalk<SPLIT> walk(a, units);
        for (uint32_t u = blockIdx.x; u < units && ok; u += gridDim.x) {
            const UnitInfo w = walk.next(a, u, units);
            // the object's fields for the power pass, loaded before the folds
            const ObjInfo &ob = a.objs[w.o];
            const float nrm = ob.norm32, tsc0 = ob.tsc0, tsc1 = ob.tsc1;
            const float invw = ob.invw32, ybar = ob.ybar32;
            const uint32_t npass = (w.nkb + kPassKB - 1) / kPassKB;
            uint32_t rsum[2] = {0u, 0u};  // the running-sum slots of the two phases
            for (uint32_t ph = 0; ph < 2 && ok; ++ph) {
                const uint32_t wcols = ph ? (uint32_t)G::W1 : (uint32_t)G::W0;
                for (uint32_t pi = 0; pi < npass; ++pi) {
                    uint32_t sp;
                    const uint32_t slot = ring.pop(sp);
                    if (!__all_sync(0xffffffffu, mbar_wait(&sfull_bar[slot], sp, &s_abort, a.status, lim))) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    // the first pass's slot becomes the running sum as it is
                    if (pi == 0) {
                        rsum[ph] = slot;
                        continue;
                    }
                    const uint32_t run = tmem + lane_base + rsum[ph] * kSlotCols;
                    const uint32_t part = tmem + lane_base + slot * kSlotCols;
                    // fold: running += partial over this warp's part of each quantity block;
                    // the slot is freed as soon as the quarter's warps have read it
                    constexpr uint32_t HALF = SPAN >= 32u ? 32u : 16u;  // columns per round
                    static_assert(SPAN % HALF == 0, "fold rounds of 32 or 16 columns");
#pragma unroll 1
                    for (uint32_t blk = 0; blk < wcols; blk += G::NM) {  // quantity blocks
#pragma unroll 1
                    for (uint32_t cc = 0; cc < SPAN; cc += HALF) {
                        const uint32_t c = blk + SPAN * eh + cc;
                        uint32_t x[HALF], y[HALF];
                        if (HALF == 32) {
                            tmem_ld32(part + c, *reinterpret_cast<uint32_t(*)[32]>(x));
                            tmem_ld32(run + c, *reinterpret_cast<uint32_t(*)[32]>(y));
                        } else {
                            tmem_ld16(part + c, x);
                            tmem_ld16(run + c, y);
                        }
                        tmem_wait_ld();
#pragma unroll
                        for (uint32_t i = 0; i < HALF; i += 2) {
                            const uint64_t sum =
                                fadd2(pack2(__uint_as_float(x[i]), __uint_as_float(x[i + 1])),
                                      pack2(__uint_as_float(y[i]), __uint_as_float(y[i + 1])));
                            float s0f, s1f;
                            unpack2(sum, s0f, s1f);
                            x[i] = __float_as_uint(s0f);
                            x[i + 1] = __float_as_uint(s1f);
                        }
                        if (HALF == 32)
                            tmem_st32(run + c, *reinterpret_cast<const uint32_t(*)[32]>(x));
                        else
                            tmem_st16(run + c, x);
                    }
                    }
                    tmem_wait_st();
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&sempty_bar[slot]);
                    ring.push(slot);
                }
            }
            if (!ok) break;
            // power from the running sums of both phases
            const uint32_t run1 = tmem + lane_base + rsum[0] * kSlotCols;
            const uint32_t run2 = tmem + lane_base + rsum[1] * kSlotCols;
            const uint32_t kT = w.tile * (uint32_t)G::TILE;
            const SumPower<GEN> power2(nrm, tsc0, tsc1, invw, ybar, w.n);
            const uint64_t out0 = (uint64_t)w.o * a.n_freq;
            float bp = 0.0f;
            uint32_t bk = 0xffffffffu;
            if (w.tile == 0 && pl == 0 && eh == 0) bk = 0;  // the reference's (power 0, index 0) start
            // split units store their raw sums for ksum_kernel instead of powers
            constexpr bool split = SPLIT;
            constexpr bool top3 = TOP3 && !SPLIT;
            static_assert(!top3 || kEpiPerQuarter == 1, "tile_key3 holds one triple per quarter");
            // top three: the object's floor, a key no larger than its third best so far (the
            // largest third key any warp has stored): whatever is not above it is dropped
            const unsigned long long g3 =
                top3 ? *(volatile unsigned long long *)(a.best_key + 3ull * w.o + 2) : 0ull;
            Top3 t3;
            t3.seed(g3);
            // quantities: phase 0 groups (re, im) then phase 1 (re, im)
            constexpr int NQ = GEN ? 6 : 4;
            // frequencies per chunk: 16 for the standard variant (eight independent packed
            // chains per chunk), 8 for the generalized one (six quantities per frequency)
            constexpr int CHK = GEN ? 8 : 16;
            static_assert(SPAN % CHK == 0, "whole chunks per warp");
            uint32_t x[NQ][CHK];
            auto load_chunk = [&](int m0) {
#pragma unroll
                for (int k = 0; k < NQ; ++k) {
                    const bool p1 = k >= NQ - 2;
                    const int kk = p1 ? k - (NQ - 2) : k;
                    // phase 0: group g = kk / 2 of G0, re / im = kk % 2 in [Re groups | Im groups]
                    const uint32_t gq = p1 ? 1u : (uint32_t)G::G0;
                    const uint32_t col = (uint32_t)(kk & 1) * gq * G::NM + (uint32_t)(kk >> 1) * G::NM + (uint32_t)m0;
                    if constexpr (CHK == 16) tmem_ld16((p1 ? run2 : run1) + col, x[k]);
                    else tmem_ld8((p1 ? run2 : run1) + col, *reinterpret_cast<uint32_t(*)[8]>(x[k]));
                }
            };
            const int mbeg = (int)(eh * SPAN), mend = mbeg + (int)SPAN;
#pragma unroll 1
            for (int m0 = mbeg; m0 < mend; m0 += CHK) {
                load_chunk(m0);
                tmem_wait_ld();
                if constexpr (split) {
                    // [unit][quantity][p + 128 m]: a warp's stores are 128 contiguous bytes
                    float *dst = a.partial + (uint64_t)w.u * (uint32_t)(NQ * G::TILE) + pl +
                                 (uint32_t)kTP * (uint32_t)m0;
#pragma unroll
                    for (int k = 0; k < NQ; ++k)
#pragma unroll
                        for (int i = 0; i < CHK; ++i)
                            __stcg(dst + (uint32_t)k * (uint32_t)G::TILE + (uint32_t)kTP * (uint32_t)i,
                                   __uint_as_float(x[k][i]));
                    continue;
                }
                float q[NQ][CHK];
#pragma unroll
                for (int k = 0; k < NQ; ++k)
#pragma unroll
                    for (int i = 0; i < CHK; ++i) q[k][i] = __uint_as_float(x[k][i]);
                // the chunk's powers first, branch-free and in packed pairs of frequencies, so
                // that their chains interleave
                float P[CHK];
                auto power_at = [&](int i) {
                    if ((i & 1) != 0) return;
                    auto pq = [&](int k) { return pack2(q[k][i], q[k][i + 1]); };
                    unpack2(power2(pq(0), pq(1), pq(2), pq(3), pq(GEN ? 4 : 0), pq(GEN ? 5 : 0)),
                            P[i], P[i + 1]);
                };
#pragma unroll
                for (int i = 0; i < CHK; ++i) power_at(i);
                // a thread visits its frequencies in increasing k, so a strictly larger power
                // is the only way to displace its current best (ties keep the lower index, as
                // the reference's argmax does)
                const uint32_t k0 = kT + pl + (uint32_t)kTP * (uint32_t)m0;
                if (k0 + (uint32_t)kTP * (uint32_t)(CHK - 1) < a.n_freq) {  // the whole chunk is on the grid
                    if (a.pgram) {
#pragma unroll
                        for (int i = 0; i < CHK; ++i) store_out<OutT>(a.pgram, out0 + k0 + (uint32_t)kTP * (uint32_t)i, P[i]);
                    }
                    if constexpr (top3) {
                        t3.offer_run(P, k0, (uint32_t)kTP);
                    } else {
#pragma unroll
                        for (int i = 0; i < CHK; ++i)
                            if (P[i] > bp) { bp = P[i]; bk = k0 + (uint32_t)kTP * (uint32_t)i; }
                    }
                } else {
#pragma unroll
                    for (int i = 0; i < CHK; ++i) {
                        const uint32_t k = k0 + (uint32_t)kTP * (uint32_t)i;
                        if (k < a.n_freq) {
                            if (a.pgram) store_out<OutT>(a.pgram, out0 + k, P[i]);
                            if constexpr (top3) t3.offer(P[i], k);
                            else if (P[i] > bp) { bp = P[i]; bk = k; }
                        }
                    }
                }
            }
            // every load of the running sums has completed: free their slots
            tc_fence_before();
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(&sempty_bar[rsum[0]]);
                mbar_arrive(&sempty_bar[rsum[1]]);
            }
            ring.push(rsum[0]);
            ring.push(rsum[1]);
            if constexpr (top3) {
                // the warp's keys above the floor (at most three), stored for
                // top3_merge_kernel; the warp's third key then raises the floor (a reduction
                // without a return value: no round trip on this warp's path). A warp with
                // nothing above the floor leaves its zeroed entries.
                if (__any_sync(0xffffffffu, t3.t0 > g3)) {
                    t3.warp_merge();
                    if (lane < 3) {
                        const unsigned long long key = lane == 0 ? t3.t0 : lane == 1 ? t3.t1 : t3.t2;
                        a.tile_key3[(((uint64_t)w.o * a.n_tiles + w.tile) * 4u + eq) * 3u + lane] =
                            key > g3 ? key : 0ull;
                    }
                    if (lane == 0 && t3.t2 > g3) atomicMax(a.best_key + 3ull * w.o + 2, t3.t2);
                }
            } else if (!split && a.best_key) {
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) {
                    const float op = __shfl_xor_sync(0xffffffffu, bp, off);
                    const uint32_t ok2 = __shfl_xor_sync(0xffffffffu, bk, off);
                    if (better(op, ok2, bp, bk)) { bp = op; bk = ok2; }
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
    // After an abort some stages are never consumed, and a bulk copy into one of them may
    // still be in flight: the CTA must not exit (and give its shared memory up) before such
    // copies have landed. They are not observable on their own (a stage's full barrier also
    // needs the producers' arrivals), so one thread keeps the CTA for a fixed
    // kAbortCopyCycles, about 1 ms, far beyond the few microseconds a copy of two
    // operand-table K-blocks takes. (The MMA warp has already waited for its MMAs.)
    if (s_abort && tid == 0) {
        const long long t0 = clock64();
        while (clock64() - t0 < kAbortCopyCycles) {
        }
    }
    if (warp == 4) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(kTmemCols)
                     : "memory");
    }
}

// The finishing pass of split units: for each (object, tile) pair q and frequency of the
// tile, the S slices' raw sums added in FP32 in slice order, then the power, the
// periodogram store and the object's best frequencies as the tensor kernel's epilogue
// forms them. A thread takes two consecutive frequencies of one tile.
constexpr uint32_t kKsumFreqs = 512;  // frequencies per CTA (256 threads)

template <bool GEN, typename OutT>
__global__ void __launch_bounds__(256) ksum_kernel(MixedArgs a) {
    using G = TGeo<GEN>;
    constexpr int NQ = GEN ? 6 : 4;
    constexpr uint32_t CPT = (uint32_t)G::TILE / kKsumFreqs;  // CTAs per tile
    const uint32_t S = a.ksplit;
    const uint32_t q = blockIdx.x / CPT;
    const uint32_t f = (blockIdx.x - q * CPT) * kKsumFreqs + 2u * threadIdx.x;
    const uint32_t o = a.perm[q / a.n_tiles];
    const uint32_t k0 = (q % a.n_tiles) * (uint32_t)G::TILE + f;
    const ObjInfo &ob = a.objs[o];
    const SumPower<GEN> power2(ob.norm32, ob.tsc0, ob.tsc1, ob.invw32, ob.ybar32, ob.n);
    float2 v[NQ];
#pragma unroll
    for (int k = 0; k < NQ; ++k) v[k] = make_float2(0.0f, 0.0f);
    const float *src = a.partial + (uint64_t)q * S * (uint32_t)(NQ * G::TILE) + f;
    for (uint32_t s = 0; s < S; ++s, src += NQ * G::TILE) {
#pragma unroll
        for (int k = 0; k < NQ; ++k) {
            const float2 x = __ldcg(reinterpret_cast<const float2 *>(src + k * G::TILE));
            v[k].x += x.x;
            v[k].y += x.y;
        }
    }
    auto pv = [&](int k) { return pack2(v[k].x, v[k].y); };
    float P[2];
    unpack2(power2(pv(0), pv(1), pv(2), pv(3), pv(GEN ? 4 : 0), pv(GEN ? 5 : 0)), P[0], P[1]);
    const uint64_t out0 = (uint64_t)o * a.n_freq;
    const bool top3 = a.top == 3u && a.best_key;
    const unsigned long long g3 =
        top3 ? *(volatile unsigned long long *)(a.best_key + 3ull * o + 2) : 0ull;
    Top3 t3;
    t3.seed(g3);
    float bp = 0.0f;
    uint32_t bk = 0xffffffffu;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        const uint32_t k = k0 + (uint32_t)i;
        if (k < a.n_freq) {
            if (a.pgram) store_out<OutT>(a.pgram, out0 + k, P[i]);
            if (top3) t3.offer(P[i], k);
            else if (P[i] > bp) { bp = P[i]; bk = k; }
        }
    }
    if (top3) {
        if (__any_sync(0xffffffffu, t3.t0 > g3)) t3.warp_merge();
        if ((threadIdx.x & 31u) == 0 && t3.t0 > g3) {
            unsigned long long *slots = a.best_key + 3ull * o;
            top3_insert(slots, t3.t0);
            top3_insert(slots, t3.t1);
            top3_insert(slots, t3.t2);
        }
    } else if (a.best_key) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const float op = __shfl_xor_sync(0xffffffffu, bp, off);
            const uint32_t ok2 = __shfl_xor_sync(0xffffffffu, bk, off);
            if (better(op, ok2, bp, bk)) { bp = op; bk = ok2; }
        }
        if ((threadIdx.x & 31u) == 0 && bp > 0.0f)
            atomicMax(a.best_key + o, rank_key(bp, bk));
    }
}

// The top three of each object from its tiles' warp triples (tile_key3): one warp per
// object offers the 12 n_tiles keys (distinct but for zeros) and merges its lanes' triples.
// Every key of the object's top three is there: it is above every floor a warp saw (a floor
// is some warp's third key, no larger than the object's third), and its own warp stored it.
__global__ void __launch_bounds__(256) top3_merge_kernel(const unsigned long long *tile_key3,
                                                         uint32_t n_obj, uint32_t n_tiles,
                                                         unsigned long long *best_key) {
    const uint32_t o = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t lane = threadIdx.x & 31u;
    if (o >= n_obj) return;  // warp-uniform
    const unsigned long long *src = tile_key3 + (uint64_t)o * n_tiles * 12u;
    const uint32_t n = n_tiles * 12u;
    Top3 t3;
    for (uint32_t i = lane; i < n; i += 32u) {
        const unsigned long long key = src[i];
        if (key) t3.offer(key);
    }
    t3.warp_merge();
    if (lane < 3) best_key[3ull * o + lane] = lane == 0 ? t3.t0 : lane == 1 ? t3.t1 : t3.t2;
}

// The operand table: one CTA per K-block builds its A matrices of both phases for p < 128,
// split FP16 (re / im, hi / lo) in the layout the tensor kernel stages, from one sine /
// cosine per (p, observation) (phase 1 by the double-angle formulas), and writes the
// K-block's steps array entries.
//   standard:    phase 0 v0 tsc0 exp(i alpha), phase 1 exp(2i alpha); steps {b}
//   generalized: phase 0 exp(i alpha),         phase 1 exp(2i alpha); steps {b, v0 tsc0,
//                v1 tsc1} (the weights go on the right operand, built by the producers)
// with alpha = a + p b in 64-bit fixed point. Observations past the object's end get zero
// A entries (and zero steps and weights), so they add nothing to any product. A thread's
// four observations of one row p are 8 contiguous bytes of a core matrix, and a warp's
// eight rows two whole 128-byte lines, so the entries go straight to global memory.
template <bool GEN>
__global__ void __launch_bounds__(256) agen_kernel(MixedArgs a, uint32_t total_kb) {
    using G = TGeo<GEN>;
    const uint32_t kbg = blockIdx.x;
    if (kbg >= total_kb) return;
    const ObjInfo &ob = a.objs[a.kb_obj[kbg]];  // the object of this K-block
    const uint32_t kb = kbg - ob.kb0;
    const uint32_t cnt = min((uint32_t)kTK, ob.n - kb * kTK);
    const ObsRec *rec = static_cast<const ObsRec *>(a.rec) + ob.row0 + (uint64_t)kb * kTK;
    const float sc0 = ob.tsc0, sc1 = ob.tsc1;
    unsigned char *tab = static_cast<unsigned char *>(const_cast<void *>(a.optab));
    unsigned char *const dst[2] = {tab + (uint64_t)kbg * G::AKB,
                                   tab + ((uint64_t)total_kb + kbg) * G::AKB};
    for (uint32_t e = threadIdx.x; e < (uint32_t)kTP * (kTK / 4); e += blockDim.x) {
        const uint32_t p = e >> 2, j0 = 4u * (e & 3u);
        float x[2][2][4];  // [phase][re / im][observation]
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint32_t j = j0 + (uint32_t)q;
            const ObsRec &r = rec[min(j, cnt - 1u)];
            const uint64_t pa = (uint64_t)p * r.b_lo + (((uint64_t)r.a_hi << 32) | r.a_lo);
            const uint32_t t32 = (uint32_t)(pa >> 32) + p * r.b_hi;
            float sn, cs;
            turn_sincos(t32, sn, cs);
            const float mk = j < cnt ? 1.0f : 0.0f;
            const float v = (GEN ? 1.0f : r.v0 * sc0) * mk;
            x[0][0][q] = v * cs;
            x[0][1][q] = v * sn;
            x[1][0][q] = mk * fmaf(cs, cs, -sn * sn);
            x[1][1][q] = mk * (2.0f * cs * sn);
        }
#pragma unroll
        for (int ph = 0; ph < 2; ++ph)
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                float h4[4], l4[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) vsplit(x[ph][c][q], h4[q], l4[q]);
                unsigned char *base = dst[ph] + 2u * (uint32_t)c * G::A_BYTES + kmaj_off(p, j0);
                *reinterpret_cast<uint2 *>(base) =
                    make_uint2(pack_h2(h4[0], h4[1]), pack_h2(h4[2], h4[3]));
                *reinterpret_cast<uint2 *>(base + G::A_BYTES) =
                    make_uint2(pack_h2(l4[0], l4[1]), pack_h2(l4[2], l4[3]));
            }
    }
    if (threadIdx.x < (uint32_t)kTK) {
        const uint32_t j = threadIdx.x;
        const bool in = j < cnt;
        const uint32_t b_lo = in ? rec[j].b_lo : 0u, b_hi = in ? rec[j].b_hi : 0u;
        unsigned char *sdst = static_cast<unsigned char *>(const_cast<void *>(a.steps)) +
                              ((uint64_t)kbg * kTK + j) * (uint32_t)G::SB;
        if (GEN)
            *reinterpret_cast<uint4 *>(sdst) =
                make_uint4(b_lo, b_hi, __float_as_uint(in ? rec[j].v0 * sc0 : 0.0f),
                           __float_as_uint(in ? rec[j].v1 * sc1 : 0.0f));
        else
            *reinterpret_cast<uint2 *>(sdst) = make_uint2(b_lo, b_hi);
    }
}

template <bool GEN>
size_t tensor_smem() {
    return (size_t)TGeo<GEN>::STAGES * TGeo<GEN>::STAGE + 1024;
}

template <bool GEN, typename OutT>
cudaError_t launch_t(const MixedArgs &a, int grid, cudaStream_t st) {
    void (*k)(MixedArgs) = tensor_kernel<GEN, OutT, false, false>;
    if (a.ksplit > 1u) k = tensor_kernel<GEN, OutT, true, false>;  // ksum_kernel finishes
    else if (a.top == 3u && a.best_key) k = tensor_kernel<GEN, OutT, false, true>;
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

size_t tensor_step_bytes(int variant) {
    return (size_t)kTK * (size_t)(variant ? TGeo<true>::SB : TGeo<false>::SB);
}

size_t tensor_optab_bytes(int variant, uint64_t total_kb) {
    return (size_t)total_kb *
           (2u * (size_t)(variant ? TGeo<true>::AKB : TGeo<false>::AKB) + tensor_step_bytes(variant));
}

cudaError_t launch_tensor_optab(int variant, const MixedArgs &a, uint64_t total_kb, cudaStream_t st) {
    if (total_kb == 0) return cudaSuccess;
    const uint64_t blocks = total_kb;
    if (blocks > 0x7fffffffull) return cudaErrorInvalidValue;
    if (variant == 0)
        agen_kernel<false><<<(unsigned)blocks, 256, 0, st>>>(a, (uint32_t)total_kb);
    else
        agen_kernel<true><<<(unsigned)blocks, 256, 0, st>>>(a, (uint32_t)total_kb);
    return cudaGetLastError();
}

cudaError_t launch_tensor(int variant, int dtype, const MixedArgs &a, int grid, cudaStream_t st) {
    cudaError_t e;
    if (a.ksplit <= 1u && a.top == 3u && a.best_key) {
        e = cudaMemsetAsync(a.tile_key3, 0, tensor_tile_key3_bytes((uint64_t)a.n_obj * a.n_tiles), st);
        if (e != cudaSuccess) return e;
    }
    if (variant == 0)
        e = dtype == 0 ? launch_t<false, float>(a, grid, st) : launch_t<false, double>(a, grid, st);
    else
        e = dtype == 0 ? launch_t<true, float>(a, grid, st) : launch_t<true, double>(a, grid, st);
    if (e != cudaSuccess) return e;
    if (a.ksplit <= 1u) {
        if (a.top != 3u || !a.best_key) return cudaSuccess;
        // top three: merge the tiles' warp triples
        const uint64_t blocks = ((uint64_t)a.n_obj * 32u + 255u) / 256u;
        if (blocks > 0x7fffffffull) return cudaErrorInvalidValue;
        top3_merge_kernel<<<(unsigned)blocks, 256, 0, st>>>(a.tile_key3, a.n_obj, a.n_tiles,
                                                             a.best_key);
        return cudaGetLastError();
    }
    // split units: the finishing pass over every (object, tile) pair
    const uint64_t blocks = (uint64_t)a.n_obj * a.n_tiles * (tensor_tile_freqs(variant) / kKsumFreqs);
    if (blocks > 0x7fffffffull) return cudaErrorInvalidValue;
    if (variant == 0) {
        if (dtype == 0) ksum_kernel<false, float><<<(unsigned)blocks, 256, 0, st>>>(a);
        else ksum_kernel<false, double><<<(unsigned)blocks, 256, 0, st>>>(a);
    } else {
        if (dtype == 0) ksum_kernel<true, float><<<(unsigned)blocks, 256, 0, st>>>(a);
        else ksum_kernel<true, double><<<(unsigned)blocks, 256, 0, st>>>(a);
    }
    return cudaGetLastError();
}

size_t tensor_tile_key3_bytes(uint64_t pairs) { return sizeof(unsigned long long) * 12u * pairs; }

size_t tensor_partial_bytes(int variant) {
    return sizeof(float) * (variant ? 6u * (size_t)TGeo<true>::TILE : 4u * (size_t)TGeo<false>::TILE);
}

}  // namespace lsgb
