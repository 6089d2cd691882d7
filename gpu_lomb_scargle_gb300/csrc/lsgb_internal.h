// lsgb_internal.h -- types shared by the kernels (lsgb_kernels.cu) and the host
// engine (lsgb_engine.cu). Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace lsgb {

// One observation as the mixed kernel consumes it (32 bytes, two 16-byte halves).
//   a = frac(f0 * t)  and  b = frac(dfturn * t)  in units of 2^-64 turns, where
//   f0 = fmin / 2pi and dfturn = df / 2pi, so the phase of grid point k is
//   a + k*b (mod 2^64), exact to ~(1+k) * 2^-64 turns;
//   cd, sd = cos, sin(2 pi s b): the rotation by s grid points (s = 1 for the
//   recurrence loops; the tensor form does not use them, and its records leave them 0);
//   standard:    v0 = y,          v1 = 0
//   generalized: v0 = w / W,      v1 = (w / W) * (y - ybar_w),   w = 1/dy^2.
struct __align__(16) ObsRec {
    uint32_t a_lo, a_hi, b_lo, b_hi;
    float v0, v1, cd, sd;
};
static_assert(sizeof(ObsRec) == 32, "ObsRec must be 32 bytes");

// One observation for the second-order form of the packed loop (96 bytes, six 16-byte
// quads laid out as the kernel reads them from shared memory; each 64-bit half of q1..q5
// is a ready-made f32x2 operand). A thread of that form takes the frequencies
// k0, k0 + S, k0 + 2S, ... (S = threads per CTA) as pairs (k0 + 2mS, k0 + (2m+1)S); both
// lanes of a pair advance by the angle phi = 2 S (2 pi b) per step, with
//   x[m+1] = 2 cos(phi) x[m] - x[m-1]
// when |sin phi| >= kSecondOrderMinSin (two operations per lane instead of the four of a
// rotation), else by the rotation. With u = S (2 pi b):
//   q0 = {a_lo, a_hi, b_lo, b_hi}            (as ObsRec)
//   q1 = {v0, v0, cos u, sin u}              (the odd lane's offset from the anchor)
//   q2 = {cos phi, cos phi, sin phi, sin phi}
//   q3 = {-sin phi, -sin phi, v1, v1}
//   q4 = {K, K, -K, -K},  K = 2 cos phi      (rounded once from FP64)
//   q5 = {-cos phi, -cos phi, well, 0}       (well = 1: |sin phi| >= kSecondOrderMinSin)
// All trigonometric values are computed in FP64 from the exact fixed-point phase S*b.
struct __align__(16) SoRec {
    uint4 q[6];
};
static_assert(sizeof(SoRec) == 96, "SoRec must be 96 bytes");
// Below this |sin phi| the rounding of K = 2 cos phi (up to 2^-24) would move the
// recurrence's angle by more than 2^-24 / (2 |sin phi|) per step, so such observations
// take the rotation.
constexpr double kSecondOrderMinSin = 0.125;

// Per-object parameters, indexed by the caller's object index.
struct ObjInfo {
    uint64_t row0;  // first row of the object in t / y / dy / records
    uint32_t n;     // rows
    uint32_t kb0;   // tensor form: the object's first K-block in the operand table (the sum of
                    // ceil(n / 16) over the preceding objects)
    double norm;    // standard: 2/(N var(y)) or 1; generalized mixed: 1 / weighted var(y)
    double wtot;    // generalized: sum of 1/dy^2
    double ymean;   // generalized: sum(y/dy^2) / sum(1/dy^2)
    double wsum_f;  // generalized mixed: sum of the stored float weights (~1)
    double ybar_f;  // generalized mixed: sum of the stored float w*y' / wsum_f (~0)
    // float copies for the mixed kernel, which keeps FP64 out of its loops
    float norm32;   // (float)norm
    float invw32;   // (float)(1 / wsum_f)
    float ybar32;   // (float)ybar_f
    float pad32;
    // tensor form: powers of two that bring the largest |v0| / |v1| of the object's
    // records into (1/2, 1] (FP16 operands); 1 when the weights are all zero
    float tsc0, tsc1;
};

// Best (power, index) of one (object, frequency tile).
struct TileBest {
    double p;
    uint32_t k;
    uint32_t pad;
};

// Frequency grid in turns per unit time as double-double values.
struct GridTurns {
    double f0_hi, f0_lo;  // fmin / 2pi
    double df_hi, df_lo;  // df / 2pi
};

struct MixedArgs {
    const void *rec;       // ObsRec or SoRec records (per the shape)
    const ObjInfo *objs;
    const uint32_t *perm;  // work order: objects by decreasing size
    uint32_t n_obj, n_tiles, n_freq, chunk;
    uint32_t *counter;     // persistent work-queue head (zeroed before launch)
    void *pgram;           // [n_obj x n_freq] or null
    TileBest *tile_best;   // [n_obj x n_tiles] or null
    uint32_t reanchor;     // 0: anchor at every thread's run start; R > 0: anchor every R
                           // grid points and reach the run start by the FP32 recurrence
    unsigned long long *best_key;  // [n_obj x top] packed (power bits << 32 | ~index) maxima
                                   // (the `top` best of each object, best first), or null
                                   // to use tile_best; zero means "no positive power"
    uint32_t fold;         // 1: shared memory holds a second-level sum area after the records
                           // (objects longer than `chunk` fold their chunk sums into it)
    uint32_t *status;      // tensor form: kStatusTimeout is set when a bounded pipeline wait
                           // ran out (may be null)
    const void *optab;     // tensor form: the operand table's A matrices, and
    const void *steps;     // the K-blocks' steps arrays (tensor_step_bytes each); both
                           // filled by launch_tensor_optab for this batch
    uint32_t total_kb;     // tensor form: K-blocks of the batch (the table's phase stride)
    uint32_t top;          // best frequencies kept per object: 1 (argmax) or 3
    long long wait_cycles; // tensor form: limit of a bounded pipeline wait (0: the default)
    uint32_t ksplit;       // tensor form: slices of every object's K-blocks (0 or 1: none);
                           // with slices, a unit's raw sums go to `partial` and a finishing
                           // pass forms the powers
    float *partial;        // tensor form with ksplit > 1: [units x tensor_partial_bytes]
    const uint32_t *kb_obj;  // tensor form: the object of each K-block of the batch
    unsigned long long *tile_key3;  // tensor form, top three, no slices: [n_obj x n_tiles x
                                    // 4 x 3] the three best keys of each epilogue warp of
                                    // each (object, tile), merged into best_key afterwards
};


struct PlainArgs {
    const void *t, *y, *dy;
    const ObjInfo *objs;
    const uint32_t *perm;
    uint32_t n_obj, n_tiles, n_freq, chunk;
    double fmin, df;
    uint32_t *counter;
    void *pgram;
    TileBest *tile_best;   // [n_obj x n_tiles x top]: each tile's `top` best, best first
    uint32_t top;          // 1 or 3
};

// Compiled tile shapes of the mixed kernel: frequencies per thread, threads per CTA,
// and the minimum CTAs per SM its register budget is compiled for.
struct MixedShape {
    int f, nt, minb;
    int x2;  // 0: scalar loop; 1: packed f32x2 loop (two interleaved frequency chains per
             // thread, rotation steps); 2: packed loop with strided frequencies and
             // second-order recurrence steps (SoRec records); 3: tensor-core form
             // (lsgb_tensor.cu; f = coarse steps per unit, nt = 128 fine steps)
    int uj;  // 1: two observations per inner-loop iteration (independent chains), 0: one
};
// Bytes of shared memory per staged observation of a mixed shape.
inline int mixed_rec_bytes(const MixedShape &s) { return s.x2 == 2 ? 96 : (s.x2 ? 64 : 32); }
// Bytes of the device record of one observation (ObsRec or SoRec).
inline size_t mixed_global_rec_bytes(const MixedShape &s) { return s.x2 == 2 ? 96 : 32; }
// Bytes of the second-level sum area of a mixed shape (NA sums x F x threads floats).
inline size_t mixed_fold_bytes(int variant, const MixedShape &s) {
    return (size_t)(variant ? 6 : 4) * s.f * s.nt * sizeof(float);
}

// ---- launchers (lsgb_kernels.cu); all asynchronous on `st` ----
// Bits of the status word a call's kernels set (MixedArgs::status, launch_stats).
constexpr uint32_t kStatusTimeout = 1u;   // a bounded pipeline wait of the tensor form ran out
constexpr uint32_t kStatusBadInput = 2u;  // a non-finite t / y, or a non-finite or non-positive
                                          // dy (generalized variant)
// Per-object statistics; when status is non-null it also checks the inputs (kStatusBadInput).
// Also zeroes, when given, each object's `top` best keys and the work-queue counter (the
// kernels that use them run after it), in place of two memsets.
cudaError_t launch_stats(int variant, int mixed, int dtype, int normalize, const void *t,
                         const void *y, const void *dy, ObjInfo *objs, uint32_t n_obj,
                         uint32_t *status, cudaStream_t st, unsigned long long *keys = nullptr,
                         uint32_t top = 0, uint32_t *counter = nullptr);
// so_stride 0: ObsRec records whose (cd, sd) step is one grid point (the rotation loops;
// the tensor form reads only a, b, v0, v1); > 0: SoRec records for a
// second-order shape whose CTA has so_stride threads. `rec` holds rows x 32 or rows x 96
// bytes accordingly.
cudaError_t launch_records(int variant, int dtype, const void *t, const void *y, const void *dy,
                           const uint64_t *offsets, uint32_t n_obj, const ObjInfo *objs,
                           uint64_t rows, GridTurns g, void *rec, uint32_t so_stride,
                           cudaStream_t st, bool rotation = true);
// Mixed kernel: returns cudaErrorInvalidValue when (variant, dtype, shape) is not compiled.
cudaError_t launch_mixed(int variant, int dtype, MixedShape shape, const MixedArgs &a,
                         int grid, size_t smem, cudaStream_t st);
cudaError_t mixed_occupancy(int variant, int dtype, MixedShape shape, size_t smem, int *blocks);
// Tensor-core form (lsgb_tensor.cu): frequencies per work unit, dynamic shared memory,
// launch (one persistent CTA per SM, grid <= SMs; MixedArgs as for the mixed kernel,
// ObsRec records).
uint32_t tensor_tile_freqs(int variant);
size_t tensor_smem_bytes(int variant);
cudaError_t launch_tensor(int variant, int dtype, const MixedArgs &a, int grid, cudaStream_t st);
// The tensor form's operand table: for every K-block (16 observations) of every object and
// both phases, the tile-independent left operand exp(i (a + p b)) (phase 0; times v0 for
// the standard variant) or exp(2i (a + p b)) (phase 1) for p < 128, split into FP16 hi / lo
// matrices in the kernel's shared-memory layout; and the K-block's steps array: the 16
// frequency steps b (64-bit), with the generalized variant's two scaled weights (zero past
// the object's end). One buffer of tensor_optab_bytes: the steps arrays of all K-blocks
// (total_kb x tensor_step_bytes) at its start, the A matrices after them. Needs the
// records. total_kb = sum over objects of ceil(n / 16); ObjInfo::kb0 must hold the prefix
// sums.
constexpr uint32_t kTensorKBlock = 16;
// Shortest K slice (K-blocks) a batch with fewer (object, tile) pairs than SMs is cut into:
// two of the kernel's 8-K-block passes, so that a unit's fixed costs (pipeline start, the
// store of its raw sums) stay small beside its MMAs.
constexpr uint32_t kMinSliceKB = 16;
size_t tensor_step_bytes(int variant);
size_t tensor_optab_bytes(int variant, uint64_t total_kb);
size_t tensor_partial_bytes(int variant);  // raw sums of one split unit
size_t tensor_tile_key3_bytes(uint64_t pairs);  // top three: the warp triples of the pairs
cudaError_t launch_tensor_optab(int variant, const MixedArgs &a, uint64_t total_kb, cudaStream_t st);
// Compiled mixed shapes as (variant, F, threads, min CTAs, packed, unroll); returns the count.
int mixed_shapes(int *out, int max_shapes);
cudaError_t launch_plain(int variant, int in_dtype, int out_dtype, const PlainArgs &a, int grid,
                         size_t smem, cudaStream_t st);
cudaError_t plain_occupancy(int variant, int in_dtype, int out_dtype, size_t smem, int *blocks);
// Per-object best `top` (1 or 3) frequencies from the tiles' results: best_idx and
// best_power are [n_obj x top], best first.
cudaError_t launch_best_reduce(int dtype, const TileBest *tb, uint32_t n_obj, uint32_t n_tiles,
                               uint32_t top, uint32_t *best_idx, void *best_power, cudaStream_t st);
// Largest |difference| of the plain kernel's FP64 sine/cosine from sincos() over n
// arguments spread over [-scale, scale]; *max_err (device) must start at 0.
cudaError_t launch_sincos_check(uint32_t n, uint64_t seed, double scale, double *max_err,
                                cudaStream_t st);
// Unpacks n packed keys (MixedArgs::best_key) into (index, power); an empty key gives
// (0, 0).
cudaError_t launch_key_decode(int dtype, const unsigned long long *keys, uint32_t n,
                              uint32_t *best_idx, void *best_power, cudaStream_t st);

constexpr int kPlainThreads = 256;
constexpr uint32_t kMixedSmemMax = 64 * 1024;  // shared memory for staged observations per CTA
constexpr uint32_t kPlainChunkMax = 2048;

}  // namespace lsgb
