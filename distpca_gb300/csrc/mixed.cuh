// Shared by the two tensor-core pass kernels (k_mixed.cu: G' and M products; k_gprod.cu: the
// G' product with the missing-genotype term on the CUDA cores): launch arguments, per-handle
// state, the exact fixed-point and double-float helpers, the 2-bit decode and the work-item walk.
#pragma once
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "common.cuh"
#include "dpca_internal.h"
#include "tc.cuh"

namespace dpca {

constexpr int kXW = 1;   // Y = X Omega (rows = SNPs, K = individuals)
constexpr int kXTY = 2;  // Z = X^T Y   (rows = individuals, K = SNPs)
constexpr int kWarps = 15;
constexpr int kIssuerWarpM = 14;
constexpr int kThreads = 32 * kWarps;
constexpr int kDecodeGroups = 2;         // one TMEM A stage per group
constexpr int kAStages = 2;              // TMEM A stages (batch parity)
constexpr int kPStages = 3;
constexpr int kPStageBytes = 128 * 128;  // 128 rows x 128 B = 512 K-elements = 8 K-blocks = 4 batches
constexpr int kTmemCols = 512;
constexpr int kSmemFloor = 120 * 1024;   // keeps one CTA per SM (the CTA owns all of TMEM)
constexpr int kSmemBudget = 220 * 1024;
// Batches per exact accumulation chunk.  A batch is 8 K steps of 16 products; an f1 or f2
// product term is at most 2 * 2048 in magnitude, so a batch adds at most 2^19 and 32 batches at
// most 2^24.  Every partial sum is then an integer of magnitude <= 2^24, which the FP32
// accumulator holds exactly whatever the summation order.  No chunk is longer than 32 batches:
// the f1 accumulator is staggered by a short first chunk.
constexpr int kChunkG = 32;              // f2 (= g') accumulator
constexpr int kChunkM = 32;              // f1 accumulator
constexpr int kFirstChunkM = 16;         // staggers the f1 drains against the f2 drains
constexpr int kMaxMixedNrhs = 48;        // accumulators 2 x N <= 192 columns + 2 A stages of 128
constexpr int kDrainCols = 24;           // accumulator columns the X Omega drain copies at a time
constexpr int kLongKIndividuals = 32768; // X Omega over at least this many individuals drains at once

struct GemmArgs {
    int rows;          // valid output rows
    int nkb_total;     // 64-element K blocks covering K
    int kb_per_split;  // K blocks per CTA (multiple of 8)
    int k, kp, N;
    int ring;          // batches in flight (B stages in shared memory)
    int a_ktiles;      // kXTY: 128-byte K tiles per 128-row tile of the tile-blocked A operand
    const double *coef;     // kXW: [rows][2] {b, a}
    const double *scales;   // [4][k]: omega scale, its inverse, b/aY scale, its inverse
    float *yt;              // kXW: Y transposed, [k][yt_ld] (FP32)
    int64_t yt_ld;
    unsigned int *colmax;   // kXW: per column, bits of max(|a.Y|, |(b-a).Y|) (non-negative float)
    const long long *colsumq;  // kXW: per column, sum over individuals of the quantised Omega
    double *y_out;          // kXW: optional FP64 Y [rows][k]
    double *partial;        // kXTY: [splits][rows][k]
    int *err;
    // Batched windows (independent problems over consecutive SNP ranges, each padded to whole
    // 512-SNP K tiles): kXW reads the window of each 128-row tile from tile_win and its Omega
    // slices from rows [w N, w N + N) of the B map; kXTY runs one K range per blockIdx.y
    // (win_kb0/win_nkb) and writes partial[w].  scales, colmax and colsumq then hold one block
    // per window ([4][k], [k], [k]); CTAs of windows whose win_active entry is 0 return at once.
    const int *tile_win;
    const int *win_kb0, *win_nkb;
    const int *win_active;
    int tiles, items;  // work items = tiles x splits (tile fastest); the grid is one CTA per SM at most
    // Limit of every barrier wait, in cycles (normally ~4 s).  A test shortens it together with
    // `inject` = 1, which makes CTA 0's load producer withhold its first batch: the MMA issuer's
    // wait for that batch then runs out, the kernel reports DPCA_ERR_TIMEOUT and exits cleanly.
    long long wait_cycles = tc::kWaitCycles;
    int inject = 0;
    int pstages = kPStages;  // packed-tile stages in shared memory (G'-product kernel: 2 or 3)
};

// How long a role waits, on the way out after an error, for asynchronous work it started (TMA
// copies, MMAs) to finish: far longer than either takes.
constexpr long long kExitCycles = 4000000;

struct MixedState {
    int kp = 0, N = 0;
    __half *omega_s = nullptr;  // [N][n_ind_pad]
    __half *bop = nullptr;      // [2N][n_snp_pad]
    float *yt = nullptr;        // [k][n_snp_pad]
    unsigned int *colmax = nullptr;  // [k]
    long long *colsumq = nullptr;    // [k] sum of the quantised Omega column (integers)
    long long *rq = nullptr;         // [k] sum over SNPs of the quantised a.Y column (integers)
    double *scales = nullptr;   // [4][k]
    double *partial = nullptr;  // [splits][n_ind][k]
    int splits = 1, kb_per_split = 8;
    int ring1 = 2, ring2 = 2;
    size_t smem1 = 0, smem2 = 0;
    int splits_cap = 1;          // partial buffer capacity (splits)
    int xty_cl = 0;              // X^T Y cluster width (1, 2 or 4: the dense operand is multicast; 0: by item length)
    int xty_persistent = -1;     // X^T Y grid: 1 persistent, 0 one CTA per item, -1 by item length
    int max_clusters[3] = {0, 0, 0};  // co-resident X^T Y clusters of width 1, 2, 4 (0: not queried)
    CUtensorMap map_p[2], map_pt[2], map_om, map_bop;  // [1]: second block buffer when streaming
    CUtensorMap map_bop_band[2];  // map_bop with one K-block, 2N/2 and 2N/4 rows per box (clusters of 2 and 4)
    CUtensorMap map_om_band;      // map_om with one K-block and N/2 rows per box (X Omega in pairs)
    int xw_cl = 0;                // X Omega cluster width (1 or 2; 0: by tile count)
    int xw_max_clusters = 0;      // co-resident X Omega pairs (0: not queried)
    // 0: the two-product kernel (k_mixed.cu); 1: the G'-product kernel (k_gprod.cu)
    int kernel = 0;
    int *omega_q = nullptr;       // [n_ind_pad][kp] quantised Omega as int32 (the missing term's operand)
    int *aq = nullptr;            // [rows_pad][kp] quantised a.Y as int32 (X^T Y's missing term)
    CUtensorMap map_oq[2], map_aq[2];    // their [kp] x 128-row boxes, [1]: 64-row bands (pairs)
    CUtensorMap map_bg, map_bg_band;     // b.Y slices (the first N rows of bop), full and pair-band boxes
    int gring1 = 2, gring2 = 2, gps = 3;  // B/Q ring depths and packed stages of the G'-product kernel
    size_t gsmem1 = 0, gsmem2 = 0;
    int g_max_clusters[2] = {0, 0};       // co-resident pairs: X Omega, X^T Y
};

// ------------------------------------------------------------------ decode
// K order inside every 16-element group.  Pair register p of a 32-bit word of 16 codes holds
// code p in its low half and code p + 8 in its high half (16 bits apart, so one mask picks both).
// The dense operands are stored in the same order: logical K position L of a group holds element
// perm16(L) of that group.
__host__ __device__ __forceinline__ int perm16(int L) { return (L >> 1) + 8 * (L & 1); }

__device__ __forceinline__ uint32_t fma_f16x2(uint32_t a, uint32_t b, uint32_t c) {
    uint32_t d;
    asm("fma.rn.f16x2 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
}

__device__ __forceinline__ uint32_t fma_relu_f16x2(uint32_t a, uint32_t b, uint32_t c) {
    uint32_t d;
    asm("fma.rn.relu.f16x2 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
}

// 16 packed bytes = 64 codes -> FP16 pairs: M[8q + p] holds f1 of the codes (p, p + 8) of word q,
// G[8q + p] = relu(f1) = g'.
//   f1: 00 -> 0, 01 (missing) -> -1, 10 -> 1, 11 -> 2;  t = f1 + 1 = c ^ (~c_hi & 1) in {1, 0, 2, 3}
// One 3-input logic op turns a word of 16 codes c into 16 fields t.  A field at bit offset o (even,
// o <= 8) of a 16-bit half, ORed into 0x6400 (FP16 1024, whose ulp is 1), is the FP16 value
// 1024 + t 2^o; one FP16 FMA by 2^-o, minus (1024 2^-o + 1), gives t - 1 = f1 exactly (every
// intermediate is a small integer or an exact power-of-two multiple).  Codes 0-4 and 8-12 sit at
// offsets 0-8 of the word's halves; codes 5-7 and 13-15 at offsets 4-8 of the word shifted by 6.
// So a pair costs one logic op plus two FP16 FMAs (f1, and relu(f1) for g'): the integer pipe,
// which the byte-table decode loaded with a shift, a mask and a byte permute per pair, is the
// busier one beside the tensor core.
__device__ __forceinline__ void decode64(uint4 v, uint32_t (&G)[32], uint32_t (&M)[32]) {
    // FP16 pairs {2^-o, 2^-o} and {-(1024 2^-o + 1), same} for o = 0, 2, 4, 6, 8
    const uint32_t kScale[5] = {0x3C003C00u, 0x34003400u, 0x2C002C00u, 0x24002400u, 0x1C001C00u};
    const uint32_t kBias[5] = {0xE401E401u, 0xDC04DC04u, 0xD410D410u, 0xCC40CC40u, 0xC500C500u};
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const uint32_t x = w[q];
        const uint32_t t = x ^ (~(x >> 1) & 0x55555555u);
        const uint32_t t6 = t >> 6;
#pragma unroll
        for (int p = 0; p < 8; ++p) {
            const int o = p < 5 ? 2 * p : 2 * (p - 3);  // field offset inside each half
            const uint32_t src = p < 5 ? t : t6;
            const uint32_t h = (src & (0x00030003u << o)) | 0x64006400u;
            M[q * 8 + p] = fma_f16x2(h, kScale[o >> 1], kBias[o >> 1]);
            G[q * 8 + p] = fma_relu_f16x2(h, kScale[o >> 1], kBias[o >> 1]);
        }
    }
}

// v (already scaled, |v| < 2^23) -> nearest integer n = 4096 h + l, h and l in [-2048, 2048].
__device__ __forceinline__ void fixed_slices(double v, __half &hi, __half &lo) {
    const double n = rint(v);
    const double h = rint(n * (1.0 / 4096.0));
    hi = __double2half(h);               // exact: |h| <= 2048
    lo = __double2half(n - 4096.0 * h);  // exact: |l| <= 2048
}

// An accumulator pair (h slice, l slice) of one chunk -> the exact integer 4096 h + l.  Both halves
// are integers below 2^24 in FP32, so the conversions are exact; the fold stays in integer
// arithmetic (FP64 throughput is a small fraction of the integer pipes').
__device__ __forceinline__ long long slices_int(uint32_t hbits, uint32_t lbits) {
    return (long long)__float2int_rz(__uint_as_float(hbits)) * 4096LL +
           (long long)__float2int_rz(__uint_as_float(lbits));
}

// Double-float arithmetic: a value hi + lo of two FP32 numbers carries ~48 bits.  The X Omega
// epilogue combines exact 64-bit integer sums with FP64 per-SNP coefficients; GB300's FP64 pipe
// runs at a small fraction of its FP32 rate, and ~11 FP64 operations per output element made
// the epilogue, not the MMAs, the cost of every short-K tile (cohorts of a few thousand).  So the
// combination is formed from error-free FP32 products (FMA) and compensated sums (Knuth's
// TwoSum), then rounded once to FP32.  The _rn intrinsics keep the compiler from contracting them.
struct DF {
    float hi, lo;
};

__device__ __forceinline__ DF df_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}

// FP64 coefficient -> hi + lo
__device__ __forceinline__ DF df_from_double(double x) {
    const float h = (float)x;
    return {h, (float)(x - (double)h)};
}

// A power of two held in FP64 as FP32, by integer arithmetic on its exponent; 0 when it is not an
// FP32 normal number (an Omega column below ~1e-31 or above ~1e45), for which the caller falls back
// to FP64.  (Y itself is FP32, so the mixed pass serves Omega columns whose Y = X Omega stays in
// FP32's normal range, about 1e-37 to 1e37 for unit-variance columns; the solver's Omega is
// orthonormal.)
__device__ __forceinline__ float pow2_to_float(double x) {
    const long long bits = __double_as_longlong(x);
    const int e = (int)((bits >> 52) & 0x7FF) - 1023;
    if (e < -126 || e > 127) return 0.f;
    return __int_as_float((int)(bits >> 32 & 0x80000000) | ((e + 127) << 23));
}

// A power-of-two scale held in FP64 as two FP32 factors, so that (y * a) * b = y * scale exactly
// wherever that product is an FP32 number: scales above 2^126 (the X^T Y operand of a Y column
// whose largest |value| is below ~2^-103) overflow FP32 as one factor.
struct Pow2Pair {
    float a, b;
};
__device__ __forceinline__ Pow2Pair pow2_pair(double sc) {
    return sc > 0x1p126 ? Pow2Pair{0x1p126f, (float)(sc * 0x1p-126)} : Pow2Pair{(float)sc, 1.f};
}

// c * x for an exact integer x (|x| < 2^48: x = H 2^24 + L with H, L exact in FP32).
__device__ __forceinline__ DF df_mul_int(DF c, long long x) {
    const float xh = __fmul_rn((float)(int)(x >> 24), 16777216.f);
    const float xl = (float)(int)(x & 0xFFFFFF);
    const float p1 = __fmul_rn(c.hi, xh), p2 = __fmul_rn(c.hi, xl);
    const float e1 = __fmaf_rn(c.hi, xh, -p1), e2 = __fmaf_rn(c.hi, xl, -p2);
    const DF s = df_two_sum(p1, p2);
    const float t = __fmaf_rn(c.lo, __fadd_rn(xh, xl), __fadd_rn(__fadd_rn(e1, e2), s.lo));
    return df_two_sum(s.hi, t);
}

// Slow path of a wait, out of line so that the MMA issue loop stays compact (an inlined wait
// loop in that loop costs ~90 cycles per iteration even when it never runs).
static __device__ __noinline__ bool wait_slow(uint64_t *bar, uint32_t parity, int *err, int code, long long limit) {
    return tc::mbar_wait(bar, parity, err, code, false, limit);
}

__device__ __forceinline__ bool wait_fast(uint64_t *bar, uint32_t parity, int *err, int code, long long limit) {
    return tc::mbar_try_wait(bar, parity) || wait_slow(bar, parity, err, code, limit);
}

// Chunks of an accumulator whose first chunk has `first` batches and the others `len`.
__device__ __forceinline__ int chunk_count(int nb, int first, int len) {
    return nb <= first ? 1 : 1 + (nb - first + len - 1) / len;
}

__device__ __forceinline__ int chunk_end(int c, int nb, int first, int len) {
    return min(first - 1 + c * len, nb - 1);
}

// Work item `it` of a launch: tile it % tiles, split it / tiles (for batched windows, the window
// of the tile or the split); nb = 0 for a window that has converged.  Every role of a CTA
// evaluates the same items in the same order.
struct WorkItem {
    int tile, split, win, kb0, nb;
};

__device__ __forceinline__ WorkItem work_item(const GemmArgs &a, int it, int kb_per_batch) {
    WorkItem x;
    x.tile = it % a.tiles;
    x.split = it / a.tiles;
    x.win = a.tile_win ? a.tile_win[min(x.tile, (a.rows + 127) / 128 - 1)] : (a.win_kb0 ? x.split : 0);
    const bool skip = (a.tile_win || a.win_kb0) && a.win_active && !a.win_active[x.win];
    x.kb0 = a.win_kb0 ? a.win_kb0[x.split] : x.split * a.kb_per_split;
    const int nkb = a.win_kb0 ? a.win_nkb[x.split] : min(a.nkb_total, x.kb0 + a.kb_per_split) - x.kb0;
    x.nb = skip ? 0 : (nkb + kb_per_batch - 1) / kb_per_batch;  // a trailing half batch reads zeros
    return x;
}

__device__ __forceinline__ double pow2_scale_below(double bound) {
    // largest power of two s with bound * s < 2^23 (1 when bound is 0 or not finite)
    if (!(bound > 0.0) || !isfinite(bound)) return 1.0;
    int e;
    frexp(bound, &e);  // bound < 2^e
    return ldexp(1.0, 23 - e);
}

// Tensor maps (k_mixed.cu).
dpca_status make_map(CUtensorMap *map, CUtensorMapDataType dt, void *base, uint64_t inner, uint64_t outer,
                     uint64_t row_bytes, uint32_t box_inner, uint32_t box_outer,
                     CUtensorMapSwizzle swizzle = CU_TENSOR_MAP_SWIZZLE_128B);
dpca_status make_batch_map(CUtensorMap *map, void *base, uint64_t n_pad, uint64_t rows, uint32_t box_rows = 0,
                           uint32_t box_kblocks = 2);

inline MixedState *mstate(Handle *h) { return (MixedState *)h->mx; }

// X^T Y grid: one CTA per work item or a persistent grid (k_mixed.cu).
int xty_grid(Handle *h, int items, int batches_per_item);

// The G'-product kernel (k_gprod.cu).
dpca_status gprod_prepare(Handle *h);
void gprod_release(Handle *h);
size_t gprod_footprint(int n_ind, int n_snp, int nrhs);
void gprod_set_rings(Handle *h, int ring1, int ring2);
int gprod_max_ring(Handle *h);
dpca_status gprod_xw(Handle *h, const CUtensorMap &map_a, GemmArgs a);
dpca_status gprod_xty(Handle *h, const CUtensorMap &map_a, GemmArgs a, int splits, int batches_per_item);
dpca_status gprod_split_bop(Handle *h, int rows, const double *coef);

}  // namespace dpca
