// Mixed-precision pass on the 5th-generation tensor cores (tcgen05), sm_103a.
//
// The standardized matrix is never materialised.  With g' = genotype (0/1/2, 0 when missing),
// m = 1 for non-missing entries, and per-SNP b = 1/(sd*sqrt(n_snp)), a = -avg*b,
//     X[s,i] = b_s g'[s,i] + a_s m[s,i]          (the value standardize() gives, utilities.cpp:294-305)
// so the two products of the pass (methods.cpp:853-854, 862-863) become
//     Y  = X Omega  = diag(b) (G' Omega) + diag(a) (M Omega)                      (gemm<kXW>)
//     Z  = X^T Y    = G'^T (b.Y) + M^T (a.Y)                                      (gemm<kXTY>)
// G' and M are exact in FP16.  The dense operands (Omega; b.Y and a.Y) are scaled per column by a
// power of two and split into hi + lo FP16 halves (22 significant bits), laid side by side along
// the MMA's N dimension ([hi | lo], N = 2*round_up(k, 8)), and accumulated in FP32 in TMEM.
// The per-SNP coefficients, the hi+lo recombination and the scale removal run in FP64 in the
// epilogues.
//
// Kernel structure (one CTA per 128-row output tile, 192 threads):
//   warp 0      TMA producer: packed 2-bit tiles [128 rows x 128 B] (SWIZZLE_128B) and FP16
//               operand tiles [N rows x 64 elements] (SWIZZLE_128B).
//   warp 1      TMEM allocation and the single MMA-issuing thread
//               (tcgen05.mma.kind::f16, A from tensor memory, B from shared memory).
//   warps 2..5  decode: one thread per tile row turns 16 packed bytes (64 genotypes) into
//               32+32 FP16 pairs with byte-permute table lookups and stores them into TMEM
//               (tcgen05.st); afterwards the same warps run the epilogue (tcgen05.ld).
// Pipelines are mbarrier rings; every wait is bounded (tc.cuh) and reports through h->dflag.
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "dpca_internal.h"
#include "tc.cuh"

namespace dpca {

constexpr int kXW = 1;   // Y = X Omega (rows = SNPs, K = individuals)
constexpr int kXTY = 2;  // Z = X^T Y   (rows = individuals, K = SNPs)
constexpr int kThreads = 192;
constexpr int kPStages = 3;
constexpr int kPStageBytes = 128 * 128;  // 128 rows x 128 B = 512 K-elements
constexpr int kTmemCols = 512;
constexpr int kSmemFloor = 120 * 1024;   // keeps one CTA per SM (the CTA owns all of TMEM)

struct GemmArgs {
    int rows;          // valid output rows
    int nkb_total;     // 64-element K blocks covering K
    int kb_per_split;  // K blocks per CTA (multiple of 8)
    int k, kp, N;
    int sa, sb;        // A stages (TMEM), B stages (SMEM)
    const double *coef;     // kXW: [rows][2] {b, a}
    const double *scales;   // [4][k]: omega scale, its inverse, b/aY scale, its inverse
    __half *bop;            // kXW: [2N][bop_ld]
    int64_t bop_ld;
    double *y_out;          // kXW: optional FP64 Y [rows][k]
    double *partial;        // kXTY: [splits][rows][k]
    int *err;
};

struct MixedState {
    int kp = 0, N = 0;
    __half *omega_s = nullptr;  // [N][n_ind_pad]
    __half *bop = nullptr;      // [2N][n_snp_pad]
    double *scales = nullptr;   // [4][k]
    double *rmax = nullptr;     // [1]
    double *partial = nullptr;  // [splits][n_ind][k]
    int splits = 1, kb_per_split = 8;
    int sb1 = 2, sb2 = 2;
    size_t smem1 = 0, smem2 = 0;
    CUtensorMap map_p, map_pt, map_om, map_bop;
};

// ------------------------------------------------------------------ decode
// 16 packed bytes = 64 codes -> FP16 pairs: G[m] holds g' of elements (2m, 2m+1), M[m] the
// non-missing indicator.  Per pair of codes (c0 low, c1 high) the selector picks, for the
// high byte of each half, entry c of a 4-byte table; the low bytes select a zero byte.
//   g': 00 -> 0, 01 (missing) -> 0, 10 -> 1.0 (0x3C00), 11 -> 2.0 (0x4000)
//   m : 00 -> 1, 01 -> 0,           10 -> 1,             11 -> 1
__device__ __forceinline__ void decode64(uint4 v, uint32_t (&G)[32], uint32_t (&M)[32]) {
    const uint32_t TG = 0x403C0000u, TM = 0x3C3C003Cu;
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int p = 0; p < 8; ++p) {
            uint32_t u = (w[q] >> (4 * p)) & 0xFu;
            uint32_t sel = ((u * 0x410u) & 0x3030u) | 0x0404u;
            G[q * 8 + p] = __byte_perm(TG, 0u, sel);
            M[q * 8 + p] = __byte_perm(TM, 0u, sel);
        }
}

__device__ __forceinline__ void split_half(double v, __half &hi, __half &lo) {
    hi = __double2half(v);
    lo = __double2half(v - (double)__half2float(hi));
}

template <int MODE>
__global__ void __launch_bounds__(kThreads, 1)
    mixed_gemm_kernel(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b,
                      const GemmArgs args) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const int N = args.N, kp = args.kp, SA = args.sa, SB = args.sb;
    const int bstage = (MODE == kXW ? 1 : 2) * N * 128;
    uint8_t *sP = smem;
    uint8_t *sB = smem + kPStages * kPStageBytes;
    uint64_t *bars = (uint64_t *)(sB + (size_t)SB * bstage);
    uint64_t *pk_full = bars, *pk_empty = bars + kPStages;
    uint64_t *b_full = pk_empty + kPStages, *b_empty = b_full + SB;
    uint64_t *a_full = b_empty + SB, *a_empty = a_full + SA;
    uint64_t *acc_full = a_empty + SA;
    uint32_t *tmem_slot = (uint32_t *)(acc_full + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tile = blockIdx.x, split = blockIdx.y;
    const int kb0 = split * args.kb_per_split;
    const int nkb = min(args.nkb_total, kb0 + args.kb_per_split) - kb0;
    const int npg = (nkb + 7) >> 3;
    int *err = args.err;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kPStages; ++s) {
            tc::mbar_init(&pk_full[s], 1);
            tc::mbar_init(&pk_empty[s], 128);
        }
        for (int s = 0; s < SB; ++s) {
            tc::mbar_init(&b_full[s], 1);
            tc::mbar_init(&b_empty[s], 1);
        }
        for (int s = 0; s < SA; ++s) {
            tc::mbar_init(&a_full[s], 128);
            tc::mbar_init(&a_empty[s], 1);
        }
        tc::mbar_init(acc_full, 1);
        tc::fence_mbar_init();
        tc::tma_prefetch(&map_a);
        tc::tma_prefetch(&map_b);
    }
    if (warp == 1) {
        tc::tmem_alloc(tmem_slot, kTmemCols);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = *tmem_slot;
    // accumulators first; A stages (32 columns per variant) start on a 32-column boundary
    const int a_base = ((MODE == kXW ? 2 : 1) * N + 31) & ~31;
    auto a_col = [&](int stage, int variant) -> uint32_t { return (uint32_t)(a_base + 64 * stage + 32 * variant); };

    if (warp == 0) {
        // ---------------------------------------------------------- TMA producer
        if (lane == 0) {
            int issued_p = 0, issued_b = 0;
            bool ok = true;
            for (int g = 0; g < npg && ok; ++g) {
                const int sp = g % kPStages;
                ok = tc::mbar_wait(&pk_empty[sp], ((g / kPStages) & 1) ^ 1, err, 11);
                if (!ok) break;
                tc::mbar_arrive_expect_tx(&pk_full[sp], kPStageBytes);
                tc::tma_load_2d(sP + sp * kPStageBytes, &map_a, &pk_full[sp], (kb0 + 8 * g) * 16, tile * 128);
                issued_p = g + 1;
                const int jn = min(8, nkb - 8 * g);
                for (int j = 0; j < jn; ++j) {
                    const int kb = 8 * g + j, sb = kb % SB;
                    ok = tc::mbar_wait(&b_empty[sb], ((kb / SB) & 1) ^ 1, err, 12);
                    if (!ok) break;
                    tc::mbar_arrive_expect_tx(&b_full[sb], bstage);
                    uint8_t *dst = sB + (size_t)sb * bstage;
                    tc::tma_load_2d(dst, &map_b, &b_full[sb], (kb0 + kb) * 64, 0);
                    if (MODE == kXTY) tc::tma_load_2d(dst + N * 128, &map_b, &b_full[sb], (kb0 + kb) * 64, N);
                    issued_b = kb + 1;
                }
            }
            // drain: every issued copy must land before the CTA may exit
            for (int g = max(0, issued_p - kPStages); g < issued_p; ++g)
                tc::mbar_wait(&pk_full[g % kPStages], (g / kPStages) & 1, err, 13);
            for (int kb = max(0, issued_b - SB); kb < issued_b; ++kb)
                tc::mbar_wait(&b_full[kb % SB], (kb / SB) & 1, err, 14);
        }
    } else if (warp == 1) {
        // ---------------------------------------------------------- MMA issuer
        if (lane == 0) {
            const uint32_t idesc = tc::idesc_f16_f32(128, N);
            const uint32_t sB_addr = tc::smem_u32(sB);
            for (int kb = 0; kb < nkb; ++kb) {
                const int sb = kb % SB, sa = kb % SA;
                if (!tc::mbar_wait(&b_full[sb], (kb / SB) & 1, err, 21)) break;
                if (!tc::mbar_wait(&a_full[sa], (kb / SA) & 1, err, 22)) break;
                tc::fence_after_sync();
                const uint32_t bst = sB_addr + (uint32_t)(sb * bstage);
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) {
                    const uint64_t bdesc = tc::desc_kmajor_sw128(bst + 32 * kk);
                    const uint32_t acc = (kb > 0 || kk > 0) ? 1u : 0u;
                    const uint32_t ag = tbase + a_col(sa, 0) + 8 * kk, am = tbase + a_col(sa, 1) + 8 * kk;
                    if (MODE == kXW) {
                        tc::mma_ts_f16(tbase, ag, bdesc, idesc, acc);
                        tc::mma_ts_f16(tbase + N, am, bdesc, idesc, acc);
                    } else {
                        tc::mma_ts_f16(tbase, ag, bdesc, idesc, acc);
                        tc::mma_ts_f16(tbase, am, tc::desc_kmajor_sw128(bst + N * 128 + 32 * kk), idesc, 1u);
                    }
                }
                tc::mma_commit(&b_empty[sb]);
                tc::mma_commit(&a_empty[sa]);
            }
            tc::mma_commit(acc_full);
        }
    } else {
        // ---------------------------------------------------------- decode (warps 2..5)
        const int q = warp & 3;
        const int r = 32 * q + lane;
        const uint32_t lane_base = tbase + ((uint32_t)(32 * q) << 16);
        uint32_t G[32], M[32];
        for (int kb = 0; kb < nkb; ++kb) {
            const int g = kb >> 3, j = kb & 7, sp = g % kPStages, sa = kb % SA;
            bool ok = true;
            if (j == 0) ok = tc::mbar_wait(&pk_full[sp], (g / kPStages) & 1, err, 31);
            ok = ok && tc::mbar_wait(&a_empty[sa], ((kb / SA) & 1) ^ 1, err, 32);
            if (!__all_sync(0xffffffffu, ok)) break;  // TMEM stores below are warp-collective
            const uint4 v = *reinterpret_cast<const uint4 *>(sP + sp * kPStageBytes + r * 128 + ((j ^ (r & 7)) << 4));
            decode64(v, G, M);
            tc::tmem_st_x32(lane_base + a_col(sa, 0), G);
            tc::tmem_st_x32(lane_base + a_col(sa, 1), M);
            tc::tmem_wait_st();
            tc::fence_before_sync();
            tc::mbar_arrive(&a_full[sa]);
            if (j == 7 || kb == nkb - 1) tc::mbar_arrive(&pk_empty[sp]);
        }
        // ---------------------------------------------------------- epilogue
        const bool ok = __all_sync(0xffffffffu, tc::mbar_wait(acc_full, 0, err, 41));
        tc::fence_after_sync();
        const int row = tile * 128 + r;
        const bool valid = ok && row < args.rows;
        const int k = args.k;
        const double *sc = args.scales;
        if (MODE == kXW) {
            const double b = valid ? args.coef[2 * (size_t)row] : 0.0;
            const double a = valid ? args.coef[2 * (size_t)row + 1] : 0.0;
            for (int c0 = 0; c0 < kp; c0 += 8) {
                uint32_t gh[8], gl[8], mh[8], ml[8];
                tc::tmem_ld_x8(lane_base + c0, gh);
                tc::tmem_ld_x8(lane_base + kp + c0, gl);
                tc::tmem_ld_x8(lane_base + N + c0, mh);
                tc::tmem_ld_x8(lane_base + N + kp + c0, ml);
                tc::tmem_wait_ld();
                if (!valid) continue;
#pragma unroll
                for (int jj = 0; jj < 8; ++jj) {
                    const int c = c0 + jj;
                    if (c >= k) break;
                    const double dg = (double)__uint_as_float(gh[jj]) + (double)__uint_as_float(gl[jj]);
                    const double dm = (double)__uint_as_float(mh[jj]) + (double)__uint_as_float(ml[jj]);
                    const double y = (b * dg + a * dm) * sc[k + c];
                    if (args.y_out) args.y_out[(size_t)row * k + c] = y;
                    const double s2 = sc[2 * k + c];
                    __half h1, l1, h2, l2;
                    split_half(b * y * s2, h1, l1);
                    split_half(a * y * s2, h2, l2);
                    __half *bo = args.bop + row;
                    const int64_t ld = args.bop_ld;
                    bo[(int64_t)c * ld] = h1;
                    bo[(int64_t)(kp + c) * ld] = l1;
                    bo[(int64_t)(N + c) * ld] = h2;
                    bo[(int64_t)(N + kp + c) * ld] = l2;
                }
            }
        } else {
            double *out = args.partial + ((size_t)split * args.rows + row) * k;
            for (int c0 = 0; c0 < kp; c0 += 8) {
                uint32_t hi[8], lo[8];
                tc::tmem_ld_x8(lane_base + c0, hi);
                tc::tmem_ld_x8(lane_base + kp + c0, lo);
                tc::tmem_wait_ld();
                if (!valid) continue;
#pragma unroll
                for (int jj = 0; jj < 8; ++jj) {
                    const int c = c0 + jj;
                    if (c >= k) break;
                    out[c] = ((double)__uint_as_float(hi[jj]) + (double)__uint_as_float(lo[jj])) * sc[3 * k + c];
                }
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 1) tc::tmem_dealloc(tbase, kTmemCols);
}

// ------------------------------------------------------------------ operand preparation
// max over SNPs of max(|a|,|b|) * ||X_s||_2 (single block, fixed order).
__global__ void __launch_bounds__(1024) rowbound_max_kernel(const double *rb, int n, double *out) {
    __shared__ double red[32];
    double m = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) m = fmax(m, rb[i]);
    m = warp_max(m);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = threadIdx.x < (int)(blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
        m = warp_max(m);
        if (threadIdx.x == 0) out[0] = m;
    }
}

__device__ __forceinline__ double pow2_scale_below(double bound) {
    // largest power of two s with bound * s < 2^15 (1 when bound is 0 or not finite)
    if (!(bound > 0.0) || !isfinite(bound)) return 1.0;
    int e;
    frexp(bound, &e);  // bound < 2^e
    return ldexp(1.0, 15 - e);
}

// Block per column c of Omega: scale factors for the hi/lo split of Omega and of b.Y, a.Y
// (|b_s Y_sc|, |a_s Y_sc| <= max_s(max(|a_s|,|b_s|) ||X_s||) * ||Omega_c|| by Cauchy-Schwarz).
__global__ void __launch_bounds__(256) omega_scales_kernel(const double *__restrict__ om, int n, int k,
                                                           const double *__restrict__ rmax,
                                                           double *__restrict__ scales) {
    __shared__ double red[32];
    __shared__ double redm[32];
    const int c = blockIdx.x;
    double mx = 0.0, ss = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double v = om[(size_t)i * k + c];
        mx = fmax(mx, fabs(v));
        ss += v * v;
    }
    mx = warp_max(mx);
    if ((threadIdx.x & 31) == 0) redm[threadIdx.x >> 5] = mx;
    ss = block_sum(ss, red);
    if (threadIdx.x == 0) {
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) mx = fmax(mx, redm[w]);
        double so = pow2_scale_below(mx);
        double sb = pow2_scale_below(rmax[0] * sqrt(ss) * (1.0 + 1e-3));
        scales[c] = so;
        scales[k + c] = 1.0 / so;
        scales[2 * k + c] = sb;
        scales[3 * k + c] = 1.0 / sb;
    }
}

// omega_s[c][i] = hi, omega_s[kp + c][i] = lo of Omega[i][c] * scale_c; zero padding elsewhere.
__global__ void __launch_bounds__(256) omega_split_kernel(const double *__restrict__ om, int n, int k, int kp,
                                                          int n_pad, const double *__restrict__ scales,
                                                          __half *__restrict__ out) {
    const int64_t total = (int64_t)kp * n_pad;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int c = (int)(e / n_pad), i = (int)(e - (int64_t)c * n_pad);
        __half hi = __float2half(0.f), lo = __float2half(0.f);
        if (c < k && i < n) split_half(om[(size_t)i * k + c] * scales[c], hi, lo);
        out[(int64_t)c * n_pad + i] = hi;
        out[(int64_t)(kp + c) * n_pad + i] = lo;
    }
}

__global__ void reduce_parts_kernel(const double *__restrict__ partial, int64_t elems, int splits,
                                    double *__restrict__ z) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < elems; e += (int64_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int p = 0; p < splits; ++p) s += partial[(int64_t)p * elems + e];
        z[e] = s;
    }
}

// ------------------------------------------------------------------ host side
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
    }
    return fn;
}

static dpca_status make_map(CUtensorMap *map, CUtensorMapDataType dt, void *base, uint64_t inner, uint64_t outer,
                            uint64_t row_bytes, uint32_t box_inner, uint32_t box_outer) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) {
        set_error("cuTensorMapEncodeTiled unavailable");
        return DPCA_ERR_CUDA;
    }
    cuuint64_t dims[2] = {inner, outer};
    cuuint64_t strides[1] = {row_bytes};
    cuuint32_t box[2] = {box_inner, box_outer};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(map, dt, 2, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed (%d): dims %llu x %llu, box %u x %u", (int)r,
                  (unsigned long long)inner, (unsigned long long)outer, box_inner, box_outer);
        return DPCA_ERR_CUDA;
    }
    return DPCA_OK;
}

static MixedState *mstate(Handle *h) { return (MixedState *)h->mx; }

static size_t smem_bytes(int mode, int N, int sb, int sa) {
    size_t b = 1024 + (size_t)kPStages * kPStageBytes + (size_t)sb * (mode == kXW ? 1 : 2) * N * 128 +
               (size_t)(2 * kPStages + 2 * sb + 2 * sa + 1) * 8 + 16;
    return std::max<size_t>(b, kSmemFloor);
}

static int pick_sb(int mode, int N) {
    const size_t budget = 200 * 1024 - (size_t)kPStages * kPStageBytes;
    int sb = (int)(budget / ((size_t)(mode == kXW ? 1 : 2) * N * 128));
    return std::max(2, std::min(8, sb));
}

static int pick_sa(int acc_cols) { return std::min(8, (kTmemCols - ((acc_cols + 31) & ~31)) / 64); }

dpca_status mixed_prepare(Handle *h) {
    const int k = h->k;
    MixedState *m = new (std::nothrow) MixedState();
    if (!m) return DPCA_ERR_NOMEM;
    h->mx = m;
    m->kp = (k + 7) / 8 * 8;
    m->N = 2 * m->kp;
    if (m->N > 192) {
        set_error("mixed precision supports nrhs <= 96 (got %d); use the FP64 path", k);
        return DPCA_ERR_UNSUPPORTED;
    }
    const int N = m->N;
    cudaError_t e;
    size_t om_elems = (size_t)N * h->n_ind_pad, bop_elems = (size_t)2 * N * h->n_snp_pad;
    if ((e = cudaMalloc(&m->omega_s, om_elems * 2)) != cudaSuccess ||
        (e = cudaMalloc(&m->bop, bop_elems * 2)) != cudaSuccess ||
        (e = cudaMalloc(&m->scales, 4 * (size_t)k * 8)) != cudaSuccess ||
        (e = cudaMalloc(&m->rmax, 8)) != cudaSuccess) {
        set_error("mixed operand allocation: %s", cudaGetErrorString(e));
        return DPCA_ERR_NOMEM;
    }
    DPCA_CUDA(cudaMemsetAsync(m->omega_s, 0, om_elems * 2, h->stream));
    DPCA_CUDA(cudaMemsetAsync(m->bop, 0, bop_elems * 2, h->stream));
    // split-K of X^T Y over SNPs: fill the SMs evenly (one CTA per SM owns all of TMEM)
    const int tiles2 = ceil_div(h->n_ind, 128);
    const int nkb2 = ceil_div(h->n_snp, 64);
    const int ngroups = ceil_div(nkb2, 8);
    double best = -1.0;
    int best_s = 1;
    for (int s = 1; s <= std::min(16, ngroups); ++s) {
        int per = ceil_div(ngroups, s);
        int sreal = ceil_div(ngroups, per);
        int64_t items = (int64_t)tiles2 * sreal;
        double eff = (double)items / (double)(h->sm_count * ((items + h->sm_count - 1) / h->sm_count));
        if (eff > best + 0.02) {
            best = eff;
            best_s = sreal;
        }
    }
    m->kb_per_split = 8 * ceil_div(ngroups, best_s);
    m->splits = ceil_div(nkb2, m->kb_per_split);
    if ((e = cudaMalloc(&m->partial, (size_t)m->splits * h->n_ind * k * 8)) != cudaSuccess) {
        set_error("mixed partial allocation: %s", cudaGetErrorString(e));
        return DPCA_ERR_NOMEM;
    }
    m->sb1 = pick_sb(kXW, N);
    m->sb2 = pick_sb(kXTY, N);
    m->smem1 = smem_bytes(kXW, N, m->sb1, pick_sa(2 * N));
    m->smem2 = smem_bytes(kXTY, N, m->sb2, pick_sa(N));
    DPCA_TRY(make_map(&m->map_p, CU_TENSOR_MAP_DATA_TYPE_UINT8, h->P, h->pitch, h->n_snp, h->pitch, 128, 128));
    DPCA_TRY(make_map(&m->map_pt, CU_TENSOR_MAP_DATA_TYPE_UINT8, h->PT, h->pitchT, h->n_ind, h->pitchT, 128, 128));
    DPCA_TRY(make_map(&m->map_om, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, m->omega_s, h->n_ind_pad, N,
                      (uint64_t)h->n_ind_pad * 2, 64, N));
    DPCA_TRY(make_map(&m->map_bop, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, m->bop, h->n_snp_pad, 2 * N,
                      (uint64_t)h->n_snp_pad * 2, 64, N));
    DPCA_CUDA(cudaFuncSetAttribute(mixed_gemm_kernel<kXW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)m->smem1));
    DPCA_CUDA(cudaFuncSetAttribute(mixed_gemm_kernel<kXTY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)m->smem2));
    return DPCA_OK;
}

dpca_status mixed_release(Handle *h) {
    MixedState *m = mstate(h);
    if (!m) return DPCA_OK;
    void *ptrs[] = {m->omega_s, m->bop, m->scales, m->rmax, m->partial};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    delete m;
    h->mx = nullptr;
    return DPCA_OK;
}

dpca_status mixed_after_stats(Handle *h) {
    MixedState *m = mstate(h);
    rowbound_max_kernel<<<1, 1024, 0, h->stream>>>(h->rowbound, h->n_snp, m->rmax);
    DPCA_CUDA(cudaGetLastError());
    return DPCA_OK;
}

dpca_status launch_mixed_xw(Handle *h, const double *omega, double *y_out) {
    MixedState *m = mstate(h);
    const int k = h->k, N = m->N;
    {
        ScopedLaunch t(&h->clock, h->stream, "split_omega");
        omega_scales_kernel<<<k, 256, 0, h->stream>>>(omega, h->n_ind, k, m->rmax, m->scales);
        int64_t total = (int64_t)m->kp * h->n_ind_pad;
        int grid = (int)std::min<int64_t>((total + 255) / 256, (int64_t)h->sm_count * 8);
        omega_split_kernel<<<grid, 256, 0, h->stream>>>(omega, h->n_ind, k, m->kp, h->n_ind_pad, m->scales,
                                                        m->omega_s);
        DPCA_CUDA(cudaGetLastError());
    }
    GemmArgs a{};
    a.rows = h->n_snp;
    a.nkb_total = ceil_div(h->n_ind, 64);
    a.kb_per_split = 8 * ceil_div(a.nkb_total, 8);
    a.k = k;
    a.kp = m->kp;
    a.N = N;
    a.sa = pick_sa(2 * N);
    a.sb = m->sb1;
    a.coef = h->coef;
    a.scales = m->scales;
    a.bop = m->bop;
    a.bop_ld = h->n_snp_pad;
    a.y_out = y_out;
    a.err = h->dflag;
    ScopedLaunch t(&h->clock, h->stream, "mixed_xw");
    mixed_gemm_kernel<kXW><<<dim3(ceil_div(h->n_snp, 128), 1), kThreads, m->smem1, h->stream>>>(m->map_p, m->map_om,
                                                                                                 a);
    DPCA_CUDA(cudaGetLastError());
    return DPCA_OK;
}

dpca_status launch_mixed_xty(Handle *h, double *z) {
    MixedState *m = mstate(h);
    const int k = h->k, N = m->N;
    GemmArgs a{};
    a.rows = h->n_ind;
    a.nkb_total = ceil_div(h->n_snp, 64);
    a.kb_per_split = m->kb_per_split;
    a.k = k;
    a.kp = m->kp;
    a.N = N;
    a.sa = pick_sa(N);
    a.sb = m->sb2;
    a.scales = m->scales;
    a.partial = m->partial;
    a.err = h->dflag;
    {
        ScopedLaunch t(&h->clock, h->stream, "mixed_xty");
        mixed_gemm_kernel<kXTY><<<dim3(ceil_div(h->n_ind, 128), m->splits), kThreads, m->smem2, h->stream>>>(
            m->map_pt, m->map_bop, a);
        DPCA_CUDA(cudaGetLastError());
    }
    ScopedLaunch t(&h->clock, h->stream, "mixed_reduce");
    int64_t elems = (int64_t)h->n_ind * k;
    int grid = (int)std::min<int64_t>((elems + 255) / 256, (int64_t)h->sm_count * 8);
    reduce_parts_kernel<<<grid, 256, 0, h->stream>>>(m->partial, elems, m->splits, z);
    DPCA_CUDA(cudaGetLastError());
    return DPCA_OK;
}

}  // namespace dpca
