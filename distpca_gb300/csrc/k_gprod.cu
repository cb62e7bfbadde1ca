// G'-product pass: the genotype product on the tensor cores, the missing-genotype term on the CUDA
// cores, sm_103a.
//
// With g' = genotype (0/1/2, 0 when missing), miss = 1 for missing entries and per-SNP b, a, the
// standardized value is X = b g' + a (1 - miss) (utilities.cpp:294-305), so the two products of a
// pass (methods.cpp:853-854, 862-863) are
//     Y = X Omega = diag(b) (G' Omega) + diag(a) (1 colsum(Omega)^T - Miss Omega)
//     Z = X^T Y   = G'^T (b.Y) + 1 (sum_s a_s Y_s)^T - Miss^T (a.Y).
// Only G' goes through the tensor cores: one FP16 product per pass direction instead of the two of
// mixed_gemm_kernel (G' and M = G' - Miss), and half the tensor-memory columns per A stage, so
// four A stages fit beside the accumulators instead of two.  Missing entries are a few percent of
// a genotype matrix; the decode warps, which look at every code anyway, add the dense operand's
// row of each missing entry into per-row int32 sums on the CUDA cores (Miss Omega, Miss^T (a.Y)).
//
// Exactness is the two-product kernel's: the dense operand is quantised to 24-bit fixed point
// per column (v = 4096 h + l, |v| <= 2^23), the tensor cores see the FP16 slices h, l, and the
// missing term reads the same integers v from an int32 copy [K][kp] staged by TMA beside the
// slices.  Every sum is an exact integer: the int32 row sums are folded into 64-bit integers
// before 255 entries could overflow them.  X Omega's integers are therefore those of the
// two-product kernel (F1 Omega = G' Omega - Miss Omega) and Y is bit-identical to it.  X^T Y
// quantises b.Y for the tensor cores and a.Y for the missing term at one power-of-two scale per
// column, chosen from max(|b.Y|, |a.Y|) (the X Omega epilogue's column maxima).
//
// CTA (448 threads, one per SM: it owns all of tensor memory), per batch of two 64-element
// K-blocks:
//   warp 0       TMA producer: packed 2-bit tiles [128 rows x 128 B] (4 batches per stage); per
//                batch one box of FP16 slice tiles [2 K-blocks][N rows][64] (128-byte swizzle)
//                and one box of int32 operand rows [128 K positions][kp], both on one barrier.
//   warp 1       TMEM allocation and the MMA issuer (one elected lane): 8 MMAs per batch,
//                M = 128, N = 2 kp, K = 16, A from one of four tensor-memory stages, into one of
//                two accumulators (alternating 32-batch chunks, so one drains while the other
//                accumulates).
//   warps 2..9   two groups of four warps taking alternate batches, one thread per tile row:
//                decode G' (FP16 pairs, tcgen05.st into the batch's A stage), then the missing
//                term of the row (its missing codes' int32 operand rows, summed in registers).
//   warps 10..13 drain: accumulator chunks into 64-bit integers in registers; at the end of a
//                work item the missing sums (shared memory) are subtracted and the outputs
//                written (X Omega: Y and column maxima; X^T Y: FP64 K-split partials).
// Clusters of two CTAs (consecutive row tiles, same K range) load half of each B and int32 stage
// and multicast it to both.  Every wait is bounded (tc.cuh) and reports through h->dflag.
#include "mixed.cuh"

namespace dpca {

constexpr int kGWarps = 14;
constexpr int kGThreads = 32 * kGWarps;
constexpr int kGAStages = 4;      // tensor-memory A stages; decode group g fills stages g and g + 2
constexpr int kGChunk = 32;       // batches per exact accumulation chunk (see kChunkG)
constexpr int kGFlushAt = 255;    // int32 row sums take at most 255 operand rows (|v| <= 2^23) per fold
constexpr int kGMaxRing = 6;
constexpr int kGMaxPStages = 3;
constexpr int kGSmemBudget = 232448 - 512;  // the opt-in maximum per CTA, less a margin

// 16 packed bytes = 64 codes -> FP16 pairs of g' (decode64 without the f1 half).
__device__ __forceinline__ void decode64_g(uint4 v, uint32_t (&G)[32]) {
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
            const int o = p < 5 ? 2 * p : 2 * (p - 3);
            const uint32_t src = p < 5 ? t : t6;
            const uint32_t h = (src & (0x00030003u << o)) | 0x64006400u;
            G[q * 8 + p] = fma_relu_f16x2(h, kScale[o >> 1], kBias[o >> 1]);
        }
    }
}

// Missing codes (01) of a 32-bit word of 16 codes: bit 2c set for code c.
__device__ __forceinline__ uint32_t missing_bits(uint32_t x) { return x & ~(x >> 1) & 0x55555555u; }

// Fold a thread's int32 row sums into the work item's 64-bit sums in shared memory (both decode
// groups add to the same row: atomics).  Before the first fold of item li the drain must have
// consumed (and zeroed) item li - 1's sums.
__device__ __forceinline__ bool fold_missing(int (&corr)[kMaxMixedNrhs], long long *miss, int row, int kp, int li,
                                             bool &waited, uint64_t *miss_empty, int *err, long long lim) {
    if (li >= 1 && !waited) {
        if (!__all_sync(0xffffffffu, tc::mbar_wait(miss_empty, (uint32_t)(li - 1) & 1u, err, 34, false, lim)))
            return false;
        waited = true;
    }
#pragma unroll
    for (int c = 0; c < kMaxMixedNrhs; ++c)
        if (c < kp) {
            if (corr[c] != 0)
                atomicAdd(reinterpret_cast<unsigned long long *>(miss + c * 128 + row),
                          (unsigned long long)(long long)corr[c]);
            corr[c] = 0;
        }
    return true;
}

template <int MODE, int CL>
__global__ void __launch_bounds__(kGThreads, 1)
    gprod_kernel(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b,
                 const __grid_constant__ CUtensorMap map_q, const GemmArgs args) {
    static_assert(CL == 1 || CL == 2, "clusters of 1 or 2 CTAs");
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const int N = args.N, kp = args.kp, R = args.ring, PS = args.pstages;
    const int tile_bytes = N * 128;        // one K-block of slices: N rows x 128 B
    const int bstage = 2 * tile_bytes;     // one batch
    const int qstage = 128 * kp * 4;       // int32 operand rows of one batch
    uint8_t *sP = smem;
    uint8_t *sB = sP + PS * kPStageBytes;
    uint8_t *sQ = sB + (size_t)R * bstage;
    long long *miss = (long long *)(sQ + (size_t)R * qstage);  // [kp][128] the item's missing sums
    uint64_t *bars = (uint64_t *)(miss + (size_t)kp * 128);
    uint64_t *pk_full = bars, *pk_empty = pk_full + kGMaxPStages;
    uint64_t *bfull = pk_empty + kGMaxPStages, *full = bfull + kGMaxRing, *free_ = full + kGMaxRing;
    uint64_t *aempty = free_ + kGMaxRing;
    uint64_t *acc_full = aempty + kGAStages, *acc_empty = acc_full + 2;
    uint64_t *miss_full = acc_empty + 2, *miss_empty = miss_full + 1, *mma_done = miss_empty + 1;
    uint32_t *tmem_slot = (uint32_t *)(mma_done + 1);
    unsigned int *cmax_s = tmem_slot + 1;  // X Omega column maxima of this CTA's tiles

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int *err = args.err;
    const long long lim = args.wait_cycles;

    if (threadIdx.x == 0) {
        for (int s = 0; s < PS; ++s) {
            tc::mbar_init(&pk_full[s], 1);
            tc::mbar_init(&pk_empty[s], 8);  // every decode warp releases every packed stage
        }
        for (int s = 0; s < R; ++s) {
            tc::mbar_init(&bfull[s], 1);     // producer, with the TMA bytes of all CL bands
            tc::mbar_init(&full[s], 4);      // the batch's decode group
            tc::mbar_init(&free_[s], CL);    // the MMA commit of every CTA of the cluster
        }
        for (int s = 0; s < kGAStages; ++s) tc::mbar_init(&aempty[s], 1);
        for (int v = 0; v < 2; ++v) {
            tc::mbar_init(&acc_full[v], 1);
            tc::mbar_init(&acc_empty[v], 4);
        }
        tc::mbar_init(miss_full, 8);
        tc::mbar_init(miss_empty, 4);
        tc::mbar_init(mma_done, 1);
        tc::fence_mbar_init();
        for (int c = 0; c < kMaxMixedNrhs; ++c) cmax_s[c] = 0u;
        tc::tma_prefetch(&map_a);
        tc::tma_prefetch(&map_b);
        tc::tma_prefetch(&map_q);
    }
    for (int i = threadIdx.x; i < kp * 128; i += blockDim.x) miss[i] = 0;
    if (warp == 1) {
        tc::tmem_alloc(tmem_slot, kTmemCols);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    if (CL > 1) tc::cluster_sync();
    tc::fence_after_sync();
    const uint32_t tbase = *tmem_slot;
    const int rank = CL > 1 ? (int)tc::cluster_ctarank() : 0;
    constexpr uint16_t kMask = (uint16_t)((1u << CL) - 1u);
    // TMEM columns: accumulators [0, N) and [N, 2N) ([h | l] slices each), then 4 A stages of 64
    const uint32_t a_base = (uint32_t)((2 * N + 31) & ~31);

    if (warp == 0) {
        // ---------------------------------------------------------- TMA producer
        if (lane == 0) {
            const int bband = N / CL, qband = 128 / CL;
            int sp = 0, r = 0, issued_p = 0, issued_b = 0, withheld = 0;
            uint32_t pph = 0, bph = 0;
            bool ok = true;
            bool withhold = args.inject == 1 && blockIdx.x == 0;
            for (int it = blockIdx.x; ok && it < args.items; it += gridDim.x) {
                const WorkItem x = work_item(args, it, 2);
                const int tile = min(x.tile, (args.rows + 127) / 128 - 1);  // a pair's padding tile reads a real one
                for (int t = 0; t < x.nb; ++t) {
                    if ((t & 3) == 0) {
                        if (!(ok = tc::mbar_wait(&pk_empty[sp], pph ^ 1, err, 11, true, lim))) break;
                        tc::mbar_arrive_expect_tx(&pk_full[sp], kPStageBytes);
                        if (MODE == kXTY)
                            tc::tma_load_2d(sP + sp * kPStageBytes, &map_a, &pk_full[sp], 0,
                                            (tile * args.a_ktiles + ((x.kb0 + 2 * t) >> 3)) * 128);
                        else
                            tc::tma_load_2d(sP + sp * kPStageBytes, &map_a, &pk_full[sp], (x.kb0 + 2 * t) * 16,
                                            tile * 128);
                        ++issued_p;
                        if (++sp == PS) sp = 0, pph ^= 1;
                    }
                    if (!(ok = tc::mbar_wait(&free_[r], bph ^ 1, err, 12, true, lim))) break;
                    if (withhold) {
                        withhold = false;  // injected fault: this batch never arrives
                        ++withheld;
                    } else {
                        const int kb = x.kb0 + 2 * t;
                        tc::mbar_arrive_expect_tx(&bfull[r], bstage + qstage);
                        if (CL == 1) {
                            tc::tma_load_3d(sB + (size_t)r * bstage, &map_b, &bfull[r], 0, 0, kb);
                            tc::tma_load_2d(sQ + (size_t)r * qstage, &map_q, &bfull[r], 0, kb * 64);
                        } else {
#pragma unroll
                            for (int j = 0; j < 2; ++j)
                                tc::tma_load_3d_mc(sB + (size_t)r * bstage + j * tile_bytes + rank * bband * 128,
                                                   &map_b, &bfull[r], 0, rank * bband, kb + j, kMask);
                            tc::tma_load_2d_mc(sQ + (size_t)r * qstage + rank * qband * kp * 4, &map_q, &bfull[r], 0,
                                               kb * 64 + rank * qband, kMask);
                        }
                        ++issued_b;
                    }
                    if (++r == R) r = 0, bph ^= 1;
                }
            }
            // drain: every issued copy must land before the CTA may exit (see mixed_gemm_kernel)
            for (int g = max(0, issued_p - PS); g < issued_p; ++g)
                if (!tc::mbar_wait(&pk_full[g % PS], (g / PS) & 1, err, 13, true, lim))
                    tc::mbar_wait_exit(&pk_full[g % PS], (g / PS) & 1, kExitCycles);
            const int reached = issued_b + withheld;
            for (int t = max(0, reached - R); t < reached; ++t)
                if (!tc::mbar_wait(&bfull[t % R], (t / R) & 1, err, 14, true, lim))
                    tc::mbar_wait_exit(&bfull[t % R], (t / R) & 1, kExitCycles);
            if (CL > 1)
                for (int t = max(0, reached - R); t < reached; ++t)
                    if (!tc::mbar_wait(&free_[t % R], (t / R) & 1, err, 15, true, lim))
                        tc::mbar_wait_exit(&free_[t % R], (t / R) & 1, kExitCycles);
        }
    } else if (warp == 1) {
        // ---------------------------------------------------------- MMA issuer (whole warp, one lane issues)
        const uint32_t idesc = tc::idesc_f16_f32(128, N);
        const uint64_t bdesc0 = tc::desc_kmajor_sw128(tc::smem_u32(sB));
        const uint64_t tile_units = (uint64_t)(tile_bytes >> 4);
        int r = 0, gt = 0, gch = 0;
        uint32_t ph = 0;
        bool ok = true;
        for (int it = blockIdx.x; ok && it < args.items; it += gridDim.x) {
            const int nb = work_item(args, it, 2).nb;
            for (int t = 0; t < nb; ++t) {
                if (!(ok = __all_sync(0xffffffffu, wait_fast(&full[r], ph, err, 21, lim)))) break;
                const bool fresh = t % kGChunk == 0;
                const int v = gch & 1;
                if (fresh && gch >= 2 &&
                    !(ok = __all_sync(0xffffffffu, wait_fast(&acc_empty[v], (uint32_t)((gch >> 1) - 1) & 1u, err,
                                                             22, lim))))
                    break;
                const bool chunk_done = t % kGChunk == kGChunk - 1 || t == nb - 1;
                tc::fence_after_sync();
                const uint64_t b1 = bdesc0 + (uint64_t)((r * bstage) >> 4), b2 = b1 + tile_units;
                const uint32_t a = tbase + a_base + 64u * (uint32_t)(gt & 3);
                const uint32_t d = tbase + (uint32_t)(v * N);
                if (tc::elect_one_sync()) {
                    tc::mma_ts_f16(d, a, b1, idesc, fresh ? 0u : 1u);
                    tc::mma_ts_f16(d, a + 8, b1 + 2, idesc, 1u);
                    tc::mma_ts_f16(d, a + 16, b1 + 4, idesc, 1u);
                    tc::mma_ts_f16(d, a + 24, b1 + 6, idesc, 1u);
                    tc::mma_ts_f16(d, a + 32, b2, idesc, 1u);
                    tc::mma_ts_f16(d, a + 40, b2 + 2, idesc, 1u);
                    tc::mma_ts_f16(d, a + 48, b2 + 4, idesc, 1u);
                    tc::mma_ts_f16(d, a + 56, b2 + 6, idesc, 1u);
                    if (CL == 1) tc::mma_commit(&free_[r]);
                    else tc::mma_commit_mc(&free_[r], kMask);
                    tc::mma_commit(&aempty[gt & 3]);
                    if (chunk_done) tc::mma_commit(&acc_full[v]);
                }
                __syncwarp();
                if (chunk_done) ++gch;
                if (++r == R) r = 0, ph ^= 1;
                ++gt;
            }
        }
        // every MMA must have finished before the CTA frees tensor memory, also after an error
        if (tc::elect_one_sync()) tc::mma_commit(mma_done);
        __syncwarp();
        tc::mbar_wait_exit(mma_done, 0, kExitCycles);
    } else if (warp < 10) {
        // ---------------------------------------------------------- decode + missing term (warps 2..9)
        const int grp = (warp - 2) >> 2;
        const int q = warp & 3;
        const int row = 32 * q + lane;
        const uint32_t lane_base = tbase + ((uint32_t)(32 * q) << 16);
        uint32_t G[32];
        int corr[kMaxMixedNrhs];
#pragma unroll
        for (int c = 0; c < kMaxMixedNrhs; ++c) corr[c] = 0;
        int cnt = 0;            // operand rows in corr since the last fold
        int slot = grp;         // ring slot of this group's next batch (global batch gb + t)
        uint32_t sph = 0;
        int gb = 0, pgl = 0, li = 0;
        bool ok = true;
        for (int it = blockIdx.x; ok && it < args.items; it += gridDim.x) {
            const int nb = work_item(args, it, 2).nb;
            const int nst = (nb + 3) >> 2;
            bool waited = false;
            for (int pgi = 0; ok && pgi < nst; ++pgi) {
                const int pg = pgl + pgi, sp = pg % PS;
                ok = __all_sync(0xffffffffu, tc::mbar_wait(&pk_full[sp], (pg / PS) & 1, err, 31, false, lim));
                if (!ok) break;
                const int t_end = min(4 * pgi + 4, nb);
                for (int t = 4 * pgi + (((gb + 4 * pgi) & 1) != grp ? 1 : 0); t < t_end; t += 2) {
                    const int gt = gb + t, s = gt & 3;
                    if (gt >= 4 &&
                        !(ok = __all_sync(0xffffffffu, tc::mbar_wait(&aempty[s], (uint32_t)((gt >> 2) - 1) & 1u, err,
                                                                     32, false, lim))))
                        break;
                    if (!(ok = __all_sync(0xffffffffu, tc::mbar_wait(&bfull[slot], sph, err, 33, false, lim)))) break;
                    tc::fence_after_sync();
                    const uint8_t *rowp = sP + sp * kPStageBytes + row * 128;
                    const int j0 = (2 * t) & 7;
                    const uint4 v0 = *reinterpret_cast<const uint4 *>(rowp + (((j0 + 0) ^ (row & 7)) << 4));
                    const uint4 v1 = *reinterpret_cast<const uint4 *>(rowp + (((j0 + 1) ^ (row & 7)) << 4));
                    const uint32_t a_stage = lane_base + a_base + 64u * (uint32_t)s;
                    decode64_g(v0, G);
                    tc::tmem_st_x32(a_stage, G);
                    decode64_g(v1, G);
                    tc::tmem_st_x32(a_stage + 32, G);
                    // missing codes of the batch: bit j of word pair p <-> word 2p + (j & 1), code j >> 1
                    const uint32_t m0 = missing_bits(v0.x) | (missing_bits(v0.y) << 1);
                    const uint32_t m1 = missing_bits(v0.z) | (missing_bits(v0.w) << 1);
                    const uint32_t m2 = missing_bits(v1.x) | (missing_bits(v1.y) << 1);
                    const uint32_t m3 = missing_bits(v1.z) | (missing_bits(v1.w) << 1);
                    uint64_t lo = ((uint64_t)m1 << 32) | m0, hi = ((uint64_t)m3 << 32) | m2;
                    const int nm = __popcll(lo) + __popcll(hi);
                    if (__any_sync(0xffffffffu, cnt + nm > kGFlushAt)) {
                        if (!(ok = fold_missing(corr, miss, row, kp, li, waited, miss_empty, err, lim))) break;
                        cnt = 0;
                    }
                    cnt += nm;
                    const uint8_t *qs = sQ + (size_t)slot * qstage;
                    while (__any_sync(0xffffffffu, (lo | hi) != 0ull)) {
                        if ((lo | hi) != 0ull) {
                            const bool use_lo = lo != 0ull;
                            const uint64_t cur = use_lo ? lo : hi;
                            const int b = __ffsll((long long)cur) - 1;
                            if (use_lo) lo &= lo - 1;
                            else hi &= hi - 1;
                            const int j = b & 31;
                            const int wi = 2 * ((use_lo ? 0 : 2) + (b >> 5)) + (j & 1);
                            const int4 *qr = reinterpret_cast<const int4 *>(qs + (size_t)(16 * wi + (j >> 1)) * kp * 4);
#pragma unroll
                            for (int jj = 0; jj < kMaxMixedNrhs / 4; ++jj)
                                if (4 * jj < kp) {
                                    const int4 qv = qr[jj];
                                    corr[4 * jj] += qv.x;
                                    corr[4 * jj + 1] += qv.y;
                                    corr[4 * jj + 2] += qv.z;
                                    corr[4 * jj + 3] += qv.w;
                                }
                        }
                    }
                    tc::tmem_wait_st();
                    tc::fence_before_sync();
                    __syncwarp();
                    if (lane == 0) tc::mbar_arrive(&full[slot]);
                    slot += 2;
                    if (slot >= R) slot -= R, sph ^= 1;
                }
                if (!ok) break;
                __syncwarp();
                if (lane == 0) tc::mbar_arrive(&pk_empty[sp]);  // done reading this packed stage
            }
            if (!ok) break;
            // end of the item: this group's sums into the item's, for the drain
            if (!(ok = fold_missing(corr, miss, row, kp, li, waited, miss_empty, err, lim))) break;
            cnt = 0;
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(miss_full);
            gb += nb;
            pgl += nst;
            ++li;
        }
    } else {
        // ---------------------------------------------------------- drain + epilogue (warps 10..13)
        const int q = warp & 3;
        const int r = 32 * q + lane;
        const uint32_t lane_base = tbase + ((uint32_t)(32 * q) << 16);
        const int k = args.k;
        int gch = 0, li = 0;
        bool ok = true;
        long long acc[kMaxMixedNrhs];
        for (int it = blockIdx.x; ok && it < args.items; it += gridDim.x) {
            const WorkItem x = work_item(args, it, 2);
            const int nb = x.nb;
            const int row = x.tile * 128 + r;
#pragma unroll
            for (int c = 0; c < kMaxMixedNrhs; ++c) acc[c] = 0;
            const int nch = (nb + kGChunk - 1) / kGChunk;
            for (int ch = 0; ch < nch; ++ch) {
                const int v = gch & 1;
                ok = __all_sync(0xffffffffu, tc::mbar_wait(&acc_full[v], (uint32_t)(gch >> 1) & 1u, err, 41, true, lim));
                if (!ok) break;
                tc::fence_after_sync();
                const uint32_t cb = lane_base + (uint32_t)(v * N);
#pragma unroll
                for (int j = 0; j < kMaxMixedNrhs / 8; ++j)
                    if (8 * j < kp) {
                        uint32_t hv[8], lv[8];
                        tc::tmem_ld_x8(cb + 8 * j, hv);
                        tc::tmem_ld_x8(cb + kp + 8 * j, lv);
                        tc::tmem_wait_ld();
#pragma unroll
                        for (int i = 0; i < 8; ++i) acc[8 * j + i] += slices_int(hv[i], lv[i]);
                    }
                tc::fence_before_sync();
                __syncwarp();
                if (lane == 0) tc::mbar_arrive(&acc_empty[v]);
                ++gch;
            }
            if (!ok) break;
            ok = __all_sync(0xffffffffu, tc::mbar_wait(miss_full, (uint32_t)li & 1u, err, 42, true, lim));
            if (!ok) break;
            const bool valid = row < args.rows;
            const double *sc = args.scales;
            const int c0 = lane, c1 = lane + 32;
            if (MODE == kXW) {
                double b = 0.0, a = 0.0;
                if (valid) {
                    b = args.coef[2 * (size_t)row];
                    a = args.coef[2 * (size_t)row + 1];
                }
                const DF cba = df_from_double(b - a), ca = df_from_double(a);
                // the X^T Y operands are b.Y (tensor cores) and a.Y (missing term): one scale for both
                const float cmax = (float)fmax(fabs(b), fabs(a));
                const float inv0 = c0 < k ? pow2_to_float(sc[k + c0]) : 0.f;
                const float inv1 = c1 < k ? pow2_to_float(sc[k + c1]) : 0.f;
                const long long cs0 = c0 < k ? args.colsumq[c0] : 0, cs1 = c1 < k ? args.colsumq[c1] : 0;
#pragma unroll
                for (int c = 0; c < kMaxMixedNrhs; c += 2) {
                    if (c < k) {
                        float mg[2];
#pragma unroll
                        for (int j = 0; j < 2; ++j) {
                            const int cc = c + j;
                            const float inv = __shfl_sync(0xffffffffu, cc < 32 ? inv0 : inv1, cc & 31);
                            const long long cs = __shfl_sync(0xffffffffu, cc < 32 ? cs0 : cs1, cc & 31);
                            mg[j] = 0.f;
                            if (cc < k) {
                                const long long mi = miss[cc * 128 + r];
                                miss[cc * 128 + r] = 0;
                                if (valid) {
                                    // G' Omega = acc, F1 Omega = G' Omega - Miss Omega: the two-product
                                    // kernel's integers, combined by the same formula
                                    const DF u = df_mul_int(cba, acc[cc]);
                                    const DF w = df_mul_int(ca, acc[cc] - mi + cs);
                                    const DF t = df_two_sum(u.hi, w.hi);
                                    const DF y = df_two_sum(t.hi, __fadd_rn(t.lo, __fadd_rn(u.lo, w.lo)));
                                    float yf;
                                    double yd = 0.0;
                                    if (inv != 0.f) {
                                        yf = __fmul_rn(y.hi, inv);
                                        if (args.y_out) yd = ((double)y.hi + (double)y.lo) * (double)inv;
                                    } else {
                                        yd = ((double)y.hi + (double)y.lo) * sc[k + cc];
                                        yf = (float)yd;
                                    }
                                    if (args.y_out) args.y_out[(size_t)row * k + cc] = yd;
                                    args.yt[(int64_t)cc * args.yt_ld + row] = yf;
                                    mg[j] = cmax * fabsf(yf);
                                }
                            }
                        }
#pragma unroll
                        for (int o = 16; o > 0; o >>= 1) {
                            mg[0] = fmaxf(mg[0], __shfl_xor_sync(0xffffffffu, mg[0], o));
                            mg[1] = fmaxf(mg[1], __shfl_xor_sync(0xffffffffu, mg[1], o));
                        }
                        if (lane == 0) {
                            if (mg[0] > 0.f) atomicMax(cmax_s + c, __float_as_uint(mg[0]));
                            if (c + 1 < k && mg[1] > 0.f) atomicMax(cmax_s + c + 1, __float_as_uint(mg[1]));
                        }
                    }
                }
            } else {
                const double s0 = c0 < k ? sc[3 * k + c0] : 0.0, s1 = c1 < k ? sc[3 * k + c1] : 0.0;
                double *out = args.partial + ((size_t)x.split * args.rows + (valid ? row : 0)) * k;
#pragma unroll
                for (int c = 0; c < kMaxMixedNrhs; ++c)
                    if (c < k) {
                        const double scl = __shfl_sync(0xffffffffu, c < 32 ? s0 : s1, c & 31);
                        const long long mi = miss[c * 128 + r];
                        miss[c * 128 + r] = 0;
                        if (valid) out[c] = (double)(acc[c] - mi) * scl;
                    }
            }
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(miss_empty);  // sums read and zeroed for the next item
            ++li;
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (CL > 1) tc::cluster_sync();
    tc::fence_after_sync();
    if (MODE == kXW && threadIdx.x < args.k && cmax_s[threadIdx.x] != 0u)
        atomicMax(args.colmax + threadIdx.x, cmax_s[threadIdx.x]);
    if (warp == 1) tc::tmem_dealloc(tbase, kTmemCols);
}

// ------------------------------------------------------------------ operand preparation
// Scale per column from the exact maxima of max(|a|, |b|) |Y|, then the X^T Y operands: bop[c],
// bop[kp + c] = h, l of b.Y at K position s (perm16 order in groups of 16, as the tensor cores read
// it), aq[s'][c] = the quantised a.Y of SNP s' (natural order, as the missing term reads it), and
// rq[c] = sum over SNPs of the quantised a.Y (the rank-one term).  A block covers 128 K
// positions; aq rows go out through shared memory so that its stores are coalesced.
__global__ void __launch_bounds__(128) gprod_bop_split_kernel(const float *__restrict__ yt, int64_t ld, int n_snp,
                                                              int k, int kp, const double *__restrict__ coef,
                                                              const unsigned int *__restrict__ colmax,
                                                              double *__restrict__ scales, __half *__restrict__ bop,
                                                              int *__restrict__ aq, long long *__restrict__ rq) {
    __shared__ Pow2Pair scf[kMaxMixedNrhs];
    __shared__ long long rqs[kMaxMixedNrhs];
    __shared__ int tile[128 * (kMaxMixedNrhs + 1)];
    for (int c = threadIdx.x; c < k; c += blockDim.x) {
        const double sc = pow2_scale_below((double)__uint_as_float(colmax[c]) * 1.001);
        scf[c] = pow2_pair(sc);
        rqs[c] = 0;
        if (blockIdx.x == 0) {
            scales[2 * k + c] = sc;
            scales[3 * k + c] = 1.0 / sc;
        }
    }
    __syncthreads();
    const int n128 = (n_snp + 127) & ~127;
    const int ts = kp + 1;  // padded row of the staging tile
    for (int base = blockIdx.x * 128; base < n128; base += gridDim.x * 128) {
        const int s = base + threadIdx.x;
        const int src = (s & ~15) | perm16(s & 15);
        const bool valid = src < n_snp;
        const float b = valid ? (float)coef[2 * (size_t)src] : 0.f;
        const float a = valid ? (float)coef[2 * (size_t)src + 1] : 0.f;
        int *trow = tile + (src - base) * ts;
        for (int c = 0; c < kp; ++c) {
            int na = 0;
            if (c < k) {
                const float y = valid ? yt[(int64_t)c * ld + src] * scf[c].a * scf[c].b : 0.f;
                const int nb = __float2int_rn(b * y);
                na = __float2int_rn(a * y);
                const int h = (nb + 2048) >> 12;
                bop[(int64_t)c * ld + s] = __int2half_rn(h);
                bop[(int64_t)(kp + c) * ld + s] = __int2half_rn(nb - (h << 12));
                const int ws = __reduce_add_sync(0xffffffffu, na);  // |na| <= 2^23: 32 of them fit
                if ((threadIdx.x & 31) == 0 && ws != 0)
                    atomicAdd((unsigned long long *)(rqs + c), (unsigned long long)(long long)ws);
            }
            trow[c] = na;
        }
        __syncthreads();
        int *dst = aq + (int64_t)base * kp;
        for (int e = threadIdx.x; e < 128 * kp; e += blockDim.x) dst[e] = tile[(e / kp) * ts + e % kp];
        __syncthreads();
    }
    for (int c = threadIdx.x; c < k; c += blockDim.x)
        if (rqs[c] != 0) atomicAdd((unsigned long long *)(rq + c), (unsigned long long)rqs[c]);
}

// ------------------------------------------------------------------ host side
static size_t g_fixed_bytes(int kp, int ps) {
    return 1024 + (size_t)ps * kPStageBytes + (size_t)kp * 128 * 8 + 512;  // align, packed, missing sums, barriers
}

static size_t g_slot_bytes(int N, int kp) { return (size_t)2 * N * 128 + (size_t)128 * kp * 4; }

// Deepest B/int32 ring that fits (at most kGMaxRing), with three packed stages when that leaves a
// ring of 3 or more, else two.
static void g_limits(int N, int kp, int *max_ring, int *ps) {
    for (int p = kGMaxPStages; p >= 2; --p) {
        const long long room = (long long)kGSmemBudget - (long long)g_fixed_bytes(kp, p);
        const int r = (int)std::min<long long>(kGMaxRing, room / (long long)g_slot_bytes(N, kp));
        *max_ring = r;
        *ps = p;
        if (r >= 3) return;
    }
}

static size_t g_smem(int N, int kp, int ps, int ring) {
    return std::max<size_t>(g_fixed_bytes(kp, ps) + (size_t)ring * g_slot_bytes(N, kp), kSmemFloor);
}

void gprod_set_rings(Handle *h, int ring1, int ring2) {
    MixedState *m = mstate(h);
    int maxr = 2, ps = 2;
    g_limits(m->N, m->kp, &maxr, &ps);
    m->gps = ps;
    m->gring1 = std::max(2, std::min(ring1, maxr));
    m->gring2 = std::max(2, std::min(ring2, maxr));
    m->gsmem1 = g_smem(m->N, m->kp, ps, m->gring1);
    m->gsmem2 = g_smem(m->N, m->kp, ps, m->gring2);
}

int gprod_max_ring(Handle *h) {
    MixedState *m = mstate(h);
    int maxr = 2, ps = 2;
    g_limits(m->N, m->kp, &maxr, &ps);
    return maxr;
}

static dpca_status make_q_map(CUtensorMap *map, int *base, uint64_t rows, int kp, uint32_t box_rows) {
    return make_map(map, CU_TENSOR_MAP_DATA_TYPE_INT32, base, (uint64_t)kp, rows, (uint64_t)kp * 4, (uint32_t)kp,
                    box_rows, CU_TENSOR_MAP_SWIZZLE_NONE);
}

size_t gprod_footprint(int n_ind, int n_snp, int nrhs) {
    const size_t kp = (size_t)(nrhs + 7) / 8 * 8;
    const size_t n_pad = (size_t)(n_ind + 127) / 128 * 128, rows_pad = (size_t)(n_snp + 127) / 128 * 128;
    return (n_pad + rows_pad) * kp * 4;
}

dpca_status gprod_prepare(Handle *h) {
    MixedState *m = mstate(h);
    const int kp = m->kp, N = m->N;
    if ((int)((2 * N + 31) & ~31) + 64 * kGAStages > kTmemCols) {
        set_error("internal: TMEM budget exceeded for nrhs %d", h->k);
        return DPCA_ERR_UNSUPPORTED;
    }
    const int rows_pad = (h->rows_dev + 127) / 128 * 128;
    DPCA_TRY(dev_alloc(h, (void **)&m->omega_q, (size_t)h->n_ind_pad * kp * 4));
    DPCA_TRY(dev_alloc(h, (void **)&m->aq, (size_t)rows_pad * kp * 4));
    DPCA_CUDA(cudaMemsetAsync(m->omega_q, 0, (size_t)h->n_ind_pad * kp * 4, h->stream));
    DPCA_CUDA(cudaMemsetAsync(m->aq, 0, (size_t)rows_pad * kp * 4, h->stream));
    DPCA_TRY(make_q_map(&m->map_oq[0], m->omega_q, h->n_ind_pad, kp, 128));
    DPCA_TRY(make_q_map(&m->map_oq[1], m->omega_q, h->n_ind_pad, kp, 64));
    DPCA_TRY(make_q_map(&m->map_aq[0], m->aq, rows_pad, kp, 128));
    DPCA_TRY(make_q_map(&m->map_aq[1], m->aq, rows_pad, kp, 64));
    DPCA_TRY(make_batch_map(&m->map_bg, m->bop, rows_pad, N));
    DPCA_TRY(make_batch_map(&m->map_bg_band, m->bop, rows_pad, N, (uint32_t)(N / 2), 1));
    DPCA_TRY(allow_max_smem((const void *)gprod_kernel<kXW, 1>));
    DPCA_TRY(allow_max_smem((const void *)gprod_kernel<kXW, 2>));
    DPCA_TRY(allow_max_smem((const void *)gprod_kernel<kXTY, 1>));
    DPCA_TRY(allow_max_smem((const void *)gprod_kernel<kXTY, 2>));
    int maxr = 2, ps = 2;
    g_limits(N, kp, &maxr, &ps);
    gprod_set_rings(h, maxr, maxr);
    return DPCA_OK;
}

void gprod_release(Handle *h) {
    MixedState *m = mstate(h);
    dev_free(h, m->omega_q);
    dev_free(h, m->aq);
    m->omega_q = m->aq = nullptr;
}

template <int MODE, int CL>
static dpca_status g_launch(Handle *h, const CUtensorMap &ma, const CUtensorMap &mb, const CUtensorMap &mq,
                            const GemmArgs &a, int grid, size_t smem) {
    if (CL == 1) {
        gprod_kernel<MODE, 1><<<grid, kGThreads, smem, h->stream>>>(ma, mb, mq, a);
        DPCA_CUDA(cudaGetLastError());
        return DPCA_OK;
    }
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = CL;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(kGThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = h->stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cfg.gridDim = dim3(grid);
    DPCA_CUDA(cudaLaunchKernelEx(&cfg, gprod_kernel<MODE, CL>, ma, mb, mq, a));
    return DPCA_OK;
}

// Co-resident pairs of a clustered launch (queried once per handle and kernel).
template <int MODE>
static dpca_status g_pairs(Handle *h, size_t smem, int *maxc) {
    if (*maxc > 0) return DPCA_OK;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 2;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(kGThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = h->stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cfg.gridDim = dim3(2 * h->sm_count);
    DPCA_CUDA(cudaOccupancyMaxActiveClusters(maxc, gprod_kernel<MODE, 2>, &cfg));
    if (*maxc < 1) {
        set_error("G'-product kernel: no pair of CTAs fits on this device");
        return DPCA_ERR_UNSUPPORTED;
    }
    return DPCA_OK;
}

// Y = X Omega over the rows behind map_a: a persistent grid of single CTAs, or of pairs sharing
// each Omega stage (xw_cl = 2, or DPCA_XW_CLUSTER = 2).
dpca_status gprod_xw(Handle *h, const CUtensorMap &map_a, GemmArgs a) {
    MixedState *m = mstate(h);
    a.ring = m->gring1;
    a.pstages = m->gps;
    int cl = m->xw_cl;
    if (const char *e = getenv("DPCA_XW_CLUSTER")) {
        const int v = atoi(e);
        if (v == 1 || v == 2) cl = v;
    }
    const int tiles = ceil_div(a.rows, 128);
    if (cl != 2 || tiles < 2) {
        a.tiles = a.items = tiles;
        return g_launch<kXW, 1>(h, map_a, m->map_om, m->map_oq[0], a, std::min(a.items, h->sm_count), m->gsmem1);
    }
    a.tiles = a.items = (tiles + 1) / 2 * 2;
    DPCA_TRY(g_pairs<kXW>(h, m->gsmem1, &m->g_max_clusters[0]));
    return g_launch<kXW, 2>(h, map_a, m->map_om_band, m->map_oq[1], a, std::min(a.items, 2 * m->g_max_clusters[0]),
                            m->gsmem1);
}

// Z partials = X^T Y: pairs of CTAs for long items (cluster width 0 = by item length, as the
// two-product kernel; a width of 4 runs as pairs), single CTAs otherwise.
dpca_status gprod_xty(Handle *h, const CUtensorMap &map_a, GemmArgs a, int splits, int batches_per_item) {
    MixedState *m = mstate(h);
    a.ring = m->gring2;
    a.pstages = m->gps;
    const int tiles = ceil_div(h->n_ind, 128);
    int cl = m->xty_cl;
    if (cl == 0) cl = batches_per_item > 128 && tiles >= 2 ? 2 : 1;
    if (cl > 2) cl = 2;
    if (tiles < 2) cl = 1;
    a.tiles = (tiles + cl - 1) / cl * cl;
    a.items = a.tiles * splits;
    int grid = xty_grid(h, a.items, batches_per_item);
    if (cl == 1) return g_launch<kXTY, 1>(h, map_a, m->map_bg, m->map_aq[0], a, grid, m->gsmem2);
    DPCA_TRY(g_pairs<kXTY>(h, m->gsmem2, &m->g_max_clusters[1]));
    if (grid < a.items) grid = std::min(a.items, 2 * m->g_max_clusters[1]);
    grid = (grid + 1) / 2 * 2;
    return g_launch<kXTY, 2>(h, map_a, m->map_bg_band, m->map_aq[1], a, grid, m->gsmem2);
}

dpca_status gprod_split_bop(Handle *h, int rows, const double *coef) {
    MixedState *m = mstate(h);
    const int rows_pad = (h->rows_dev + 127) / 128 * 128;
    const int n128 = (rows + 127) & ~127;
    const int grid = std::min(n128 / 128, h->sm_count * 16);
    gprod_bop_split_kernel<<<grid, 128, 0, h->stream>>>(m->yt, rows_pad, rows, h->k, m->kp, coef, m->colmax, m->scales,
                                                        m->bop, m->aq, m->rq);
    DPCA_CUDA(cudaGetLastError());
    return DPCA_OK;
}

}  // namespace dpca
