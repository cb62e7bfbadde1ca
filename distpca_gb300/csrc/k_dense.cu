// Small dense FP64 steps of the subspace iteration (methods.cpp:944-1063), all on the device:
//   launch_qr         thin QR of the n x k panel by shifted CholeskyQR3: the Gram, the k x k
//                     Cholesky factor and its inverse (one block) and A R^-1, three times, in one
//                     cooperative launch (qr_fused_kernel) or as separate kernels
//                     (methods.cpp:947-961, see launch_qr).
//   atb_kernel        C = A^T B over the n rows (B = Q^T Z, methods.cpp:972-973; the in-core
//                     Gram (XQ)^T (XQ), methods.cpp:141-142).
//   launch_eig_desc   the k x k eigenproblem (dsyev 'V','U' and the column reversal,
//                     methods.cpp:981-1000): sym_eig_kernel, parallel cyclic Jacobi in one block.
//   apply_w_kernel    Omega = Q W (methods.cpp:1006-1007).
//   coldots_kernel + criterion_kernel: sigma = sqrt(w), sum, and crit 0/1/2
//                     (methods.cpp:1012-1063).
// None of them synchronises with the host: the solve reads results back once per outer
// iteration (the criterion), so the host enqueues a whole iteration ahead of the device.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>

#include <cooperative_groups.h>

#include "common.cuh"
#include "dpca_internal.h"

namespace cg = cooperative_groups;

namespace dpca {

// ------------------------------------------------------------------ C = A^T B (k x k)
// Upper-triangle entry t (row-major, diagonal included) of a k x k matrix: row a is the largest
// with a (2k - a + 1) / 2 <= t, from a single-precision estimate corrected by whole steps.
__device__ __forceinline__ void tri_index(int t, int k, int &a, int &c) {
    const float b = 2.f * (float)k + 1.f;
    int x = (int)((b - sqrtf(fmaxf(b * b - 8.f * (float)t, 0.f))) * 0.5f);
    x = max(0, min(x, k - 1));
    while (x > 0 && x * (2 * k - x + 1) / 2 > t) --x;
    while (x + 1 < k && (x + 1) * (2 * k - x) / 2 <= t) ++x;
    a = x;
    c = t - x * (2 * k - x + 1) / 2 + x;
}

// Block b accumulates rows [b*rpb, ...) into red[b][k*k]; outputs are spread over threads.  The
// block-level body is shared with the fused QR kernel below; `tile` is [2][32][k] doubles of shared
// memory.  With `sym` (B == A, a Gram matrix) only the upper triangle's k (k + 1) / 2 sums are
// formed and each is written to both mirrored places: x y == y x in floating point, so the result
// has the bits of the full product at half the FMAs.
__device__ __forceinline__ void atb_block(const double *__restrict__ A, const double *__restrict__ B, int n, int k,
                                          int rpb, double *__restrict__ part, int bid, double *tile, bool sym) {
    double *ta = tile, *tb = sym ? tile : tile + 32 * k;
    const int r0 = bid * rpb, r1 = min(n, r0 + rpb);
    const int kk = k * k, outs = sym ? k * (k + 1) / 2 : kk;
    for (int o0 = 0; o0 < outs; o0 += 256 * 8) {
        double acc[8];
        int oa[8], oc[8];
#pragma unroll
        for (int m = 0; m < 8; ++m) {
            acc[m] = 0.0;
            const int o = o0 + threadIdx.x + 256 * m;
            oa[m] = oc[m] = 0;
            if (o < outs) {
                if (sym) {
                    tri_index(o, k, oa[m], oc[m]);
                } else {
                    oa[m] = o / k;
                    oc[m] = o - oa[m] * k;
                }
            }
        }
        for (int i0 = r0; i0 < r1; i0 += 32) {
            __syncthreads();
            for (int e = threadIdx.x; e < 32 * k; e += 256) {
                int ii = e / k, c = e - ii * k;
                int i = i0 + ii;
                ta[e] = i < r1 ? A[(size_t)i * k + c] : 0.0;
                if (!sym) tb[e] = i < r1 ? B[(size_t)i * k + c] : 0.0;
            }
            __syncthreads();
#pragma unroll
            for (int m = 0; m < 8; ++m) {
                if (o0 + (int)threadIdx.x + 256 * m < outs) {
                    const int a = oa[m], c = oc[m];
                    double s = acc[m];
#pragma unroll 1
                    for (int ii = 0; ii < 32; ++ii) s = fma(ta[ii * k + a], tb[ii * k + c], s);
                    acc[m] = s;
                }
            }
        }
#pragma unroll
        for (int m = 0; m < 8; ++m) {
            if (o0 + (int)threadIdx.x + 256 * m < outs) {
                part[(size_t)bid * kk + oa[m] * k + oc[m]] = acc[m];
                if (sym && oa[m] != oc[m]) part[(size_t)bid * kk + oc[m] * k + oa[m]] = acc[m];
            }
        }
    }
}

__global__ void __launch_bounds__(256) atb_kernel(const double *__restrict__ A, const double *__restrict__ B, int n,
                                                  int k, int rpb, double *__restrict__ part) {
    extern __shared__ double tile[];  // [2][32][k]
    atb_block(A, B, n, k, rpb, part, blockIdx.x, tile, A == B);
}

// out[e] = sum over p of part[p][e]: one warp per element, its lanes taking every 32nd part, then
// a fixed-order shuffle reduction (deterministic).  With one thread per element the k^2 sums ran
// on k^2 / 256 blocks, each thread walking all parts: ~36 us per Gram at 12,919 x 40, more than
// the Gram itself.
__device__ __forceinline__ void sum_parts_body(const double *__restrict__ part, int nparts, int elems,
                                               double *__restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int e = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; e < elems; e += warps) {
        double s = 0.0;
        for (int p = lane; p < nparts; p += 32) s += part[(size_t)p * elems + e];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) out[e] = s;
    }
}

__global__ void __launch_bounds__(256) sum_parts_kernel(const double *__restrict__ part, int nparts, int elems,
                                                        double *__restrict__ out) {
    sum_parts_body(part, nparts, elems, out);
}

// Row blocks of a Gram over n rows: as many as there are 32-row tiles, up to two per SM (FP64 is
// a small fraction of this GPU's arithmetic: the n k^2 FMAs want many SMs), within the partials
// buffer.
static void gram_split(const Handle *h, int n, int *nparts, int *rpb) {
    const int kk = h->k * h->k;
    int np = std::max(1, std::min(2 * h->sm_count, ceil_div(n, 32)));
    np = (int)std::min<int64_t>(np, (int64_t)(h->red_elems / kk));
    *rpb = ceil_div(n, np);
    *nparts = ceil_div(n, *rpb);
}

// A^T B over n rows in two launches (block partials, then their sum), timed under the given names.
static dpca_status atb_timed(Handle *h, const double *a, const double *b, int n, double *out, const char *name,
                             const char *sum_name) {
    int k = h->k;
    int kk = k * k;
    // FP64 is a small fraction of this GPU's arithmetic: spread the n k^2 FMAs over as many SMs
    // as there are 32-row tiles (up to two blocks per SM)
    int nparts = 0, rpb = 0;
    gram_split(h, n, &nparts, &rpb);
    size_t smem = (size_t)2 * 32 * k * sizeof(double);
    DPCA_TRY(allow_max_smem((const void *)atb_kernel));
    {
        ScopedLaunch t(&h->clock, h->stream, name);
        atb_kernel<<<nparts, 256, smem, h->stream>>>(a, b, n, k, rpb, h->red);
        DPCA_CUDA(cudaGetLastError());
    }
    {
        ScopedLaunch t(&h->clock, h->stream, sum_name);
        sum_parts_kernel<<<std::min(ceil_div(kk * 32, 256), 8 * h->sm_count), 256, 0, h->stream>>>(h->red, nparts, kk,
                                                                                                 out);
        DPCA_CUDA(cudaGetLastError());
    }
    return DPCA_OK;
}

dpca_status launch_atb(Handle *h, const double *a, const double *b, int n, double *out) {
    return atb_timed(h, a, b, n, out, "atb", "atb_sum");
}

// ------------------------------------------------------------------ k x k eigenproblem
// The Rayleigh-Ritz matrix B (k x k, upper triangle used, as dsyev 'U') -> eigenvalues w in
// descending order and eigenvectors W (row-major, column c belongs to w[c]): one block, cyclic
// Jacobi with the round-robin ordering, in which each round rotates k/2 disjoint index pairs at
// once (Golub & Van Loan, Matrix Computations, 4th ed., section 8.5.5, parallel Jacobi).  A round
// is three barrier-separated steps: the k/2 rotations (one thread each: theta = (a_qq - a_pp) /
// 2 a_pq, t = sgn(theta) / (|theta| + sqrt(theta^2 + 1)), c = 1 / sqrt(t^2 + 1), s = t c), the
// row update A <- J^T A over every (pair, column), and the column update A <- A J, V <- V J over
// every (pair, row), which also zeroes the annihilated entries.  A pair is skipped when
// |a_pq| <= eps/2 sqrt(|a_pp a_qq|), the relative criterion under which Jacobi keeps the
// eigenvalues of a positive semi-definite matrix (B = Q^T X^T X Q is one) to high relative
// accuracy; the solve stops after the first sweep that rotates nothing.  From the second outer
// iteration on, B is nearly diagonal (the previous Ritz vectors are the start block), and Jacobi
// converges quadratically from there: two or three sweeps.
//
// Why Jacobi and not the tridiagonal QR algorithm dsyev runs: every step here is k/2 or k^2/2
// independent updates, where the tridiagonal bulge chase is one long chain of dependent FP64
// operations, and a single thread's dependent FP64 chain is what this GPU does slowest.  Both are
// backward stable; the eigenvectors' signs are arbitrary in both (the outputs are defined up to
// column sign, as the reference's are across LAPACK builds).
constexpr int kEigThreads = 256;
constexpr int kEigMaxSweeps = 60;
constexpr int kEigSmemK = 112;  // A and V both in shared memory up to this k (2 k^2 doubles)

__host__ __device__ inline size_t eig_smem_bytes(int k) {
    return (size_t)(k <= kEigSmemK ? 2 : 1) * k * k * sizeof(double);
}

__global__ void __launch_bounds__(kEigThreads) sym_eig_kernel(const double *__restrict__ Bin, int k,
                                                              double *__restrict__ Wout, double *__restrict__ wout,
                                                              double *__restrict__ vglobal, int *__restrict__ err) {
    extern __shared__ double esm[];
    __shared__ double cs[64], sn[64], dg[128];
    __shared__ int pp[64], qq[64], ord[128];
    __shared__ int rotated;
    double *A = esm;
    double *V = k <= kEigSmemK ? esm + k * k : vglobal;
    const int tid = threadIdx.x, kk2 = k * k;
    const int kk = k + (k & 1), npairs = kk / 2;
    const int i0 = tid / k, j0 = tid - i0 * k, di = kEigThreads / k, dj = kEigThreads - di * k;
    const double eps = 0x1p-52;
    for (int e = tid; e < kk2; e += kEigThreads) {
        const int i = e / k, j = e - i * k;
        A[e] = i <= j ? Bin[e] : Bin[j * k + i];  // the upper triangle, mirrored
        V[e] = i == j ? 1.0 : 0.0;
    }
    __syncthreads();
    int sweep = 0;
    for (; sweep < kEigMaxSweeps && k > 1; ++sweep) {
        if (tid == 0) rotated = 0;
        __syncthreads();
        for (int r = 0; r < kk - 1; ++r) {
            // step 1: the rotations of this round (pair 0 = (0, 1 + r); the others pair positions
            // r + i and r - i on the circle of the remaining kk - 1 indices)
            if (tid < npairs) {
                int p = tid == 0 ? 0 : 1 + (r + tid) % (kk - 1);
                int q = tid == 0 ? 1 + r % (kk - 1) : 1 + (r - tid + kk - 1) % (kk - 1);
                if (p > q) {
                    const int t = p;
                    p = q;
                    q = t;
                }
                double c = 1.0, s = 0.0;
                if (q < k) {
                    const double apq = A[p * k + q], app = A[p * k + p], aqq = A[q * k + q];
                    if (apq != 0.0 && fabs(apq) > 0.5 * eps * sqrt(fabs(app * aqq))) {
                        const double theta = (aqq - app) / (2.0 * apq);
                        double t;
                        if (fabs(theta) > 1e150) t = 0.5 / theta;
                        else t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                        c = 1.0 / sqrt(t * t + 1.0);
                        s = t * c;
                        if (s != 0.0) rotated = 1;
                    }
                }
                pp[tid] = p;
                qq[tid] = q;
                cs[tid] = c;
                sn[tid] = s;
            }
            __syncthreads();
            // step 2: rows p, q of A for every pair (pairs touch disjoint rows).  Element e = (pair
            // i, column j) of the npairs x k grid, e = tid, tid + 256, ...: (i, j) advance by
            // (di, dj) with a carry, and every lane of a warp has work (the FP64 pipe runs a warp
            // instruction for all its lanes).  The solve's time is the FP64 rotations' dependent
            // chains and the three barriers per round, not this indexing (measured: unchanged
            // from a per-element division).
            for (int i = i0, j = j0; i < npairs;) {
                const double s = sn[i];
                if (s != 0.0) {
                    const double c = cs[i];
                    const int p = pp[i], q = qq[i];
                    const double ap = A[p * k + j], aq = A[q * k + j];
                    A[p * k + j] = c * ap - s * aq;
                    A[q * k + j] = s * ap + c * aq;
                }
                i += di;
                j += dj;
                if (j >= k) j -= k, ++i;
            }
            __syncthreads();
            // step 3: columns p, q of A and V; the annihilated pair is set to zero exactly
            for (int i = i0, j = j0; i < npairs;) {
                const double s = sn[i];
                if (s != 0.0) {
                    const double c = cs[i];
                    const int p = pp[i], q = qq[i];
                    const double ap = A[j * k + p], aq = A[j * k + q];
                    A[j * k + p] = j == q ? 0.0 : c * ap - s * aq;
                    A[j * k + q] = j == p ? 0.0 : s * ap + c * aq;
                    const double vp = V[j * k + p], vq = V[j * k + q];
                    V[j * k + p] = c * vp - s * vq;
                    V[j * k + q] = s * vp + c * vq;
                }
                i += di;
                j += dj;
                if (j >= k) j -= k, ++i;
            }
            __syncthreads();
        }
        if (!rotated) break;
        __syncthreads();
    }
    if (tid == 0 && sweep >= kEigMaxSweeps) atomicCAS(err + 1, 0, 51);  // not converged
    // descending order (ties by index): rank of each diagonal entry
    for (int i = tid; i < k; i += kEigThreads) dg[i] = A[i * k + i];
    __syncthreads();
    for (int i = tid; i < k; i += kEigThreads) {
        int rank = 0;
        for (int j = 0; j < k; ++j) rank += (dg[j] > dg[i] || (dg[j] == dg[i] && j < i)) ? 1 : 0;
        ord[rank] = i;
    }
    __syncthreads();
    for (int c = tid; c < k; c += kEigThreads) wout[c] = dg[ord[c]];
    for (int e = tid; e < kk2; e += kEigThreads) {
        const int i = e / k, c = e - i * k;
        Wout[e] = V[i * k + ord[c]];
    }
}

// The same Jacobi solve with the rotations applied in double-float arithmetic: every entry of A
// and V is a pair of FP32 numbers hi + lo (~47 bits), each update c a - s b is formed from
// error-free FP32 products (FMA) and compensated sums.  GB300 runs FP32 at many times its FP64
// rate, and the row and column updates -- ~5 k^2 FMAs per round, all of the solve's arithmetic --
// bound the FP64 kernel on its one SM together with the rotations' dependent FP64 division and
// square-root chains (a warp's FP64 instruction occupies the narrow FP64 pipe for many cycles).
// The rotations are formed in double-float too, from reciprocal square roots and quotients
// refined by Newton steps in pairs (dfp_rsqrt, dfp_div_fast).  A round is two barrier-separated
// steps: the rotations, then A <- J^T A J on 2 x 2 blocks (rows, then columns) together with
// V <- V J.  The relative skip test uses 2^-44 in place of FP64's epsilon, with an absolute floor
// of 2^-47, so the sweeps end at the pairs' precision.  B is scaled by a power of two to
// max |b| in [1/2, 1) first (FP32's exponent range), and the eigenvalues scaled back exactly.
// Each rotation's c^2 + s^2 is 1 within ~2^-45, and that error compounds over the ~2k rotations an
// entry takes per sweep: eigenvalues and eigenvectors come out within 1e-12 of max |w| up to k = 48
// (checked against LAPACK in the tests, as the FP64 kernel), ~2e-12 at k = 97.  So this kernel
// serves k <= kEigDfMaxK -- every mixed-precision width and the usual nrhs -- and the FP64 kernel
// the rest.
struct DFp {
    float hi, lo;
};

__device__ __forceinline__ DFp dfp_of(double x) {
    const float h = (float)x;
    return {h, (float)(x - (double)h)};
}

__device__ __forceinline__ double dfp_val(DFp a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ DFp dfp_fast_two_sum(float a, float b) {  // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

// c x + d y for pairs c, x, d, y (d = -s or s): two error-free products, one compensated sum
__device__ __forceinline__ DFp dfp_dot2(DFp c, DFp x, DFp d, DFp y) {
    const float p1 = __fmul_rn(c.hi, x.hi), p2 = __fmul_rn(d.hi, y.hi);
    float e1 = __fmaf_rn(c.hi, x.hi, -p1), e2 = __fmaf_rn(d.hi, y.hi, -p2);
    e1 = __fmaf_rn(c.hi, x.lo, __fmaf_rn(c.lo, x.hi, e1));
    e2 = __fmaf_rn(d.hi, y.lo, __fmaf_rn(d.lo, y.hi, e2));
    const float sh = __fadd_rn(p1, p2);  // two_sum(p1, p2)
    const float bb = __fsub_rn(sh, p1);
    const float sl = __fadd_rn(__fsub_rn(p1, __fsub_rn(sh, bb)), __fsub_rn(p2, bb));
    return dfp_fast_two_sum(sh, __fadd_rn(sl, __fadd_rn(e1, e2)));
}

__device__ __forceinline__ DFp dfp_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}

__device__ __forceinline__ DFp dfp_add(DFp a, DFp b) {
    const DFp t = dfp_two_sum(a.hi, b.hi);
    return dfp_fast_two_sum(t.hi, __fadd_rn(t.lo, __fadd_rn(a.lo, b.lo)));
}

__device__ __forceinline__ DFp dfp_mul(DFp a, DFp b) {
    const float p = __fmul_rn(a.hi, b.hi);
    const float e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, __fmaf_rn(a.hi, b.hi, -p)));
    return dfp_fast_two_sum(p, e);
}

// The pivots and rotation angles below are dependent chains.  Built on the correctly rounded FP32
// square root and quotient (multi-instruction sequences), they were the cost of the k x k kernels;
// these forms start from the hardware's approximate reciprocal square root and reciprocal instead
// and refine in pairs.

// 1/sqrt(a) for a pair a > 0: rsqrtf's estimate, one Newton step x' = x + x (1 - a x^2) / 2 in
// FP32, and one more with the residual 1 - a x^2 formed from the exact square of x in pairs
// (Newton's iteration for x^-2 = a; the second step squares the first one's ~2^-23 error): within
// ~2^-45.5 relative.  An a below 2^-100 (subnormal ones included) is scaled by 2^100 first and the
// result by 2^50, so that x^2 stays inside FP32's range; both scalings are exact.
__device__ __forceinline__ DFp dfp_rsqrt(DFp a) {
    const bool tiny = a.hi < 0x1p-100f;
    if (tiny) a = DFp{__fmul_rn(a.hi, 0x1p100f), __fmul_rn(a.lo, 0x1p100f)};
    float x = rsqrtf(a.hi);
    x = __fmaf_rn(__fmul_rn(0.5f, x), __fmaf_rn(-a.hi, __fmul_rn(x, x), 1.f), x);
    const float p = __fmul_rn(x, x), pe = __fmaf_rn(x, x, -p);  // x^2 = p + pe exactly
    const DFp q = dfp_mul(a, DFp{p, pe});                        // a x^2, within 2^-22 of 1
    const float r = __fsub_rn(__fsub_rn(1.f, q.hi), q.lo);        // 1 - q.hi is exact (Sterbenz)
    DFp y = dfp_fast_two_sum(x, __fmul_rn(__fmul_rn(0.5f, x), r));
    if (tiny) y = DFp{__fmul_rn(y.hi, 0x1p50f), __fmul_rn(y.lo, 0x1p50f)};
    return y;
}

// a / b for pairs, b != 0 and a / b inside FP32's normal range: q1 = a.hi times an approximate
// reciprocal of b.hi, then two corrections q += (a - q b) / b from remainders formed in pairs,
// each dividing by the same approximate reciprocal (each step multiplies the relative error by
// ~2^-21): ~2^-46 relative.
__device__ __forceinline__ DFp dfp_div_fast(DFp a, DFp b) {
    const float rb = __fdividef(1.f, b.hi);
    const float q1 = __fmul_rn(a.hi, rb);
    const DFp r1 = dfp_add(a, dfp_mul(b, DFp{-q1, 0.f}));
    const DFp q = dfp_fast_two_sum(q1, __fmul_rn(r1.hi, rb));
    const DFp r2 = dfp_add(a, dfp_mul(b, DFp{-q.hi, -q.lo}));
    return dfp_add(q, DFp{__fmul_rn(r2.hi, rb), 0.f});
}

__global__ void __launch_bounds__(kEigThreads) sym_eig_df_kernel(const double *__restrict__ Bin, int k,
                                                                 double *__restrict__ Wout, double *__restrict__ wout,
                                                                 int *__restrict__ err) {
    extern __shared__ DFp dsm[];  // A | V, k x k pairs each
    __shared__ DFp cs[64], sn[64];
    __shared__ double dg[128], red[kEigThreads / 32];
    __shared__ int pp[64], qq[64], ord[128];
    __shared__ int rotated;
    __shared__ double scale;
    DFp *A = dsm, *V = dsm + k * k;
    const int tid = threadIdx.x, kk2 = k * k;
    const int kk = k + (k & 1), npairs = kk / 2;
    const int i0 = tid / k, j0 = tid - i0 * k, di = kEigThreads / k, dj = kEigThreads - di * k;
    const double eps = 0x1p-44;
    // power-of-two scale: max |b| of the upper triangle into [1/2, 1)
    double mx = 0.0;
    for (int e = tid; e < kk2; e += kEigThreads) {
        const int i = e / k, j = e - i * k;
        if (i <= j) mx = fmax(mx, fabs(Bin[e]));
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((tid & 31) == 0) red[tid >> 5] = mx;
    __syncthreads();
    if (tid == 0) {
        double m = 0.0;
        for (int w = 0; w < kEigThreads / 32; ++w) m = fmax(m, red[w]);
        int ex = 0;
        if (m > 0.0 && isfinite(m)) frexp(m, &ex);
        scale = ldexp(1.0, -ex);
    }
    __syncthreads();
    const double sc = scale;
    for (int e = tid; e < kk2; e += kEigThreads) {
        const int i = e / k, j = e - i * k;
        A[e] = dfp_of((i <= j ? Bin[e] : Bin[j * k + i]) * sc);
        V[e] = DFp{i == j ? 1.f : 0.f, 0.f};
    }
    __syncthreads();
    int sweep = 0;
    for (; sweep < kEigMaxSweeps && k > 1; ++sweep) {
        if (tid == 0) rotated = 0;
        __syncthreads();
        for (int r = 0; r < kk - 1; ++r) {
            if (tid < npairs) {
                int p = tid == 0 ? 0 : 1 + (r + tid) % (kk - 1);
                int q = tid == 0 ? 1 + r % (kk - 1) : 1 + (r - tid + kk - 1) % (kk - 1);
                if (p > q) {
                    const int t = p;
                    p = q;
                    q = t;
                }
                DFp c = {1.f, 0.f}, s = {0.f, 0.f};
                if (q < k) {
                    const DFp apq = A[p * k + q], app = A[p * k + p], aqq = A[q * k + q];
                    // the skip test on the leading parts; also an absolute floor at the pairs'
                    // rounding level (max |a| < 1 after the scaling), so that the sweeps end when a
                    // diagonal entry is ~0
                    if (fabsf(apq.hi) > fmaxf(0.5f * (float)eps * sqrtf(fabsf(app.hi * aqq.hi)), 0x1p-47f)) {
                        // t = tan of the angle that zeroes a_pq, in the form without cancellation:
                        // sgn(theta) 2 |a_pq| / (|d| + sqrt(d^2 + 4 a_pq^2)), d = a_qq - a_pp,
                        // theta = d / (2 a_pq) (theta = 0 takes the + sign); then
                        // c = 1 / sqrt(1 + t^2), s = t c -- all in double-float
                        const DFp d = dfp_add(aqq, DFp{-app.hi, -app.lo});
                        const bool neg = (d.hi < 0.f) != (apq.hi < 0.f) && d.hi != 0.f;
                        const DFp ad = d.hi < 0.f ? DFp{-d.hi, -d.lo} : d;
                        const DFp aa = apq.hi < 0.f ? DFp{-apq.hi, -apq.lo} : apq;
                        const DFp two_a = {2.f * aa.hi, 2.f * aa.lo};
                        const DFp h2 = dfp_add(dfp_mul(ad, ad), dfp_mul(two_a, two_a));
                        const DFp rt = dfp_mul(h2, dfp_rsqrt(h2));  // sqrt(d^2 + 4 a_pq^2)
                        DFp t = dfp_div_fast(two_a, dfp_add(ad, rt));
                        if (neg) t = DFp{-t.hi, -t.lo};
                        c = dfp_rsqrt(dfp_add(DFp{1.f, 0.f}, dfp_mul(t, t)));
                        s = dfp_mul(t, c);
                        if (s.hi != 0.f) rotated = 1;
                    }
                }
                pp[tid] = p;
                qq[tid] = q;
                cs[tid] = c;
                sn[tid] = s;
            }
            __syncthreads();
            // A <- J^T A J on the 2 x 2 blocks (pair P rows, pair Q columns), one block per thread:
            // the rows by P's rotation, then the columns by Q's, as separate row and column passes
            // would do them (the same operations, so the same bits), with one barrier instead of
            // two; the annihilated pair is set to zero exactly.  V <- V J in the same step.
            for (int bq = tid; bq < npairs * npairs; bq += kEigThreads) {
                const int P = bq / npairs, Q = bq - P * npairs;
                const DFp sP = sn[P], sQ = sn[Q];
                if (sP.hi == 0.f && sQ.hi == 0.f) continue;
                const int x0 = pp[P], x1 = qq[P], y0 = pp[Q], y1 = qq[Q];  // x1, y1 may be the pad k
                const bool vx1 = x1 < k, vy1 = y1 < k;
                DFp e00 = A[x0 * k + y0], e01 = vy1 ? A[x0 * k + y1] : DFp{0.f, 0.f};
                DFp e10 = vx1 ? A[x1 * k + y0] : DFp{0.f, 0.f};
                DFp e11 = vx1 && vy1 ? A[x1 * k + y1] : DFp{0.f, 0.f};
                if (sP.hi != 0.f) {  // rows x0, x1 (both real when P rotates)
                    const DFp c = cs[P], ms = DFp{-sP.hi, -sP.lo};
                    DFp t0 = dfp_dot2(c, e00, ms, e10), t1 = dfp_dot2(sP, e00, c, e10);
                    e00 = t0;
                    e10 = t1;
                    if (vy1) {
                        t0 = dfp_dot2(c, e01, ms, e11);
                        t1 = dfp_dot2(sP, e01, c, e11);
                        e01 = t0;
                        e11 = t1;
                    }
                }
                if (sQ.hi != 0.f) {  // columns y0, y1 (both real when Q rotates)
                    const DFp c = cs[Q], ms = DFp{-sQ.hi, -sQ.lo};
                    DFp t0 = x0 == y1 ? DFp{0.f, 0.f} : dfp_dot2(c, e00, ms, e01);
                    DFp t1 = x0 == y0 ? DFp{0.f, 0.f} : dfp_dot2(sQ, e00, c, e01);
                    e00 = t0;
                    e01 = t1;
                    if (vx1) {
                        t0 = x1 == y1 ? DFp{0.f, 0.f} : dfp_dot2(c, e10, ms, e11);
                        t1 = x1 == y0 ? DFp{0.f, 0.f} : dfp_dot2(sQ, e10, c, e11);
                        e10 = t0;
                        e11 = t1;
                    }
                }
                A[x0 * k + y0] = e00;
                if (vy1) A[x0 * k + y1] = e01;
                if (vx1) A[x1 * k + y0] = e10;
                if (vx1 && vy1) A[x1 * k + y1] = e11;
            }
            for (int i = i0, j = j0; i < npairs;) {
                const DFp s = sn[i];
                if (s.hi != 0.f) {
                    const DFp c = cs[i], ms = DFp{-s.hi, -s.lo};
                    const int p = pp[i], q = qq[i];
                    const DFp vp = V[j * k + p], vq = V[j * k + q];
                    V[j * k + p] = dfp_dot2(c, vp, ms, vq);
                    V[j * k + q] = dfp_dot2(s, vp, c, vq);
                }
                i += di;
                j += dj;
                if (j >= k) j -= k, ++i;
            }
            __syncthreads();
        }
        if (!rotated) break;
        __syncthreads();
    }
    if (tid == 0 && sweep >= kEigMaxSweeps) atomicCAS(err + 1, 0, 52);  // not converged
    for (int i = tid; i < k; i += kEigThreads) dg[i] = dfp_val(A[i * k + i]) / sc;  // sc a power of two: exact
    __syncthreads();
    for (int i = tid; i < k; i += kEigThreads) {
        int rank = 0;
        for (int j = 0; j < k; ++j) rank += (dg[j] > dg[i] || (dg[j] == dg[i] && j < i)) ? 1 : 0;
        ord[rank] = i;
    }
    __syncthreads();
    for (int c = tid; c < k; c += kEigThreads) wout[c] = dg[ord[c]];
    for (int e = tid; e < kk2; e += kEigThreads) {
        const int i = e / k, c = e - i * k;
        Wout[e] = dfp_val(V[i * k + ord[c]]);
    }
}

// The k x k eigensolve on `stream`: the double-float kernel up to kEigDfMaxK, the FP64 kernel (V
// in global scratch above kEigSmemK) beyond.  Measured at k = 40: 0.58 vs 1.20 ms per solve; at
// k = 20: 0.10 vs 0.24 ms.
constexpr int kEigDfMaxK = 48;

static dpca_status eig_launch(const double *B, int k, double *W, double *w, double *vscratch, int *flags,
                              cudaStream_t stream) {
    if (k <= kEigDfMaxK) {
        DPCA_TRY(allow_max_smem((const void *)sym_eig_df_kernel));
        sym_eig_df_kernel<<<1, kEigThreads, (size_t)2 * k * k * sizeof(DFp), stream>>>(B, k, W, w, flags);
    } else {
        DPCA_TRY(allow_max_smem((const void *)sym_eig_kernel));
        sym_eig_kernel<<<1, kEigThreads, eig_smem_bytes(k), stream>>>(B, k, W, w, vscratch, flags);
    }
    DPCA_CUDA(cudaGetLastError());
    return DPCA_OK;
}

dpca_status launch_eig_desc(Handle *h) {
    ScopedLaunch t(&h->clock, h->stream, "sym_eig");
    const int k = h->k;
    const SmallLayout L{k};
    // V lives in global memory (the reduction scratch, >= k^2 doubles, free at this step) when
    // A and V do not both fit in shared memory
    return eig_launch(h->small + L.B(), k, h->small + L.W(), h->small + L.w(), h->red, h->dflag, h->stream);
}

// ------------------------------------------------------------------ Omega = Q W
// With `upper` (W upper triangular, as R^-1 in the QR) the sum of column c stops at row c: the
// terms past it are fma(q, 0, s) = s for finite q, so the bits are those of the full sum at about
// half the FMAs.
__device__ __forceinline__ void apply_w_body(const double *__restrict__ Q, const double *__restrict__ W, int n, int k,
                                             double *__restrict__ out, double *ws, bool upper = false) {
    if (W) {  // else ws already holds it
        for (int e = threadIdx.x; e < k * k; e += blockDim.x) ws[e] = W[e];
        __syncthreads();
    }
    int64_t total = (int64_t)n * k;
    for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < total; o += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = o / k;
        int c = (int)(o - i * k);
        const double *q = Q + i * k;
        double s = 0.0;
        const int end = upper ? c + 1 : k;
        for (int a = 0; a < end; ++a) s = fma(q[a], ws[a * k + c], s);
        out[o] = s;
    }
}

__global__ void __launch_bounds__(256) apply_w_kernel(const double *__restrict__ Q, const double *__restrict__ W, int n,
                                                      int k, double *__restrict__ out, int upper) {
    extern __shared__ double ws[];
    apply_w_body(Q, W, n, k, out, ws, upper != 0);
}

dpca_status launch_apply_w(Handle *h, const double *q, double *out) {
    ScopedLaunch t(&h->clock, h->stream, "apply_w");
    int k = h->k;
    size_t smem = (size_t)k * k * sizeof(double);
    DPCA_TRY(allow_max_smem((const void *)apply_w_kernel));
    int64_t total = (int64_t)h->n_ind * k;
    int grid = (int)std::min<int64_t>((total + 255) / 256, (int64_t)h->sm_count * 4);
    apply_w_kernel<<<grid, 256, smem, h->stream>>>(q, h->small + SmallLayout{k}.W(), h->n_ind, k, out, 0);
    DPCA_CUDA(cudaGetLastError());
    return DPCA_OK;
}

// ------------------------------------------------------------------ k x k Cholesky and inverse
// Rinv = R^-1 of R = chol(G [+ s I]), both k x k row-major (upper triangle, zeros below), in one
// block: one step of the shifted CholeskyQR3 below.  The shift s = 11 (n k + k (k + 1)) u tr(G) is
// applied when `shift` is set or when a plain factorization meets a non-positive pivot; a pivot
// that still fails is replaced by 1 (a zero or non-finite column stays unnormalised instead of
// dividing by zero).  Right-looking factorization in shared memory (k barrier-separated steps:
// the pivot, the scaling of its row, the rank-one update of the trailing upper triangle over all
// threads), then the inverse in place column by column, R^-1[i][j] = -R^-1[j][j] *
// sum_{l=i..j-1} R^-1[i][l] R[l][j], each row's sum split over a team of lanes.
constexpr int kCholThreads = 256;

__device__ __forceinline__ void chol_inv_block(const double *__restrict__ G, int k, int n, int always_shift,
                                               double *__restrict__ Rinv, double *S /* k x k shared */) {
    __shared__ double pinv[128], col[128];
    __shared__ double shift;
    __shared__ int broke;
    const int tid = threadIdx.x, kk2 = k * k;
    if (tid == 0) {
        double tr = 0.0;
        for (int i = 0; i < k; ++i) tr += G[i * k + i];
        shift = 11.0 * ((double)n * k + (double)k * (k + 1)) * 0x1p-53 * tr;
    }
    for (int attempt = always_shift ? 1 : 0; attempt < 2; ++attempt) {
        __syncthreads();
        for (int e = tid; e < kk2; e += kCholThreads) {
            const int i = e / k, j = e - i * k;
            S[e] = G[e] + (attempt == 1 && i == j ? shift : 0.0);
        }
        if (tid == 0) broke = 0;
        __syncthreads();
        for (int j = 0; j < k; ++j) {
            if (tid == 0) {
                double d = S[j * k + j];
                if (!(d > 0.0) || !isfinite(d)) {
                    if (attempt == 0) broke = 1;
                    d = 1.0;
                }
                const double r = sqrt(d);
                S[j * k + j] = r;
                pinv[j] = 1.0 / r;
            }
            __syncthreads();
            if (broke) break;  // block-uniform: read after the barrier
            const double inv = pinv[j];
            for (int c = j + 1 + tid; c < k; c += kCholThreads) S[j * k + c] *= inv;
            __syncthreads();
            // trailing upper triangle: a warp per row, its lanes over the row's columns
            for (int a = j + 1 + (tid >> 5); a < k; a += kCholThreads / 32) {
                const double sa = S[j * k + a];
                for (int c = a + (tid & 31); c < k; c += 32) S[a * k + c] -= sa * S[j * k + c];
            }
            __syncthreads();
        }
        if (!broke) break;
    }
    // inverse in place: column j of R^-1 from the columns before it (already inverted) and
    // column j of R (still intact); teams of `tw` lanes (a power of two <= 32) share a row's sum
    int tw = 1;
    while (tw < 32 && tw * 2 * k <= kCholThreads) tw *= 2;
    const int team = tid / tw, lane = tid % tw, teams = kCholThreads / tw;
    for (int j = 0; j < k; ++j) {
        for (int i0 = 0; i0 < j; i0 += teams) {
            const int i = i0 + team;
            double sum = 0.0;
            if (i < j)
                for (int l = i + lane; l < j; l += tw) sum = fma(S[i * k + l], S[l * k + j], sum);
            for (int o = tw >> 1; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o, tw);
            if (i < j && lane == 0) col[i] = -sum * pinv[j];
        }
        __syncthreads();
        for (int i = tid; i < j; i += kCholThreads) S[i * k + j] = col[i];
        if (tid == 0) S[j * k + j] = pinv[j];
        __syncthreads();
    }
    for (int e = tid; e < kk2; e += kCholThreads) {
        const int i = e / k, j = e - i * k;
        Rinv[e] = j >= i ? S[e] : 0.0;
    }
}

// The same factor and inverse in double-float arithmetic (the pairs of the Jacobi solver above),
// for k <= kEigDfMaxK.  G is scaled by an even power of two 4^-e (max diagonal in [1/4, 1), FP32's
// exponent range), so R scales by 2^-e and R^-1 by 2^e, both exactly; the shift uses the pairs'
// unit roundoff 2^-47 in place of FP64's 2^-53, as the shifted CholeskyQR analysis asks of the
// working precision.  R^-1 comes out to ~k 2^-47 relative, and the last two (unshifted) steps of
// CholeskyQR3 leave Q orthonormal to that order, ~1e-13.
//
// One barrier per column: step j's pivot 1/r = 1/sqrt(d_j) (dfp_rsqrt) and r = d_j / r are taken
// by every thread from the same d_j (the same operations, so the same bits in every thread), row j
// of R is written to its own array while the trailing update recomputes the scaled entries it
// needs, and column j of R^-1 (from R's column j and the inverse's columns before it, written by
// earlier steps) is formed in the same step.  The arithmetic of every entry is that of a
// factorization followed by a column-by-column inversion with the scaled row held in place: only
// the waits are fewer.  The trailing update loads a warp's rows (at most kRowsPerWarp of them)
// before storing any, so that their independent chains overlap.
//
// Rank deficiency.  The first (shifted) step has every pivot above the shift.  In the unshifted
// steps a pivot at or below kPivotFloor (the scaled Gram's largest diagonal is in [1/4, 1), and
// these steps' Grams are near the identity) means a column that is numerically a combination of
// the columns before it -- an exactly rank-deficient panel, such as a full-width block whose
// cohort has fewer independent directions than columns.  Its pivot is replaced by kPivotFloor:
// that column comes out as rescaled rounding noise, which the next step orthonormalizes against
// the others, while every other column keeps its exact normalisation.  (A sign change of that
// noise-level pivot, from last-bit differences, used to send the whole step to a shifted retry,
// which shrinks every column by ~shift / (2 diag): 4e-9 for a 37-column full-width panel.)
constexpr int kRowsPerWarp = (kEigDfMaxK + kCholThreads / 32 - 1) / (kCholThreads / 32);
constexpr float kPivotFloor = 0x1p-47f;

__device__ __forceinline__ void chol_inv_df_block(const double *__restrict__ G, int k, int n, int always_shift,
                                                  double *__restrict__ Rinv, DFp *Sd /* 3 k x k shared */) {
    __shared__ double shift, gsc, rsc;
    DFp *Rd = Sd + k * k, *Xd = Rd + k * k;
    const int tid = threadIdx.x, warp = tid >> 5, wl = tid & 31, kk2 = k * k;
    if (tid == 0) {
        double tr = 0.0, mx = 0.0;
        for (int i = 0; i < k; ++i) {
            tr += G[i * k + i];
            mx = fmax(mx, fabs(G[i * k + i]));
        }
        int x = 0;
        if (mx > 0.0 && isfinite(mx)) frexp(mx, &x);
        const int e = (x + 1) >> 1;  // ceil(x / 2): mx 4^-e in [1/4, 1)
        gsc = ldexp(1.0, -2 * e);
        rsc = ldexp(1.0, -e);
        shift = 11.0 * ((double)n * k + (double)k * (k + 1)) * 0x1p-47 * tr * gsc;
    }
    // inverse: teams of `tw` lanes (a power of two <= 32) share a row's sum
    int tw = 1;
    while (tw < 32 && tw * 2 * k <= kCholThreads) tw *= 2;
    const int team = tid / tw, lane = tid % tw, teams = kCholThreads / tw;
    {
        __syncthreads();
        for (int e = tid; e < kk2; e += kCholThreads) {
            const int i = e / k, j = e - i * k;
            Sd[e] = dfp_of(G[e] * gsc + (always_shift && i == j ? shift : 0.0));
        }
        __syncthreads();
        for (int j = 0; j < k; ++j) {
            DFp d = Sd[j * k + j];  // the same value in every thread
            if (!(d.hi > (always_shift ? 0.f : kPivotFloor)) || !isfinite(d.hi))
                d = always_shift ? DFp{1.f, 0.f} : DFp{kPivotFloor, 0.f};
            const DFp inv = dfp_rsqrt(d);  // 1 / R[j][j]
            const DFp r = dfp_mul(d, inv);  // R[j][j]
            for (int c = j + tid; c < k; c += kCholThreads) Rd[j * k + c] = c == j ? r : dfp_mul(Sd[j * k + c], inv);
            // trailing upper triangle: a warp per row (rows j+1+warp, +8, ...), lanes over columns
            {
                DFp msa[kRowsPerWarp], sv[kRowsPerWarp][2];
                const DFp r0 = wl + 0 < k ? dfp_mul(Sd[j * k + wl], inv) : DFp{0.f, 0.f};
                const DFp r1 = wl + 32 < k ? dfp_mul(Sd[j * k + wl + 32], inv) : DFp{0.f, 0.f};
#pragma unroll
                for (int q = 0; q < kRowsPerWarp; ++q) {
                    const int a = j + 1 + warp + q * (kCholThreads / 32);
                    if (a < k) {
                        const DFp sa = dfp_mul(Sd[j * k + a], inv);
                        msa[q] = DFp{-sa.hi, -sa.lo};
                        sv[q][0] = wl >= a && wl < k ? Sd[a * k + wl] : DFp{0.f, 0.f};
                        sv[q][1] = wl + 32 >= a && wl + 32 < k ? Sd[a * k + wl + 32] : DFp{0.f, 0.f};
                    }
                }
#pragma unroll
                for (int q = 0; q < kRowsPerWarp; ++q) {
                    const int a = j + 1 + warp + q * (kCholThreads / 32);
                    if (a < k) {
                        if (wl >= a && wl < k) Sd[a * k + wl] = dfp_add(sv[q][0], dfp_mul(msa[q], r0));
                        if (wl + 32 >= a && wl + 32 < k) Sd[a * k + wl + 32] = dfp_add(sv[q][1], dfp_mul(msa[q], r1));
                    }
                }
            }
            // column j of R^-1: X[i][j] = -(sum over l in [i, j) of X[i][l] R[l][j]) / R[j][j]
            for (int i0 = 0; i0 < j; i0 += teams) {
                const int i = i0 + team;
                DFp sum = {0.f, 0.f};
                if (i < j)
                    for (int l = i + lane; l < j; l += tw) sum = dfp_add(sum, dfp_mul(Xd[i * k + l], Rd[l * k + j]));
                for (int o = tw >> 1; o > 0; o >>= 1) {
                    const DFp other = {__shfl_down_sync(0xffffffffu, sum.hi, o, tw),
                                       __shfl_down_sync(0xffffffffu, sum.lo, o, tw)};
                    sum = dfp_add(sum, other);
                }
                if (i < j && lane == 0) {
                    const DFp v = dfp_mul(sum, inv);
                    Xd[i * k + j] = DFp{-v.hi, -v.lo};
                }
            }
            if (tid == 0) Xd[j * k + j] = inv;
            __syncthreads();
        }
    }
    const double r = rsc;
    for (int e = tid; e < kk2; e += kCholThreads) {
        const int i = e / k, j = e - i * k;
        Rinv[e] = j >= i ? dfp_val(Xd[e]) * r : 0.0;
    }
}

// A Gram matrix of a panel whose columns are already orthonormal to within kNearIdentity (the
// third CholeskyQR step, and often the second) skips the factorization: with G = I + E, R = I + F
// for F the upper triangle of E with its diagonal halved has R^T R = I + E + F^T F, so R^-1 = I - F
// to O(|E|^2) < k 2^-56, and Q = A (I - F) has Q^T Q = I + O(|E|^2).
constexpr double kNearIdentity = 0x1p-28;

// Largest |G - I| entry, block-wide: every thread gets it (a NaN counts as infinite).
__device__ __forceinline__ double gram_defect(const double *__restrict__ G, int k) {
    __shared__ double buf[32];
    double m = 0.0;
    for (int e = threadIdx.x; e < k * k; e += blockDim.x) {
        const int i = e / k, c = e - i * k;
        const double d = fabs(G[e] - (i == c ? 1.0 : 0.0));
        m = d <= m ? m : (d == d ? d : INFINITY);
    }
    m = warp_max(m);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) buf[threadIdx.x >> 5] = m;
    __syncthreads();
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t = fmax(t, buf[w]);
    return t;
}

// R^-1 = I - F (upper triangular, row-major) for a G within kNearIdentity of the identity.
__device__ __forceinline__ void rinv_near_identity(const double *__restrict__ G, int k, double *__restrict__ out) {
    for (int e = threadIdx.x; e < k * k; e += blockDim.x) {
        const int i = e / k, c = e - i * k;
        out[e] = c < i ? 0.0 : (c == i ? 1.0 - 0.5 * (G[e] - 1.0) : -G[e]);
    }
}

__global__ void __launch_bounds__(kCholThreads) chol_inv_kernel(const double *__restrict__ G, int k, int n,
                                                                int always_shift, double *__restrict__ Rinv) {
    extern __shared__ double cS[];  // k x k
    if (!always_shift && gram_defect(G, k) < kNearIdentity) {
        rinv_near_identity(G, k, Rinv);
        return;
    }
    chol_inv_block(G, k, n, always_shift, Rinv, cS);
}

__global__ void __launch_bounds__(kCholThreads) chol_inv_df_kernel(const double *__restrict__ G, int k, int n,
                                                                   int always_shift, double *__restrict__ Rinv) {
    extern __shared__ DFp cSd[];  // 3 k x k pairs
    if (!always_shift && gram_defect(G, k) < kNearIdentity) {
        rinv_near_identity(G, k, Rinv);
        return;
    }
    chol_inv_df_block(G, k, n, always_shift, Rinv, cSd);
}

// The whole shifted CholeskyQR3 of the panel `a` (n x k) in one cooperative launch: per step the
// row-block Gram partials, their sum, the k x k factor and inverse (block 0; the other blocks wait
// at the grid barrier) or, for a Gram within kNearIdentity of I, its first-order inverse (every
// block, no barrier), and A <- A R^-1, with a grid-wide barrier between stages; after the third
// step the result is copied back into `a`.  The same stage bodies as the separate kernels, on the
// same row blocks, so the result is bit-identical to them; it replaces 12 launches (and the copy)
// per QR, whose launch gaps were most of a small panel's QR time.
__global__ void __launch_bounds__(256) qr_fused_kernel(double *__restrict__ a, double *__restrict__ work, int n, int k,
                                                       int nparts, int rpb, double *__restrict__ part,
                                                       double *__restrict__ G, double *__restrict__ Rinv, int df) {
    extern __shared__ __align__(16) unsigned char qsm[];
    cg::grid_group grid = cg::this_grid();
    double *src = a, *dst = work;
    for (int step = 0; step < 3; ++step) {
        if ((int)blockIdx.x < nparts) atb_block(src, src, n, k, rpb, part, blockIdx.x, (double *)qsm, true);
        grid.sync();
        sum_parts_body(part, nparts, k * k, G);
        grid.sync();
        // every block reads the same G, so all take the same branch (and the same grid barriers)
        if (step > 0 && gram_defect(G, k) < kNearIdentity) {
            rinv_near_identity(G, k, (double *)qsm);
            __syncthreads();
            apply_w_body(src, nullptr, n, k, dst, (double *)qsm, true);
        } else {
            if (blockIdx.x == 0) {
                if (df) chol_inv_df_block(G, k, n, step == 0 ? 1 : 0, Rinv, (DFp *)qsm);
                else chol_inv_block(G, k, n, step == 0 ? 1 : 0, Rinv, (double *)qsm);
            }
            grid.sync();
            apply_w_body(src, Rinv, n, k, dst, (double *)qsm, true);
        }
        grid.sync();
        double *t = src;
        src = dst;
        dst = t;
    }
    // three steps: a -> work -> a -> work
    const int64_t total = (int64_t)n * k;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x)
        a[e] = src[e];
}

// ------------------------------------------------------------------ shifted CholeskyQR3
// Thin QR of the n x k panel A (in place, Q only) by three CholeskyQR steps (Fukaya, Kannan,
// Nakatsukasa, Yamamoto, Yanagisawa, "Shifted Cholesky QR for computing the QR factorization of
// ill-conditioned matrices", SIAM J. Sci. Comput. 42 (2020)): G = A^T A, R = chol(G + s I),
// A <- A R^-1, with the shift s = 11 (n k + k (k + 1)) u ||A||_F^2 in the first step, which keeps
// the Cholesky factorization defined for condition numbers up to ~1/u (the reference's start
// block has ~5e9), and then two plain steps (CholeskyQR2) that restore orthogonality to O(u).
// The panel is read three times and written three times, and no step needs the host.  Q spans the same column space as the
// reference's dgeqrf + dorgqr (methods.cpp:947-961); its columns may differ in sign, which the
// Rayleigh-Ritz step (methods.cpp:972-1007) absorbs: the Ritz vectors come out with the
// eigensolver's signs either way.
dpca_status launch_qr(Handle *h, double *a) {
    const int n = h->n_ind, k = h->k;
    const SmallLayout L{k};
    double *G = h->small + L.B(), *Rinv = h->small + L.W();  // free until the Rayleigh-Ritz step
    const bool df = k <= kEigDfMaxK;
    int nparts = 0, rpb = 0;
    gram_split(h, n, &nparts, &rpb);
    // the k x k factor's working set: S, R and R^-1 as pairs (double-float), or S in FP64
    const size_t smem_f = df ? (size_t)3 * k * k * sizeof(DFp) : (size_t)k * k * sizeof(double);
    const size_t smem = std::max<size_t>((size_t)2 * 32 * k * sizeof(double), smem_f);
    // one cooperative launch while the grid (the Gram's row blocks, at least one block per SM for
    // the apply) fits on the device at once; the separate kernels otherwise
    if (h->qr_coresident == 0) {
        int per_sm = 0;
        DPCA_TRY(allow_max_smem((const void *)qr_fused_kernel));
        DPCA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, qr_fused_kernel, 256, smem));
        h->qr_coresident = std::max(1, per_sm) * h->sm_count;
        int coop = 0;
        DPCA_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, h->device));
        const char *mode = getenv("DPCA_QR_KERNELS");
        if (!coop || per_sm < 1 || (mode && strcmp(mode, "separate") == 0)) h->qr_coresident = -1;
    }
    const int grid = std::max(nparts, h->sm_count);
    if (h->qr_coresident > 0 && grid <= h->qr_coresident) {
        ScopedLaunch t(&h->clock, h->stream, "qr_fused");
        double *work = h->work;
        int ni = n, ki = k, npi = nparts, rpbi = rpb, dfi = df ? 1 : 0;
        double *red = h->red;
        void *args[] = {&a, &work, &ni, &ki, &npi, &rpbi, &red, &G, &Rinv, &dfi};
        DPCA_CUDA(cudaLaunchCooperativeKernel((const void *)qr_fused_kernel, dim3(grid), dim3(256), args, smem,
                                              h->stream));
        return DPCA_OK;
    }
    DPCA_TRY(allow_max_smem((const void *)apply_w_kernel));
    DPCA_TRY(allow_max_smem((const void *)chol_inv_kernel));
    DPCA_TRY(allow_max_smem((const void *)chol_inv_df_kernel));
    const size_t smem_g = (size_t)k * k * sizeof(double);
    const int64_t total = (int64_t)n * k;
    const int agrid = (int)std::min<int64_t>((total + 255) / 256, (int64_t)h->sm_count * 4);
    double *src = a, *dst = h->work;
    for (int step = 0; step < 3; ++step) {
        DPCA_TRY(atb_timed(h, src, src, n, G, "qr_gram", "qr_gram_sum"));
        {
            ScopedLaunch t(&h->clock, h->stream, "qr_chol");
            if (df)
                chol_inv_df_kernel<<<1, kCholThreads, smem_f, h->stream>>>(G, k, n, step == 0 ? 1 : 0, Rinv);
            else
                chol_inv_kernel<<<1, kCholThreads, smem_g, h->stream>>>(G, k, n, step == 0 ? 1 : 0, Rinv);
            DPCA_CUDA(cudaGetLastError());
        }
        {
            ScopedLaunch t(&h->clock, h->stream, "qr_apply");
            apply_w_kernel<<<agrid, 256, smem_g, h->stream>>>(src, Rinv, n, k, dst, 1);
            DPCA_CUDA(cudaGetLastError());
        }
        std::swap(src, dst);
    }
    // three steps: a -> work -> a -> work
    DPCA_CUDA(cudaMemcpyAsync(a, src, (size_t)total * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    return DPCA_OK;
}

// ------------------------------------------------------------------ convergence
// part[b][j] = sum over block b's rows of old[i][j] * cur[i][j], j < nsv.
__global__ void __launch_bounds__(256) coldots_kernel(const double *__restrict__ a, const double *__restrict__ b, int n,
                                                      int k, int nsv, int rpb, double *__restrict__ part) {
    __shared__ double red[32];
    int r0 = blockIdx.x * rpb, r1 = min(n, r0 + rpb);
    for (int j = 0; j < nsv; ++j) {
        double s = 0.0;
        for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) s = fma(a[(size_t)i * k + j], b[(size_t)i * k + j], s);
        s = block_sum(s, red);
        if (threadIdx.x == 0) part[(size_t)blockIdx.x * nsv + j] = s;
    }
}

// Single block: sigma_j = sqrt(w_j) (j < nsv), delta = sum sigma, then crit 0/1/2 when ii > 0.
// small.crit: [0] criterion value (NaN at ii = 0), [1] stop flag, [2] delta, [3] previous delta.
__global__ void criterion_kernel(double *__restrict__ small_, int k, int nsv, int crit, double tol, int ii,
                                 const double *__restrict__ dots_part, int nparts) {
    SmallLayout L{k};
    double *w = small_ + L.w(), *sig = small_ + L.sigma(), *old = small_ + L.sigma_old(), *cr = small_ + L.crit();
    if (threadIdx.x != 0) return;
    double delta = 0.0;
    for (int j = 0; j < nsv; ++j) {
        sig[j] = sqrt(w[j]);
        delta += sig[j];
    }
    double val = nan(""), stop = 0.0;
    if (ii > 0) {
        if (crit == 0) {
            val = fabs(cr[3] - delta) / delta;
            stop = val <= tol ? 1.0 : 0.0;
        } else if (crit == 1) {
            int conv = 0;
            for (int j = 0; j < nsv; ++j)
                if (fabs((sig[j] - old[j]) / sig[j]) <= tol) conv++;
            val = conv;
            stop = conv == nsv ? 1.0 : 0.0;
        } else if (crit == 2) {
            double mev = 0.0;
            for (int j = 0; j < nsv; ++j) {
                double d = 0.0;
                for (int p = 0; p < nparts; ++p) d += dots_part[(size_t)p * nsv + j];
                mev += d * d;
            }
            mev /= nsv;
            val = 1.0 - mev;
            stop = val <= tol ? 1.0 : 0.0;
        }
    }
    cr[0] = val;
    cr[1] = stop;
    cr[2] = delta;
    cr[3] = delta;
    for (int j = 0; j < nsv; ++j) old[j] = sig[j];
}

dpca_status launch_sigma_and_criterion(Handle *h, int nsv, int crit, double tol, int ii, const double *old,
                                       const double *omega) {
    int nparts = 0;
    if (crit == 2 && ii > 0) {
        ScopedLaunch t(&h->clock, h->stream, "coldots");
        nparts = std::max(1, std::min(2 * h->sm_count, ceil_div(h->n_ind, 256)));
        nparts = (int)std::min<int64_t>(nparts, (int64_t)(h->red_elems / std::max(1, nsv)));
        int rpb = ceil_div(h->n_ind, nparts);
        nparts = ceil_div(h->n_ind, rpb);
        coldots_kernel<<<nparts, 256, 0, h->stream>>>(old, omega, h->n_ind, h->k, nsv, rpb, h->red);
        DPCA_CUDA(cudaGetLastError());
    }
    ScopedLaunch t(&h->clock, h->stream, "criterion");
    criterion_kernel<<<1, 32, 0, h->stream>>>(h->small, h->k, nsv, crit, tol, ii, h->red, nparts);
    DPCA_CUDA(cudaGetLastError());
    return DPCA_OK;
}

}  // namespace dpca

using namespace dpca;

extern "C" dpca_status dpca_sym_eig_device(int device, int k, const double *b, double *w, double *W) {
    clear_error();
    if (k < 1 || k > kMaxNrhs || !b || !w || !W) {
        set_error("dpca_sym_eig_device: need 1 <= k <= %d and non-null arrays", kMaxNrhs);
        return DPCA_ERR_INVALID;
    }
    DPCA_CUDA(cudaSetDevice(device));
    const size_t kk = (size_t)k * k;
    double *d = nullptr;
    int *flags = nullptr;
    DPCA_CUDA(cudaMalloc(&d, (3 * kk + k) * sizeof(double)));
    if (cudaMalloc(&flags, 16 * sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(d);
        set_error("dpca_sym_eig_device: device allocation failed");
        return DPCA_ERR_NOMEM;
    }
    dpca_status st = DPCA_OK;
    int hflags[16] = {0};
    cudaError_t e = cudaSuccess;
    if (st == DPCA_OK) {
        // d: B | W | V (global, used for k > kEigSmemK) | w
        e = cudaMemcpy(d, b, kk * sizeof(double), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemset(flags, 0, 16 * sizeof(int));
        if (e == cudaSuccess) {
            st = eig_launch(d, k, d + kk, d + 3 * kk, d + 2 * kk, flags, 0);
            if (st != DPCA_OK) {
                cudaFree(d);
                cudaFree(flags);
                return st;
            }
        }
        if (e == cudaSuccess) e = cudaMemcpy(W, d + kk, kk * sizeof(double), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(w, d + 3 * kk, (size_t)k * sizeof(double), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(hflags, flags, sizeof(hflags), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) {
            set_error("dpca_sym_eig_device: %s", cudaGetErrorString(e));
            st = DPCA_ERR_CUDA;
        } else if (hflags[1]) {
            set_error("dpca_sym_eig_device: Jacobi did not converge");
            st = DPCA_ERR_NUMERIC;
        }
    }
    cudaFree(d);
    cudaFree(flags);
    return st;
}
