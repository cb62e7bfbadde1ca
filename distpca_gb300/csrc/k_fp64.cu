// Plain FP64 pass: the two products of the pass lambda (methods.cpp:853-863, 910-922)
//   Y = X Omega          (fp64_xw_kernel, reduce over individuals)
//   Z = X^T Y            (fp64_xty_kernel, split-K over SNPs + fixed-order reduction)
// with X decoded on the fly from the packed codes through the per-SNP LUT, whose entries are
// bit-identical to the reference's standardized values.  Every product and sum is FP64; the
// reduction order is fixed, so results are deterministic run to run.
#include <algorithm>

#include "common.cuh"
#include "dpca_internal.h"

namespace dpca {

__device__ __forceinline__ double lut_pick(uint32_t code, double l0, double l1, double l2, double l3) {
    double lo = (code & 1u) ? l1 : l0;
    double hi = (code & 1u) ? l3 : l2;
    return (code & 2u) ? hi : lo;
}

// Block: 64 SNP rows x all k columns; thread -> (row r = tid/4, columns cg + 4j).
template <int MAXC>
__global__ void __launch_bounds__(256) fp64_xw_kernel(const uint8_t *__restrict__ P, int64_t pitch,
                                                      const double *__restrict__ lut, int n_ind, int n_snp, int k,
                                                      const double *__restrict__ omega, double *__restrict__ y) {
    extern __shared__ double om[];  // [64][k]
    __shared__ uint32_t pk[64][5];
    int tid = threadIdx.x, r = tid >> 2, cg = tid & 3;
    int64_t s = (int64_t)blockIdx.x * 64 + r;
    double l0 = 0, l1 = 0, l2 = 0, l3 = 0;
    if (s < n_snp) {
        l0 = lut[4 * s + 0];
        l1 = lut[4 * s + 1];
        l2 = lut[4 * s + 2];
        l3 = lut[4 * s + 3];
    }
    double acc[MAXC];
#pragma unroll
    for (int j = 0; j < MAXC; ++j) acc[j] = 0.0;
    for (int i0 = 0; i0 < n_ind; i0 += 64) {
        {
            int rr = tid >> 2, w = tid & 3;
            int64_t sr = (int64_t)blockIdx.x * 64 + rr;
            pk[rr][w] = sr < n_snp ? *reinterpret_cast<const uint32_t *>(P + sr * pitch + (i0 >> 2) + 4 * w) : 0u;
        }
        for (int e = tid; e < 64 * k; e += 256) {
            int ii = e / k, c = e - ii * k;
            om[e] = (i0 + ii < n_ind) ? omega[(int64_t)(i0 + ii) * k + c] : 0.0;
        }
        __syncthreads();
#pragma unroll 4
        for (int ii = 0; ii < 64; ++ii) {
            uint32_t code = (pk[r][ii >> 4] >> (2 * (ii & 15))) & 3u;
            double x = lut_pick(code, l0, l1, l2, l3);
            const double *orow = om + ii * k;
#pragma unroll
            for (int j = 0; j < MAXC; ++j) {
                int c = cg + 4 * j;
                if (c < k) acc[j] = fma(x, orow[c], acc[j]);
            }
        }
        __syncthreads();
    }
    if (s < n_snp) {
#pragma unroll
        for (int j = 0; j < MAXC; ++j) {
            int c = cg + 4 * j;
            if (c < k) y[s * k + c] = acc[j];
        }
    }
}

// Block: 128 individuals x all k columns over one SNP split; thread -> (individual il = tid%128,
// columns cg + 4j, cg = tid/128).
template <int MAXC>
__global__ void __launch_bounds__(512) fp64_xty_kernel(const uint8_t *__restrict__ P, int64_t pitch,
                                                       const double *__restrict__ lut, int n_ind, int n_snp, int k,
                                                       const double *__restrict__ y, double *__restrict__ partial,
                                                       int snps_per_split) {
    extern __shared__ double ys[];  // [32][k]
    __shared__ uint32_t pk[32][9];
    __shared__ double lt[32][4];
    int tid = threadIdx.x, il = tid & 127, cg = tid >> 7;
    int i = blockIdx.x * 128 + il;
    int split = blockIdx.y;
    int sb = split * snps_per_split, se = min(n_snp, sb + snps_per_split);
    double acc[MAXC];
#pragma unroll
    for (int j = 0; j < MAXC; ++j) acc[j] = 0.0;
    int64_t byte0 = (int64_t)blockIdx.x * 32;
    for (int s0 = sb; s0 < se; s0 += 32) {
        if (tid < 256) {
            int rr = tid >> 3, w = tid & 7;
            int s = s0 + rr;
            pk[rr][w] = s < se ? *reinterpret_cast<const uint32_t *>(P + (int64_t)s * pitch + byte0 + 4 * w) : 0u;
        } else if (tid < 384) {
            int e = tid - 256, rr = e >> 2;
            int s = s0 + rr;
            lt[rr][e & 3] = s < se ? lut[4 * (int64_t)s + (e & 3)] : 0.0;
        }
        for (int e = tid; e < 32 * k; e += 512) {
            int rr = e / k;
            int s = s0 + rr;
            ys[e] = s < se ? y[(int64_t)s * k + (e - rr * k)] : 0.0;
        }
        __syncthreads();
#pragma unroll 4
        for (int ss = 0; ss < 32; ++ss) {
            uint32_t code = (pk[ss][il >> 4] >> (2 * (il & 15))) & 3u;
            double x = lt[ss][code];
            const double *yrow = ys + ss * k;
#pragma unroll
            for (int j = 0; j < MAXC; ++j) {
                int c = cg + 4 * j;
                if (c < k) acc[j] = fma(x, yrow[c], acc[j]);
            }
        }
        __syncthreads();
    }
    if (i < n_ind) {
        double *out = partial + ((int64_t)split * n_ind + i) * k;
#pragma unroll
        for (int j = 0; j < MAXC; ++j) {
            int c = cg + 4 * j;
            if (c < k) out[c] = acc[j];
        }
    }
}

// z[e] = sum over splits of partial[split][e], in split order.
__global__ void reduce_splits_kernel(const double *__restrict__ partial, int64_t elems, int splits,
                                     double *__restrict__ z) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < elems; e += (int64_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int p = 0; p < splits; ++p) s += partial[(int64_t)p * elems + e];
        z[e] = s;
    }
}

template <int MAXC>
static void xw_launch(Handle *h, const double *omega, double *y) {
    size_t smem = (size_t)64 * h->k * sizeof(double);
    // opt in above the default 48 KB (static shared memory counts against it as well)
    cudaFuncSetAttribute(fp64_xw_kernel<MAXC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    fp64_xw_kernel<MAXC><<<ceil_div(h->n_snp, 64), 256, smem, h->stream>>>(h->P, h->pitch, h->lut, h->n_ind,
                                                                            h->n_snp, h->k, omega, y);
}

dpca_status launch_fp64_xw(Handle *h, const double *omega, double *y) {
    ScopedLaunch t(&h->clock, h->stream, "fp64_xw");
    int mc = (h->k + 3) / 4;
    if (mc <= 4) xw_launch<4>(h, omega, y);
    else if (mc <= 8) xw_launch<8>(h, omega, y);
    else if (mc <= 16) xw_launch<16>(h, omega, y);
    else xw_launch<32>(h, omega, y);
    DPCA_CUDA(cudaGetLastError());
    return DPCA_OK;
}

static int xty_splits(const Handle *h) {
    int tiles = ceil_div(h->n_ind, 128);
    int want = std::max(1, ceil_div(4 * h->sm_count, tiles));
    int maxs = std::max(1, ceil_div(h->n_snp, 32));
    int s = std::min(want, maxs);
    // bounded by the partial buffer
    int64_t cap = (int64_t)(h->partial_elems / ((size_t)h->n_ind * h->k));
    return (int)std::max<int64_t>(1, std::min<int64_t>(s, cap));
}

template <int MAXC>
static void xty_launch(Handle *h, const double *y, int splits, int sps) {
    size_t smem = (size_t)32 * h->k * sizeof(double);
    cudaFuncSetAttribute(fp64_xty_kernel<MAXC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    dim3 grid(ceil_div(h->n_ind, 128), splits);
    fp64_xty_kernel<MAXC><<<grid, 512, smem, h->stream>>>(h->P, h->pitch, h->lut, h->n_ind, h->n_snp, h->k, y,
                                                           h->partial, sps);
}

dpca_status launch_fp64_xty(Handle *h, const double *y, double *z) {
    int splits = xty_splits(h);
    int sps = ceil_div(h->n_snp, splits);
    sps = ((sps + 31) / 32) * 32;
    splits = ceil_div(h->n_snp, sps);
    {
        ScopedLaunch t(&h->clock, h->stream, "fp64_xty");
        int mc = (h->k + 3) / 4;
        if (mc <= 4) xty_launch<4>(h, y, splits, sps);
        else if (mc <= 8) xty_launch<8>(h, y, splits, sps);
        else if (mc <= 16) xty_launch<16>(h, y, splits, sps);
        else xty_launch<32>(h, y, splits, sps);
        DPCA_CUDA(cudaGetLastError());
    }
    {
        ScopedLaunch t(&h->clock, h->stream, "reduce_splits");
        int64_t elems = (int64_t)h->n_ind * h->k;
        int grid = (int)std::min<int64_t>((elems + 255) / 256, (int64_t)h->sm_count * 8);
        reduce_splits_kernel<<<grid, 256, 0, h->stream>>>(h->partial, elems, splits, z);
        DPCA_CUDA(cudaGetLastError());
    }
    return DPCA_OK;
}

}  // namespace dpca
