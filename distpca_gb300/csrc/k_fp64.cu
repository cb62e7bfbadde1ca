// Plain FP64 pass: the two products of the pass lambda (methods.cpp:853-863, 910-922)
//   Y = X Omega          (fp64_xw_kernel, reduce over individuals)
//   Z = X^T Y            (fp64_xty_kernel, split-K over SNPs + fixed-order reduction)
// with X decoded on the fly from the packed codes through the per-SNP LUT, whose entries are
// bit-identical to the reference's standardized values.  Every product and sum is FP64; the
// reduction order is fixed, so results are deterministic run to run.
#include <algorithm>
#include <mutex>

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

// z[e] = sum over splits of partial[split][e], in split order (added to z when accumulating,
// as the streamed blocks do).
__global__ void reduce_splits_kernel(const double *__restrict__ partial, int64_t elems, int splits,
                                     double *__restrict__ z, int accumulate = 0) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < elems; e += (int64_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int p = 0; p < splits; ++p) s += partial[(int64_t)p * elems + e];
        z[e] = accumulate ? z[e] + s : s;
    }
}

template <int MAXC>
static dpca_status xw_launch(Handle *h, const double *omega, double *y) {
    size_t smem = (size_t)64 * h->k * sizeof(double);
    // opt in above the default 48 KB (static shared memory counts against it as well)
    DPCA_TRY(allow_max_smem((const void *)fp64_xw_kernel<MAXC>));
    fp64_xw_kernel<MAXC><<<ceil_div(h->n_snp, 64), 256, smem, h->stream>>>(h->P, h->pitch, h->lut, h->n_ind,
                                                                            h->n_snp, h->k, omega, y);
    return DPCA_OK;
}

dpca_status launch_fp64_xw(Handle *h, const double *omega, double *y) {
    ScopedLaunch t(&h->clock, h->stream, "fp64_xw");
    int mc = (h->k + 3) / 4;
    if (mc <= 4) DPCA_TRY(xw_launch<4>(h, omega, y));
    else if (mc <= 8) DPCA_TRY(xw_launch<8>(h, omega, y));
    else if (mc <= 16) DPCA_TRY(xw_launch<16>(h, omega, y));
    else DPCA_TRY(xw_launch<32>(h, omega, y));
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
static dpca_status xty_launch(Handle *h, const double *y, int splits, int sps) {
    size_t smem = (size_t)32 * h->k * sizeof(double);
    DPCA_TRY(allow_max_smem((const void *)fp64_xty_kernel<MAXC>));
    dim3 grid(ceil_div(h->n_ind, 128), splits);
    fp64_xty_kernel<MAXC><<<grid, 512, smem, h->stream>>>(h->P, h->pitch, h->lut, h->n_ind, h->n_snp, h->k, y,
                                                           h->partial, sps);
    return DPCA_OK;
}

dpca_status launch_fp64_xty(Handle *h, const double *y, double *z) {
    int splits = xty_splits(h);
    int sps = ceil_div(h->n_snp, splits);
    sps = ((sps + 31) / 32) * 32;
    splits = ceil_div(h->n_snp, sps);
    {
        ScopedLaunch t(&h->clock, h->stream, "fp64_xty");
        int mc = (h->k + 3) / 4;
        if (mc <= 4) DPCA_TRY(xty_launch<4>(h, y, splits, sps));
        else if (mc <= 8) DPCA_TRY(xty_launch<8>(h, y, splits, sps));
        else if (mc <= 16) DPCA_TRY(xty_launch<16>(h, y, splits, sps));
        else DPCA_TRY(xty_launch<32>(h, y, splits, sps));
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

namespace dpca {

// ------------------------------------------------------------------ allocation-free pass
// dpca_pass_fp64_noalloc: the plain FP64 pass Z = X^T (X Omega) on device buffers the caller
// owns, for callers that must not have a library allocate device memory -- applications that
// hand out all device memory from their own fixed-budget pool, and latency-sensitive loops in
// which cudaMalloc/cudaFree (which can synchronise the device) are not acceptable.  Its working
// buffers -- per-SNP counts, mean, sd and LUT, Y = X Omega, and the split partials of X^T Y --
// are carved out of one file-scope device array of kNoAllocScratchBytes, which every GPU that
// loads this library holds until the process exits.
//
// In host code the array's name is only a host-side stand-in: its device address is obtained
// once per device, with that device current, by cudaGetSymbolAddress on the first call made on
// that device, which also raises the shared-memory limits of every kernel instance the call may
// launch (so that first call should come before any stream capture).  The address belongs to the
// CUDA context it was looked up in; a call in another context (for instance after
// cudaDeviceReset) repeats this set-up, and that call too belongs outside capture.  Every call shares
// the array and it keeps the last call's contents; nothing in it needs to start at zero (each
// kernel writes every element it later reads).  Calls whose work overlaps on the GPU -- on
// different streams or from different threads -- race on the array, so callers serialise them.
constexpr size_t kNoAllocScratchBytes = (size_t)32 << 20;  // 32 MiB per device
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of the scratch array in the calling thread's current CUDA context.  The address
// belongs to that context: it is looked up again (cudaGetSymbolAddress) whenever the context id
// differs from the one it was cached for -- another device, a context the caller made current,
// or the new primary context after cudaDeviceReset -- and the kernels' shared-memory limits
// are raised in the same one-time set-up, so that no later call changes a kernel attribute.
static std::mutex g_noalloc_mu;
struct NoAllocSlot {
    unsigned long long ctx = 0;
    void *ptr = nullptr;
};
static NoAllocSlot g_noalloc_slot[kNoAllocMaxDevices];

static dpca_status noalloc_kernel_setup() {
    const void *fns[] = {(const void *)fp64_xw_kernel<4>,   (const void *)fp64_xw_kernel<8>,
                         (const void *)fp64_xw_kernel<16>,  (const void *)fp64_xw_kernel<32>,
                         (const void *)fp64_xty_kernel<4>,  (const void *)fp64_xty_kernel<8>,
                         (const void *)fp64_xty_kernel<16>, (const void *)fp64_xty_kernel<32>};
    for (const void *f : fns) DPCA_TRY(allow_max_smem(f));
    return DPCA_OK;
}

static dpca_status noalloc_scratch(void **out) {
    int dev = 0;
    DPCA_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices) {
        set_error("allocation-free pass: device ordinal %d is above %d", dev, kNoAllocMaxDevices - 1);
        return DPCA_ERR_UNSUPPORTED;
    }
    unsigned long long ctx = 0;
    DPCA_TRY(current_context_id(&ctx));
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    NoAllocSlot &slot = g_noalloc_slot[dev];
    if (slot.ctx != ctx || !slot.ptr) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            set_error("allocation-free pass: cudaGetSymbolAddress of the scratch array failed on device %d: %s", dev,
                      cudaGetErrorString(e));
            return DPCA_ERR_CUDA;
        }
        DPCA_TRY(noalloc_kernel_setup());
        slot.ctx = ctx;
        slot.ptr = p;
    }
    *out = slot.ptr;
    return DPCA_OK;
}

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

template <int MAXC>
static dpca_status xw_launch_raw(const uint8_t *P, int64_t pitch, const double *lut, int n_ind, int n_snp, int k,
                                 const double *omega, double *y, cudaStream_t st) {
    size_t smem = (size_t)64 * k * sizeof(double);
    DPCA_TRY(allow_max_smem((const void *)fp64_xw_kernel<MAXC>));
    fp64_xw_kernel<MAXC><<<ceil_div(n_snp, 64), 256, smem, st>>>(P, pitch, lut, n_ind, n_snp, k, omega, y);
    DPCA_CUDA(cudaGetLastError());
    return DPCA_OK;
}

template <int MAXC>
static dpca_status xty_launch_raw(const uint8_t *P, int64_t pitch, const double *lut, int n_ind, int n_snp, int k,
                                  const double *y, double *partial, int splits, int sps, cudaStream_t st) {
    size_t smem = (size_t)32 * k * sizeof(double);
    DPCA_TRY(allow_max_smem((const void *)fp64_xty_kernel<MAXC>));
    dim3 grid(ceil_div(n_ind, 128), splits);
    fp64_xty_kernel<MAXC><<<grid, 512, smem, st>>>(P, pitch, lut, n_ind, n_snp, k, y, partial, sps);
    DPCA_CUDA(cudaGetLastError());
    return DPCA_OK;
}

// Both products' launchers for the subspace width k (the kernel instance covers ceil(k / 4) column
// groups of four).
static dpca_status xw_dispatch(const uint8_t *P, int64_t pitch, const double *lut, int n_ind, int n_snp, int k,
                               const double *omega, double *y, cudaStream_t st) {
    const int mc = (k + 3) / 4;
    if (mc <= 4) return xw_launch_raw<4>(P, pitch, lut, n_ind, n_snp, k, omega, y, st);
    if (mc <= 8) return xw_launch_raw<8>(P, pitch, lut, n_ind, n_snp, k, omega, y, st);
    if (mc <= 16) return xw_launch_raw<16>(P, pitch, lut, n_ind, n_snp, k, omega, y, st);
    return xw_launch_raw<32>(P, pitch, lut, n_ind, n_snp, k, omega, y, st);
}

static dpca_status xty_dispatch(const uint8_t *P, int64_t pitch, const double *lut, int n_ind, int n_snp, int k,
                                const double *y, double *partial, int splits, int sps, cudaStream_t st) {
    const int mc = (k + 3) / 4;
    if (mc <= 4) return xty_launch_raw<4>(P, pitch, lut, n_ind, n_snp, k, y, partial, splits, sps, st);
    if (mc <= 8) return xty_launch_raw<8>(P, pitch, lut, n_ind, n_snp, k, y, partial, splits, sps, st);
    if (mc <= 16) return xty_launch_raw<16>(P, pitch, lut, n_ind, n_snp, k, y, partial, splits, sps, st);
    return xty_launch_raw<32>(P, pitch, lut, n_ind, n_snp, k, y, partial, splits, sps, st);
}

// One streamed block of the FP64 pass: Y_b = X_b Omega into h->y (blk x k), then
// z (+)= X_b^T Y_b through split partials, rows [s0, s0 + ns) of the matrix in buffer Pb[b].
dpca_status launch_fp64_block(Handle *h, int b, int s0, int ns, const double *omega, double *z, bool accumulate) {
    const uint8_t *P = h->Pb[b];
    const double *lut = h->lut + 4 * (size_t)s0;
    const int k = h->k;
    {
        ScopedLaunch t(&h->clock, h->stream, "fp64_xw");
        DPCA_TRY(xw_dispatch(P, h->pitch, lut, h->n_ind, ns, k, omega, h->y, h->stream));
    }
    const int tiles = ceil_div(h->n_ind, 128);
    int splits = std::max(1, ceil_div(4 * h->sm_count, tiles));
    splits = std::min(splits, std::max(1, ceil_div(ns, 32)));
    splits = (int)std::max<int64_t>(1, std::min<int64_t>(splits, (int64_t)(h->partial_elems / ((size_t)h->n_ind * k))));
    int sps = ceil_div(ns, splits);
    sps = (sps + 31) / 32 * 32;
    splits = ceil_div(ns, sps);
    {
        ScopedLaunch t(&h->clock, h->stream, "fp64_xty");
        DPCA_TRY(xty_dispatch(P, h->pitch, lut, h->n_ind, ns, k, h->y, h->partial, splits, sps, h->stream));
    }
    ScopedLaunch t(&h->clock, h->stream, "reduce_splits");
    const int64_t elems = (int64_t)h->n_ind * k;
    const int grid = (int)std::min<int64_t>((elems + 255) / 256, (int64_t)h->sm_count * 8);
    reduce_splits_kernel<<<grid, 256, 0, h->stream>>>(h->partial, elems, splits, z, accumulate ? 1 : 0);
    DPCA_CUDA(cudaGetLastError());
    return DPCA_OK;
}

}  // namespace dpca

extern "C" dpca_status dpca_pass_fp64_noalloc(const uint8_t *packed, int64_t row_stride, int n_ind, int n_snp,
                                              const double *omega, int nrhs, double *z, void *stream) {
    using namespace dpca;
    clear_error();
    if (!packed || !omega || !z || n_ind < 1 || n_snp < 1 || nrhs < 1) {
        set_error("allocation-free pass: null buffer or non-positive size");
        return DPCA_ERR_INVALID;
    }
    if (nrhs > kMaxNrhs) {
        set_error("allocation-free pass: nrhs %d is above %d", nrhs, kMaxNrhs);
        return DPCA_ERR_UNSUPPORTED;
    }
    const int64_t np = ((int64_t)n_ind + 3) / 4;
    const int64_t min_stride = (np + 31) / 32 * 32;  // the kernels read whole 32-byte groups
    if (row_stride < min_stride || row_stride % 16 != 0 || ((uintptr_t)packed & 15u) != 0) {
        set_error("allocation-free pass: rows need a 16-byte aligned base and a stride that is a multiple of 16 "
                  "and at least %lld bytes (got %lld)", (long long)min_stride, (long long)row_stride);
        return DPCA_ERR_INVALID;
    }
    // scratch layout: counts [4 n_snp] int32 | avg, sd [n_snp] | lut [4 n_snp] | y [n_snp k] | partial
    const size_t b_counts = align256((size_t)4 * n_snp * sizeof(int32_t));
    const size_t b_vec = align256((size_t)n_snp * sizeof(double));
    const size_t b_lut = align256((size_t)4 * n_snp * sizeof(double));
    const size_t b_y = align256((size_t)n_snp * nrhs * sizeof(double));
    const size_t b_part = (size_t)n_ind * nrhs * sizeof(double);  // one split
    const size_t fixed = b_counts + 2 * b_vec + b_lut + b_y;
    if (fixed + b_part > kNoAllocScratchBytes) {
        set_error("allocation-free pass: %d individuals x %d SNPs x nrhs %d needs %zu bytes of scratch; the "
                  "limit is %zu (use dpca_pass on a handle for larger inputs)",
                  n_ind, n_snp, nrhs, fixed + b_part, kNoAllocScratchBytes);
        return DPCA_ERR_UNSUPPORTED;
    }
    int dev = 0, sm_count = 1;
    DPCA_CUDA(cudaGetDevice(&dev));
    DPCA_CUDA(cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, dev));
    void *base = nullptr;
    DPCA_TRY(noalloc_scratch(&base));
    unsigned char *sc = (unsigned char *)base;
    int32_t *counts = (int32_t *)sc;
    double *avg = (double *)(sc + b_counts);
    double *sd = (double *)(sc + b_counts + b_vec);
    double *lut = (double *)(sc + b_counts + 2 * b_vec);
    double *y = (double *)(sc + b_counts + 2 * b_vec + b_lut);
    double *partial = (double *)(sc + fixed);
    // split-K of X^T Y: as many splits as fill the SMs, bounded by the scratch left for partials
    const int tiles = ceil_div(n_ind, 128);
    int splits = std::max(1, ceil_div(4 * sm_count, tiles));
    splits = std::min(splits, std::max(1, ceil_div(n_snp, 32)));
    splits = (int)std::min<size_t>((size_t)splits, (kNoAllocScratchBytes - fixed) / b_part);
    int sps = ceil_div(n_snp, splits);
    sps = (sps + 31) / 32 * 32;
    splits = ceil_div(n_snp, sps);
    cudaStream_t st = (cudaStream_t)stream;
    launch_snp_stats_raw(packed, row_stride, n_ind, n_snp, 1.0 / sqrt((double)n_snp), counts, avg, sd, lut, nullptr,
                         st);
    DPCA_CUDA(cudaGetLastError());
    DPCA_TRY(xw_dispatch(packed, row_stride, lut, n_ind, n_snp, nrhs, omega, y, st));
    DPCA_TRY(xty_dispatch(packed, row_stride, lut, n_ind, n_snp, nrhs, y, partial, splits, sps, st));
    const int64_t elems = (int64_t)n_ind * nrhs;
    const int grid = (int)std::min<int64_t>((elems + 255) / 256, (int64_t)sm_count * 8);
    reduce_splits_kernel<<<grid, 256, 0, st>>>(partial, elems, splits, z);
    DPCA_CUDA(cudaGetLastError());
    return DPCA_OK;
}
