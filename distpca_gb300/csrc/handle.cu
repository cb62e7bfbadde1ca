// Device-resident handle: allocation, upload, one pass, and the subspace iteration.
//
// The iteration follows BlockSubspaceIter_MPI_OOC_double_buffering (methods.cpp:941-1066):
//   pass; (QR -> pass) x (power-1); QR -> pass; B = Q^T Z; eig(upper B) descending;
//   Omega = Q W; sigma_j = sqrt(w_j); criterion for ii > 0;
// and, when the block size covers every SNP, SubspaceIteration_MPI (methods.cpp:52-258), whose
// last step is the half pass Y = X Q with the Gram form B = Y^T Y.  Everything runs on the
// device; the host reads back nsv singular values and the criterion flag once per iteration.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <set>

#include "common.cuh"
#include "dpca_internal.h"

namespace dpca {

// ------------------------------------------------------------------ per-kernel clock
int KernelClock::slot(const char *name) {
    for (size_t i = 0; i < names.size(); ++i)
        if (names[i] == name) return (int)i;
    names.emplace_back(name);
    ms.push_back(0.0);
    launches.push_back(0);
    return (int)names.size() - 1;
}

cudaEvent_t KernelClock::get_event() {
    if (!pool.empty()) {
        cudaEvent_t e = pool.back();
        pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

void KernelClock::resolve() {
    for (auto &p : pending) {
        float t = 0.f;
        if (cudaEventSynchronize(p.b) == cudaSuccess && cudaEventElapsedTime(&t, p.a, p.b) == cudaSuccess)
            ms[p.slot] += t;
        pool.push_back(p.a);
        pool.push_back(p.b);
    }
    pending.clear();
}

void KernelClock::reset() {
    resolve();
    for (auto &v : ms) v = 0.0;
    for (auto &v : launches) v = 0;
}

KernelClock::~KernelClock() {
    for (auto &p : pending) {
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
    }
    for (auto e : pool) cudaEventDestroy(e);
}

ScopedLaunch::ScopedLaunch(KernelClock *c, cudaStream_t s, const char *name, int n) : clk(c), st(s), kernels(n) {
    if (!clk || !clk->enabled) return;
    slot = clk->slot(name);
    a = clk->get_event();
    b = clk->get_event();
    cudaEventRecord(a, st);
}

ScopedLaunch::~ScopedLaunch() {
    if (slot < 0) return;
    cudaEventRecord(b, st);
    clk->launches[slot] += kernels;
    clk->pending.push_back({slot, a, b});
}

bool env_flag(const char *name) {
    const char *v = getenv(name);
    return v && *v && strcmp(v, "0") != 0;
}

static size_t round_up(size_t a, size_t b) { return (a + b - 1) / b * b; }

// The driver's unique id of the calling thread's current context (cuCtxGetId), made current by
// a runtime call first.  Unlike a device ordinal or a CUcontext handle, the id of a context
// created after cudaDeviceReset (or a different context the caller made current) differs from
// the old one's, so state cached per context -- kernel attributes, symbol addresses -- is
// looked up again instead of being reused from a context that no longer exists.
typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);

dpca_status current_context_id(unsigned long long *id) {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = (CtxGetCurrentFn)p;
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = (CtxGetIdFn)p;
    });
    if (!get_current || !get_id) {
        set_error("the CUDA driver does not provide cuCtxGetCurrent/cuCtxGetId");
        return DPCA_ERR_CUDA;
    }
    CUcontext ctx = nullptr;
    if (get_current(&ctx) == CUDA_SUCCESS && !ctx) {
        // no context yet on this thread: cudaSetDevice makes the device's primary context current
        int dev = 0;
        DPCA_CUDA(cudaGetDevice(&dev));
        DPCA_CUDA(cudaSetDevice(dev));
        get_current(&ctx);
    }
    if (!ctx || get_id(ctx, id) != CUDA_SUCCESS) {
        set_error("no current CUDA context");
        return DPCA_ERR_CUDA;
    }
    return DPCA_OK;
}

dpca_status allow_max_smem(const void *func) {
    static std::mutex mu;
    static std::set<std::pair<const void *, unsigned long long>> done;
    int dev = 0;
    DPCA_CUDA(cudaGetDevice(&dev));
    unsigned long long ctx = 0;
    DPCA_TRY(current_context_id(&ctx));
    std::lock_guard<std::mutex> lk(mu);
    if (done.count({func, ctx})) return DPCA_OK;
    int optin = 0;
    DPCA_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    cudaFuncAttributes fa{};
    DPCA_CUDA(cudaFuncGetAttributes(&fa, func));
    DPCA_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   optin - (int)fa.sharedSizeBytes));
    done.insert({func, ctx});
    return DPCA_OK;
}

dpca_status dev_alloc(Handle *h, void **p, size_t bytes) {
    *p = nullptr;
    if (bytes == 0) return DPCA_OK;
    cudaError_t e = !h->async_alloc ? cudaMalloc(p, bytes)
                    : h->pool       ? cudaMallocFromPoolAsync(p, bytes, h->pool, h->stream)
                                    : cudaMallocAsync(p, bytes, h->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("device allocation of %zu bytes: %s", bytes, cudaGetErrorString(e));
        *p = nullptr;
        return DPCA_ERR_NOMEM;
    }
    h->dev_bytes += bytes;
    return DPCA_OK;
}

void dev_free(Handle *h, void *p) {
    if (!p) return;
    if (h->async_alloc)
        cudaFreeAsync(p, h->stream);
    else
        cudaFree(p);
}

template <typename T>
static dpca_status dalloc(Handle *h, T **p, size_t elems) {
    return dev_alloc(h, (void **)p, elems * sizeof(T));
}

static void free_all(Handle *h) {
    if (h->mx) mixed_release(h);
    void *ptrs[] = {h->P,     h->PT,    h->counts, h->avg,      h->sd,  h->lut,    h->coef,
                    h->omega, h->z,     h->q,      h->old,      h->work, h->y,     h->partial,
                    h->small, h->red,   h->dflag,  h->Pb[0],    h->Pb[1], h->PTb[0], h->PTb[1],
                    h->Sb[0], h->Sb[1]};
    for (void *p : ptrs) dev_free(h, p);
    delete h->ring;  // waits for copies still reading its slots
    h->ring = nullptr;
    delete h->src;
    h->src = nullptr;
    for (int b = 0; b < 2; ++b) {
        if (h->copied[b]) cudaEventDestroy(h->copied[b]);
        if (h->consumed[b]) cudaEventDestroy(h->consumed[b]);
        if (h->staged_free[b]) cudaEventDestroy(h->staged_free[b]);
    }
    if (h->cstream) cudaStreamDestroy(h->cstream);
    if (h->host_small) {
        if (h->async_alloc)
            free(h->host_small);
        else
            cudaFreeHost(h->host_small);
    }
    if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
}

static dpca_status create_impl(Handle *h, int n_ind, int n_snp, int nrhs, int precision, int device, void *stream,
                               int block_snps) {
    if (n_ind <= 0 || n_snp <= 0 || nrhs <= 0) {
        set_error("dpca_create: n_ind, n_snp and nrhs must be positive");
        return DPCA_ERR_INVALID;
    }
    if (nrhs > kMaxNrhs) {
        set_error("dpca_create: nrhs=%d exceeds the device limit %d", nrhs, kMaxNrhs);
        return DPCA_ERR_UNSUPPORTED;
    }
    if (precision != DPCA_PREC_FP64 && precision != DPCA_PREC_MIXED) {
        set_error("dpca_create: unknown precision %d", precision);
        return DPCA_ERR_INVALID;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        set_error("no CUDA device available (libdpca has no CPU fallback)");
        return DPCA_ERR_CUDA;
    }
    if (device < 0 || device >= ndev) {
        set_error("device %d out of range (%d devices)", device, ndev);
        return DPCA_ERR_INVALID;
    }
    DPCA_CUDA(cudaSetDevice(device));
    h->device = device;
    DPCA_CUDA(cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, device));
    if (stream) {
        h->stream = (cudaStream_t)stream;
        h->own_stream = false;
    } else {
        DPCA_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
        h->own_stream = true;
    }
    h->n_ind = n_ind;
    h->n_snp = n_snp;
    h->k = nrhs;
    h->precision = precision;
    h->np = (n_ind + 3) / 4;
    h->pitch = (int64_t)round_up((size_t)h->np, 128);
    h->npT = (n_snp + 3) / 4;
    h->pitchT = (int64_t)round_up((size_t)h->npT, 128);
    h->n_ind_pad = (int)round_up((size_t)n_ind, 128);
    h->n_snp_pad = (int)round_up((size_t)n_snp, 128);
    h->inv_sqrt_nsnp = 1.0 / sqrt((double)n_snp);
    size_t nk = (size_t)n_ind * nrhs;
    h->streamed = block_snps > 0 && block_snps < n_snp;
    h->rows_dev = n_snp;
    if (h->streamed) {
        // two block buffers (double buffering) instead of the whole matrix
        h->blk = (int)std::min<size_t>(round_up((size_t)block_snps, 128), (size_t)n_snp);
        h->nblk = (n_snp + h->blk - 1) / h->blk;
        h->rows_dev = h->blk;
        h->pitchTb = (int64_t)round_up((size_t)(h->blk + 3) / 4, 128);
        for (int b = 0; b < 2; ++b) {
            DPCA_TRY(dalloc(h, &h->Pb[b], (size_t)h->blk * h->pitch));
            DPCA_CUDA(cudaMemsetAsync(h->Pb[b], 0, (size_t)h->blk * h->pitch, h->stream));
            if (precision == DPCA_PREC_MIXED) {
                DPCA_TRY(dalloc(h, &h->PTb[b], round_up((size_t)n_ind, 128) * h->pitchTb));
                DPCA_CUDA(cudaMemsetAsync(h->PTb[b], 0, round_up((size_t)n_ind, 128) * h->pitchTb, h->stream));
            }
            DPCA_CUDA(cudaEventCreateWithFlags(&h->copied[b], cudaEventDisableTiming));
            DPCA_CUDA(cudaEventCreateWithFlags(&h->consumed[b], cudaEventDisableTiming));
            DPCA_CUDA(cudaEventCreateWithFlags(&h->staged_free[b], cudaEventDisableTiming));
            // the first copy into buffer b (copy stream) waits for its zeroing (compute stream)
            DPCA_CUDA(cudaEventRecord(h->consumed[b], h->stream));
            DPCA_CUDA(cudaEventRecord(h->staged_free[b], h->stream));
        }
        DPCA_CUDA(cudaStreamCreateWithFlags(&h->cstream, cudaStreamNonBlocking));
    } else {
        DPCA_TRY(dalloc(h, &h->P, (size_t)n_snp * h->pitch));
        DPCA_CUDA(cudaMemsetAsync(h->P, 0, (size_t)n_snp * h->pitch, h->stream));
    }
    DPCA_TRY(dalloc(h, &h->counts, 4 * (size_t)n_snp));
    DPCA_TRY(dalloc(h, &h->avg, (size_t)n_snp));
    DPCA_TRY(dalloc(h, &h->sd, (size_t)n_snp));
    DPCA_TRY(dalloc(h, &h->lut, 4 * (size_t)n_snp));
    DPCA_TRY(dalloc(h, &h->coef, 2 * (size_t)n_snp));
    DPCA_TRY(dalloc(h, &h->omega, nk));
    DPCA_TRY(dalloc(h, &h->z, nk));
    DPCA_TRY(dalloc(h, &h->q, nk));
    DPCA_TRY(dalloc(h, &h->old, nk));
    DPCA_TRY(dalloc(h, &h->work, nk));
    DPCA_TRY(dalloc(h, &h->y, (size_t)h->rows_dev * nrhs));
    // FP64 split-K partials: up to ceil(4*SMs / tiles) splits
    {
        int tiles = (n_ind + 127) / 128;
        int s = std::max(1, (4 * h->sm_count + tiles - 1) / tiles);
        s = std::min(s, std::max(1, (h->rows_dev + 31) / 32));
        h->partial_elems = (size_t)s * nk;
        DPCA_TRY(dalloc(h, &h->partial, h->partial_elems));
    }
    SmallLayout L{nrhs};
    DPCA_TRY(dalloc(h, &h->small, L.total()));
    DPCA_CUDA(cudaMemsetAsync(h->small, 0, L.total() * sizeof(double), h->stream));
    h->red_elems = std::max<size_t>({(size_t)2 * h->sm_count * (size_t)nrhs * nrhs,
                                     (size_t)4 * h->sm_count * (nrhs + 1), (size_t)nrhs * nrhs + 64});
    DPCA_TRY(dalloc(h, &h->red, h->red_elems));
    DPCA_TRY(dalloc(h, &h->dflag, 16));
    DPCA_CUDA(cudaMemsetAsync(h->dflag, 0, 16 * sizeof(int), h->stream));
    if (h->async_alloc) {
        // pageable: pinned allocation and release can synchronise the device
        h->host_small = (double *)calloc(L.total(), sizeof(double));
        if (!h->host_small) return DPCA_ERR_NOMEM;
    } else {
        DPCA_CUDA(cudaMallocHost((void **)&h->host_small, L.total() * sizeof(double)));
    }
    if (precision == DPCA_PREC_MIXED) {
        if (!h->streamed) {
            // tile-blocked (see transpose_packed_kernel): rows padded to whole 128-row tiles
            DPCA_TRY(dalloc(h, &h->PT, round_up((size_t)n_ind, 128) * h->pitchT));
            DPCA_CUDA(cudaMemsetAsync(h->PT, 0, round_up((size_t)n_ind, 128) * h->pitchT, h->stream));
        }
        DPCA_TRY(mixed_prepare(h));
    }
    h->clock.enabled = env_flag("DPCA_KERNEL_CLOCK");
    return DPCA_OK;
}

size_t handle_footprint(int n_ind, int n_snp, int nrhs, int precision, int sm_count) {
    const size_t np = (size_t)(n_ind + 3) / 4, pitch = round_up(np, 128);
    const size_t nk = (size_t)n_ind * nrhs;
    const int tiles = (n_ind + 127) / 128;
    int s = std::max(1, (4 * sm_count + tiles - 1) / tiles);
    s = std::min(s, std::max(1, (n_snp + 31) / 32));
    const size_t L = SmallLayout{nrhs}.total();
    const size_t red = std::max<size_t>({(size_t)2 * sm_count * (size_t)nrhs * nrhs,
                                         (size_t)4 * sm_count * (nrhs + 1), (size_t)nrhs * nrhs + 64});
    size_t b = (size_t)n_snp * pitch + (size_t)n_snp * (16 + 8 + 8 + 32 + 16) + 5 * nk * 8 +
               (size_t)n_snp * nrhs * 8 + (size_t)s * nk * 8 + L * 8 + red * 8 + 64;
    if (precision == DPCA_PREC_MIXED)
        b += round_up((size_t)n_ind, 128) * round_up((size_t)(n_snp + 3) / 4, 128) +
             mixed_footprint(n_ind, n_snp, nrhs, sm_count);
    return b;
}

dpca_status create_serving_handle(dpca_handle **out, int n_ind, int n_snp, int nrhs, int precision, int device,
                                  cudaStream_t stream, cudaMemPool_t pool) {
    *out = nullptr;
    dpca_handle *hh = new (std::nothrow) dpca_handle();
    if (!hh) return DPCA_ERR_NOMEM;
    hh->h.async_alloc = true;
    hh->h.pool = pool;
    hh->h.stream = stream;  // set before create_impl so that its allocations are ordered on it
    // The QR as separate kernels: the one-launch form holds a block on every SM for the whole QR
    // (its blocks wait at grid barriers while block 0 runs the k x k factor), which keeps the other
    // jobs' kernels off those SMs.  On the 512-job serving stream: 37.4 jobs/s with the one-launch
    // QR, 43.8 with the separate kernels.
    hh->h.qr_coresident = -1;
    hh->h.no_graphs = true;
    dpca_status st = create_impl(&hh->h, n_ind, n_snp, nrhs, precision, device, stream, 0);
    if (st != DPCA_OK) {
        free_all(&hh->h);
        delete hh;
        return st;
    }
    *out = hh;
    return DPCA_OK;
}

// The blocks of a sweep over the rows: {first SNP, rows} of each block of `rows_per` rows.
static std::vector<std::pair<int64_t, int>> block_list(int n_snp, int rows_per) {
    std::vector<std::pair<int64_t, int>> v;
    for (int64_t s0 = 0; s0 < n_snp; s0 += rows_per) v.push_back({s0, (int)std::min<int64_t>(rows_per, n_snp - s0)});
    return v;
}

// Host rows of block i of the current sweep, rows [s0, s0 + ns): in place (pinned memory or
// callback blocks), or out of the pinned ring (file rows, pageable rows).  *via_ring tells the
// caller to release the ring slot once the block's copy is enqueued.
static dpca_status block_rows(Handle *h, int i, int64_t s0, int ns, const uint8_t **ptr, int64_t *stride,
                              bool *via_ring) {
    *via_ring = h->src->use_ring;
    if (*via_ring) {
        *stride = h->np;
        return h->ring->acquire(i, ptr);
    }
    bool pin = false;
    return h->src->direct(s0, ns, ptr, stride, &pin);
}

// Streaming: block j of the rows into buffer j % 2.  The copy stream runs only host-to-device
// copies, back to back: rows at the device pitch go straight into Pb, others contiguously into
// the staging buffer Sb, which the compute stream re-pitches into Pb.  The copy into a buffer
// waits until the compute stream is done with the block that used it before; the compute stream
// waits for the copy.
static dpca_status stream_in(Handle *h, int j, int *s0, int *ns) {
    const int b = j & 1;
    *s0 = j * h->blk;
    *ns = std::min(h->blk, h->n_snp - *s0);
    const uint8_t *src = nullptr;
    int64_t stride = 0;
    bool via_ring = false;
    DPCA_TRY(block_rows(h, j, *s0, *ns, &src, &stride, &via_ring));
    const bool staged = stride != h->pitch;
    cudaStream_t cs = h->cstream;
    dpca_status st = DPCA_OK;
    auto check = [&](cudaError_t e, const char *what) {
        if (e != cudaSuccess && st == DPCA_OK) {
            set_error("streamed block %d: %s: %s", j, what, cudaGetErrorString(e));
            st = DPCA_ERR_CUDA;
        }
    };
    if (staged && (size_t)*ns * stride > h->sb_bytes) {
        set_error("streamed block %d: rows of stride %lld exceed the staging buffer", j, (long long)stride);
        st = DPCA_ERR_INVALID;
    } else {
        check(cudaStreamWaitEvent(cs, staged ? h->staged_free[b] : h->consumed[b], 0), "wait");
        check(cudaMemcpyAsync(staged ? h->Sb[b] : h->Pb[b], src, (size_t)*ns * stride, cudaMemcpyHostToDevice, cs),
              "host-to-device copy");
    }
    if (via_ring) {  // always hand the slot back, also after an error
        dpca_status rs = h->ring->release(j, cs);
        if (st == DPCA_OK) st = rs;
    }
    DPCA_TRY(st);
    DPCA_CUDA(cudaEventRecord(h->copied[b], cs));
    DPCA_CUDA(cudaStreamWaitEvent(h->stream, h->copied[b], 0));
    if (staged) {
        // Pb[b] is free here: the compute stream's own earlier work on it precedes
        DPCA_CUDA(cudaMemcpy2DAsync(h->Pb[b], h->pitch, h->Sb[b], stride, h->np, *ns, cudaMemcpyDeviceToDevice,
                                    h->stream));
        DPCA_CUDA(cudaEventRecord(h->staged_free[b], h->stream));
    }
    return DPCA_OK;
}

static dpca_status start_sweep(Handle *h, int rows_per) {
    if (!h->src || h->src->kind == RowSource::kNone) {
        set_error("no genotype rows attached (call dpca_upload, dpca_upload_file or dpca_upload_blocks)");
        return DPCA_ERR_INVALID;
    }
    if (!h->src->use_ring) return DPCA_OK;
    if (!h->ring) {
        h->ring = new (std::nothrow) HostRing();
        if (!h->ring) return DPCA_ERR_NOMEM;
    }
    return h->ring->start(h->src, block_list(h->n_snp, rows_per));
}

// Per-SNP statistics of a streamed matrix: one sweep over the blocks.
static dpca_status streamed_stats(Handle *h) {
    DPCA_TRY(start_sweep(h, h->blk));
    for (int j = 0; j < h->nblk; ++j) {
        int s0 = 0, ns = 0;
        DPCA_TRY(stream_in(h, j, &s0, &ns));
        {
            ScopedLaunch t(&h->clock, h->stream, "snp_stats");
            launch_snp_stats_raw(h->Pb[j & 1], h->pitch, h->n_ind, ns, h->inv_sqrt_nsnp, h->counts + 4 * (size_t)s0,
                                 h->avg + s0, h->sd + s0, h->lut + 4 * (size_t)s0, h->coef + 2 * (size_t)s0,
                                 h->stream);
            DPCA_CUDA(cudaGetLastError());
        }
        DPCA_CUDA(cudaEventRecord(h->consumed[j & 1], h->stream));
    }
    h->stats_ready = true;
    return DPCA_OK;
}

// One pass over a streamed matrix: blocks arrive double-buffered; Z accumulates over them.
static dpca_status streamed_pass(Handle *h, const double *in, double *out) {
    if (h->precision == DPCA_PREC_MIXED) DPCA_TRY(mixed_omega_operand(h, in));
    DPCA_TRY(start_sweep(h, h->blk));
    for (int j = 0; j < h->nblk; ++j) {
        int s0 = 0, ns = 0;
        DPCA_TRY(stream_in(h, j, &s0, &ns));
        if (h->precision == DPCA_PREC_FP64) DPCA_TRY(launch_fp64_block(h, j & 1, s0, ns, in, out, j > 0));
        else DPCA_TRY(mixed_block(h, j & 1, s0, ns, out, j > 0));
        DPCA_CUDA(cudaEventRecord(h->consumed[j & 1], h->stream));
    }
    return DPCA_OK;
}

static dpca_status after_data(Handle *h) {
    if (h->streamed) return streamed_stats(h);
    DPCA_TRY(launch_snp_stats(h));
    if (h->precision == DPCA_PREC_MIXED) {
        DPCA_TRY(launch_transpose_packed(h));
    }
    h->stats_ready = true;
    return DPCA_OK;
}

dpca_status handle_pass_io(Handle *h, const double *in, double *out) {
    if (!h->stats_ready) {
        set_error("no genotype data on the device (call dpca_upload or dpca_synth_fill)");
        return DPCA_ERR_INVALID;
    }
    if (h->streamed) return streamed_pass(h, in, out);
    const bool fp64 = h->precision == DPCA_PREC_FP64;
    {
        ScopedLaunch t(h->stage, h->stream, fp64 ? "fp64_xw" : "mixed_xw");
        DPCA_TRY(fp64 ? launch_fp64_xw(h, in, h->y) : launch_mixed_xw(h, in, nullptr));
    }
    ScopedLaunch t(h->stage, h->stream, fp64 ? "fp64_xty" : "mixed_xty");
    return fp64 ? launch_fp64_xty(h, h->y, out) : launch_mixed_xty(h, out);
}

dpca_status handle_pass(Handle *h) { return handle_pass_io(h, h->omega, h->z); }

dpca_status check_device_flag(Handle *h) {
    int flags[4] = {0, 0, 0, 0};
    DPCA_CUDA(cudaMemcpyAsync(flags, h->dflag, sizeof(flags), cudaMemcpyDeviceToHost, h->stream));
    DPCA_CUDA(cudaStreamSynchronize(h->stream));
    if (flags[0]) {
        set_error("a bounded device wait gave up (site %d); results of this call are invalid", flags[0]);
        cudaMemsetAsync(h->dflag, 0, 16 * sizeof(int), h->stream);
        return DPCA_ERR_TIMEOUT;
    }
    if (flags[1]) {
        set_error("a device k x k solve did not converge (site %d)", flags[1]);
        cudaMemsetAsync(h->dflag, 0, 16 * sizeof(int), h->stream);
        return DPCA_ERR_NUMERIC;
    }
    return DPCA_OK;
}

// Y = X Q only (the in-core variant's half pass), into h->y as FP64.
static dpca_status half_pass(Handle *h, const double *in) {
    if (h->precision == DPCA_PREC_FP64) return launch_fp64_xw(h, in, h->y);
    return launch_mixed_xw(h, in, h->y);
}

static double slot_ms(const KernelClock &c, const char *name) {
    for (size_t i = 0; i < c.names.size(); ++i)
        if (c.names[i] == name) return c.ms[i];
    return 0.0;
}

// Outer iterations launched eagerly before a solve replays them as graphs.
constexpr int kGraphFromIter = 3;

static dpca_status solve_impl(Handle *h, const dpca_config *cfg, double *omega_inout, dpca_result *res) {
    const int n = h->n_ind, k = h->k;
    if (!cfg || !omega_inout || !res) {
        set_error("dpca_solve: null argument");
        return DPCA_ERR_INVALID;
    }
    const int nsv = cfg->nsv, miter = cfg->miter, power = cfg->power, crit = cfg->crit;
    if (nsv <= 0 || nsv > k) {
        set_error("dpca_solve: nsv=%d must be in [1, nrhs=%d]", nsv, k);
        return DPCA_ERR_INVALID;
    }
    if (!h->stats_ready) {
        set_error("no genotype data on the device");
        return DPCA_ERR_INVALID;
    }
    // the in-core variant's Gram form needs Y = X Q of every SNP at once: resident matrices only
    const bool in_core = cfg->bsize >= h->n_snp && !h->streamed;
    const size_t nkb = (size_t)n * k * sizeof(double);
    SmallLayout L{k};
    // Statistics (the reference's timing block) come from the per-launch clock when the caller
    // turned it on (profiling) or the handle streams (long passes), and otherwise from coarse
    // stage events: two events around each of ~80 launches per outer iteration, and resolving
    // them, cost the short solves of small cohorts ~15% of their time.
    const bool fine = h->clock.enabled || h->streamed;
    bool clock_was = h->clock.enabled;
    KernelClock coarse;
    coarse.enabled = !fine;
    h->stage = fine ? nullptr : &coarse;
    // on every way out (errors included): no stage clock left pointing at this frame, and the
    // caller's per-launch clock setting back
    struct Restore {
        Handle *h;
        bool clock_was;
        ~Restore() {
            h->stage = nullptr;
            h->clock.enabled = clock_was;
        }
    } restore{h, clock_was};
    h->clock.reset();
    h->clock.enabled = fine;
    auto qr = [&](double *a) {
        ScopedLaunch t(h->stage, h->stream, "qr_chol");
        return launch_qr(h, a);
    };
    cudaEvent_t t0, t1;
    DPCA_CUDA(cudaEventCreate(&t0));
    DPCA_CUDA(cudaEventCreate(&t1));
    DPCA_CUDA(cudaEventRecord(t0, h->stream));
    DPCA_CUDA(cudaMemcpyAsync(h->omega, omega_inout, nkb, cudaMemcpyHostToDevice, h->stream));
    DPCA_CUDA(cudaMemsetAsync(h->small, 0, L.total() * sizeof(double), h->stream));
    if (crit == 2) DPCA_CUDA(cudaMemcpyAsync(h->old, h->omega, nkb, cudaMemcpyDeviceToDevice, h->stream));
    // Mixed precision: orthonormalize the start block first.  span(X^T X Omega) -- and so every
    // later subspace and Ritz value -- is unchanged in exact arithmetic, but the reference's
    // start block is nearly rank-deficient (neighbouring columns come from neighbouring LCG
    // seeds), and a 22-bit product of it would lose its trailing directions.
    if (h->precision == DPCA_PREC_MIXED) DPCA_TRY(qr(h->omega));
    double *omega = h->omega, *z = h->z, *q = h->q;
    int ii = 0, passes = 0;
    bool stopped = false;
    // The device work of one outer iteration: the passes and QRs, the Rayleigh-Ritz step and the
    // criterion.  `iter` matters only as iter > 0 (the criterion compares with the iteration
    // before).  Rotates omega, z, q and counts the passes as it goes.
    auto body = [&](int iter) -> dpca_status {
        DPCA_TRY(handle_pass_io(h, omega, z));
        passes++;
        for (int kk = 0; kk < power - 1; ++kk) {
            DPCA_TRY(qr(z));
            std::swap(omega, z);  // Omega <- Q
            DPCA_TRY(handle_pass_io(h, omega, z));
            passes++;
        }
        DPCA_TRY(qr(z));
        std::swap(q, z);  // Q
        if (in_core) {
            {
                ScopedLaunch t(h->stage, h->stream, h->precision == DPCA_PREC_FP64 ? "fp64_xw" : "mixed_xw");
                DPCA_TRY(half_pass(h, q));
            }
            ScopedLaunch t(h->stage, h->stream, "atb");
            DPCA_TRY(launch_atb(h, h->y, h->y, h->n_snp, h->small + L.B()));
        } else {
            DPCA_TRY(handle_pass_io(h, q, z));
            passes++;
            ScopedLaunch t(h->stage, h->stream, "atb");
            DPCA_TRY(launch_atb(h, q, z, n, h->small + L.B()));
        }
        {
            ScopedLaunch t(h->stage, h->stream, "sym_eig");
            DPCA_TRY(launch_eig_desc(h));
        }
        {
            ScopedLaunch t(h->stage, h->stream, "apply_w");
            DPCA_TRY(launch_apply_w(h, q, omega));
        }
        return launch_sigma_and_criterion(h, nsv, crit, cfg->tol, iter, h->old, omega);
    };
    // Iteration graphs.  From the kGraphFromIter-th outer iteration on, an iteration's ~40 launches
    // replay as one CUDA graph: the kernels are the same, in the same order, so the results are
    // the same bits, and the gaps between dependent launches shrink.  An iteration rotates the
    // three n x k buffers, so a graph is captured for each assignment of them that occurs (at
    // most three) the first time it does.  Not for streamed handles (a pass reads host blocks),
    // under the per-launch clock, while a test fault is pending, nor on serving handles (short
    // solves, on a device whose launch gaps the other jobs' kernels fill; not measured there).  A
    // capture that fails leaves the solve on eager launches.
    struct IterGraph {
        double *pre[3], *post[3];
        cudaGraphExec_t exec;
        int passes;
    };
    std::vector<IterGraph> graphs;
    struct GraphsGuard {
        std::vector<IterGraph> &g;
        ~GraphsGuard() {
            for (auto &x : g) cudaGraphExecDestroy(x.exec);
        }
    } graphs_guard{graphs};
    const char *genv = getenv("DPCA_SOLVE_GRAPHS");
    bool use_graphs = !fine && !h->streamed && !h->no_graphs && h->inject_fault == 0 && miter > kGraphFromIter &&
                      !(genv && strcmp(genv, "0") == 0);
    auto capture = [&]() -> const IterGraph * {
        double *pre[3] = {omega, z, q};
        const int passes0 = passes;
        if (cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        KernelClock *stage = h->stage;
        h->stage = nullptr;
        const dpca_status st = body(1);
        h->stage = stage;
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(h->stream, &g);
        cudaGraphExec_t exec = nullptr;
        if (st == DPCA_OK && e == cudaSuccess && g && cudaGraphInstantiate(&exec, g, 0) != cudaSuccess) exec = nullptr;
        if (g) cudaGraphDestroy(g);
        IterGraph entry{{pre[0], pre[1], pre[2]}, {omega, z, q}, exec, passes - passes0};
        omega = pre[0];  // the captured work has not run
        z = pre[1];
        q = pre[2];
        passes = passes0;
        if (!exec) {
            cudaGetLastError();
            clear_error();
            return nullptr;
        }
        graphs.push_back(entry);
        return &graphs.back();
    };
    for (ii = 0; ii < miter; ++ii) {
        const IterGraph *gi = nullptr;
        if (use_graphs && ii >= kGraphFromIter) {
            for (const auto &x : graphs)
                if (x.pre[0] == omega && x.pre[1] == z && x.pre[2] == q) gi = &x;
            if (!gi) gi = capture();
            if (!gi) use_graphs = false;
        }
        if (gi) {
            ScopedLaunch t(h->stage, h->stream, "graph_iterations");
            DPCA_CUDA(cudaGraphLaunch(gi->exec, h->stream));
            omega = gi->post[0];
            z = gi->post[1];
            q = gi->post[2];
            passes += gi->passes;
        } else {
            DPCA_TRY(body(ii));
        }
        DPCA_CUDA(cudaMemcpyAsync(h->host_small, h->small, L.total() * sizeof(double), cudaMemcpyDeviceToHost,
                                  h->stream));
        DPCA_CUDA(cudaStreamSynchronize(h->stream));
        DPCA_TRY(check_device_flag(h));
        const double *hs = h->host_small;
        if (res->delta_iter) res->delta_iter[ii] = hs[L.crit() + 2];
        if (cfg->verbose > 1 && ii > 0) {
            if (crit == 0) printf("Iteration %d: rel. error: %02.13f\n", ii, hs[L.crit()]);
            else if (crit == 1) printf("Iteration %d: %d converged\n", ii, (int)hs[L.crit()]);
            else if (crit == 2) printf("Iteration %d: MEV error: %02.13f\n", ii, hs[L.crit()]);
        }
        if (hs[L.crit() + 1] != 0.0) {
            stopped = true;
            break;
        }
        if (crit == 2) DPCA_CUDA(cudaMemcpyAsync(h->old, omega, nkb, cudaMemcpyDeviceToDevice, h->stream));
    }
    DPCA_CUDA(cudaEventRecord(t1, h->stream));
    DPCA_CUDA(cudaMemcpyAsync(omega_inout, omega, nkb, cudaMemcpyDeviceToHost, h->stream));
    DPCA_CUDA(cudaStreamSynchronize(h->stream));
    // keep the handle's canonical buffers pointing at distinct allocations
    h->omega = omega;
    h->z = z;
    h->q = q;
    float total_ms = 0.f;
    cudaEventElapsedTime(&total_ms, t0, t1);
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    res->n_ind = n;
    res->n_snp = h->n_snp;
    res->nsv = nsv;
    res->nrhs = k;
    res->total_its = stopped ? ii + 1 : ii;
    res->passes = passes;
    res->in_core = in_core ? 1 : 0;
    res->streamed = h->streamed ? 1 : 0;
    if (res->sigma) memcpy(res->sigma, h->host_small + L.sigma(), (size_t)nsv * sizeof(double));
    if (res->u)
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < nsv; ++j) res->u[(size_t)i * nsv + j] = omega_inout[(size_t)i * k + j];
    h->clock.resolve();
    coarse.resolve();
    h->stage = nullptr;
    const KernelClock &c = fine ? h->clock : coarse;
    double xw = slot_ms(c, "fp64_xw") + slot_ms(c, "mixed_xw") + slot_ms(c, "split_omega");
    double xty = slot_ms(c, "fp64_xty") + slot_ms(c, "reduce_splits") + slot_ms(c, "mixed_xty") +
                 slot_ms(c, "mixed_reduce");
    res->time_mm_a = xw * 1e-3;
    res->time_mm_a_t = xty * 1e-3;
    res->time_mm = (xw + xty + slot_ms(c, "atb") + slot_ms(c, "atb_sum") + slot_ms(c, "apply_w")) * 1e-3;
    res->time_gs = (slot_ms(c, "qr_gram") + slot_ms(c, "qr_gram_sum") + slot_ms(c, "qr_chol") +
                    slot_ms(c, "qr_apply") + slot_ms(c, "qr_fused")) * 1e-3;
    res->time_projected_svd = slot_ms(c, "sym_eig") * 1e-3;
    // graph-replayed iterations are timed as a whole: their time is split among the stages in the
    // proportions of the eagerly launched iterations
    const double staged = res->time_mm + res->time_gs + res->time_projected_svd;
    const double graphed = slot_ms(c, "graph_iterations") * 1e-3;
    if (graphed > 0.0 && staged > 0.0) {
        const double f = (staged + graphed) / staged;
        res->time_mm_a *= f;
        res->time_mm_a_t *= f;
        res->time_mm *= f;
        res->time_gs *= f;
        res->time_projected_svd *= f;
    }
    res->time_other = total_ms * 1e-3 - res->time_mm - res->time_gs - res->time_projected_svd;
    if (res->time_other < 0) res->time_other = 0;
    h->clock.enabled = clock_was;
    for (int j = 0; j < nsv; ++j)
        if (!std::isfinite(h->host_small[L.sigma() + j]) && h->host_small[L.w() + j] >= 0) {
            set_error("non-finite singular value %d", j);
            return DPCA_ERR_NUMERIC;
        }
    return DPCA_OK;
}

// Resident upload, pipelined in chunks of whole 512-SNP tiles: each chunk's rows (in place, or out
// of the pinned ring for file and pageable rows) are copied contiguously (full host-link speed; a
// row-pitched copy of .bed-layout rows ran ~25% slower) into a staging buffer on a copy stream,
// re-pitched into P on the device, and its per-SNP statistics and transposed tiles computed while
// the next chunk is copied.
static dpca_status upload_pipelined(Handle *h) {
    ScopedLaunch t(&h->clock, h->stream, "h2d_packed");
    const int64_t cstride = h->src->copy_stride();
    int64_t rows_per = std::max<int64_t>(512, ((int64_t)(256 << 20) / std::max<int64_t>(1, cstride)) / 512 * 512);
    rows_per = std::min<int64_t>(rows_per, ((int64_t)h->n_snp + 511) / 512 * 512);
    dpca_status st = DPCA_OK;
    auto check = [&](cudaError_t e, const char *what) {
        if (e != cudaSuccess && st == DPCA_OK) {
            set_error("upload: %s: %s", what, cudaGetErrorString(e));
            st = e == cudaErrorMemoryAllocation ? DPCA_ERR_NOMEM : DPCA_ERR_CUDA;
        }
        return st == DPCA_OK;
    };
    // copy stream, events and staging buffers are kept by the handle (freed with it)
    if (!h->cstream) check(cudaStreamCreateWithFlags(&h->cstream, cudaStreamNonBlocking), "stream");
    const size_t stage_bytes = (size_t)rows_per * cstride;
    for (int b = 0; b < 2 && st == DPCA_OK; ++b) {
        if (!h->copied[b]) check(cudaEventCreateWithFlags(&h->copied[b], cudaEventDisableTiming), "event");
        if (!h->consumed[b]) check(cudaEventCreateWithFlags(&h->consumed[b], cudaEventDisableTiming), "event");
        if (!h->Sb[b] || h->sb_bytes < stage_bytes) {
            dev_free(h, h->Sb[b]);
            h->Sb[b] = nullptr;
            if (st == DPCA_OK) st = dev_alloc(h, (void **)&h->Sb[b], stage_bytes);
        }
        // the copy stream's first use of each buffer waits for everything queued on the compute
        // stream so far: the allocations (stream-ordered ones are usable from that point) and
        // the zeroing of P
        check(cudaEventRecord(h->consumed[b], h->stream), "record");
    }
    if (st == DPCA_OK) h->sb_bytes = std::max(h->sb_bytes, stage_bytes);
    if (st == DPCA_OK) st = start_sweep(h, (int)rows_per);
    cudaStream_t cs = h->cstream;
    for (int64_t s0 = 0, j = 0; s0 < h->n_snp && st == DPCA_OK; s0 += rows_per, ++j) {
        const int b = (int)(j & 1);
        const int rows = (int)std::min<int64_t>(rows_per, h->n_snp - s0);
        const uint8_t *src = nullptr;
        int64_t stride = 0;
        bool via_ring = false;
        st = block_rows(h, (int)j, s0, rows, &src, &stride, &via_ring);
        if (st != DPCA_OK) break;
        uint8_t *dst = h->P + s0 * h->pitch;
        const bool direct = stride == h->pitch;  // rows already at the device pitch
        if ((size_t)rows * stride > h->sb_bytes && !direct) {
            set_error("upload: rows of stride %lld exceed the staging buffer", (long long)stride);
            st = DPCA_ERR_INVALID;
        }
        check(cudaStreamWaitEvent(cs, h->consumed[b], 0), "wait");
        check(cudaMemcpyAsync(direct ? (void *)dst : (void *)h->Sb[b], src, (size_t)rows * stride,
                              cudaMemcpyHostToDevice, cs),
              "copy");
        if (via_ring) {
            dpca_status rs = h->ring->release((int)j, cs);
            if (st == DPCA_OK) st = rs;
        }
        check(cudaEventRecord(h->copied[b], cs), "record");
        check(cudaStreamWaitEvent(h->stream, h->copied[b], 0), "wait");
        if (!direct)
            check(cudaMemcpy2DAsync(dst, h->pitch, h->Sb[b], stride, h->np, rows, cudaMemcpyDeviceToDevice, h->stream),
                  "re-pitch");
        check(cudaEventRecord(h->consumed[b], h->stream), "record");
        if (st != DPCA_OK) break;
        launch_snp_stats_raw(dst, h->pitch, h->n_ind, rows, h->inv_sqrt_nsnp, h->counts + 4 * s0, h->avg + s0,
                             h->sd + s0, h->lut + 4 * s0, h->coef + 2 * s0, h->stream);
        if (h->precision == DPCA_PREC_MIXED)
            launch_transpose_raw(dst, h->pitch, h->PT, h->pitchT, h->n_ind, rows, h->stream, (int)s0);
        check(cudaGetLastError(), "launch");
    }
    return st;
}

// Attach a row source to the handle (replacing any earlier one) and load it: a resident handle
// copies every row to the device now; a streaming handle computes its per-SNP statistics in one
// sweep and reads the rows again in every pass.
static dpca_status attach_source(Handle *h, RowSource *src) {
    if (h->ring) {
        delete h->ring;  // its reader may hold the old source
        h->ring = nullptr;
    }
    delete h->src;
    h->src = src;
    h->stats_ready = false;
    if (h->streamed) {
        const int64_t cs = src->copy_stride();
        if (cs != h->pitch) {
            for (int b = 0; b < 2; ++b) {
                dev_free(h, h->Sb[b]);  // the compute stream is ordered after every copy that used it
                h->Sb[b] = nullptr;
                DPCA_TRY(dev_alloc(h, (void **)&h->Sb[b], (size_t)h->blk * cs));
                DPCA_CUDA(cudaEventRecord(h->staged_free[b], h->stream));
            }
            h->sb_bytes = (size_t)h->blk * cs;
        }
        return after_data(h);
    }
    DPCA_TRY(upload_pipelined(h));
    h->stats_ready = true;
    return DPCA_OK;
}

}  // namespace dpca

using namespace dpca;

extern "C" {

dpca_status dpca_create(dpca_handle **out, int n_ind, int n_snp, int nrhs, int precision, int device, void *stream) {
    clear_error();
    if (!out) return DPCA_ERR_INVALID;
    *out = nullptr;
    dpca_handle *hh = new (std::nothrow) dpca_handle();
    if (!hh) return DPCA_ERR_NOMEM;
    dpca_status st = create_impl(&hh->h, n_ind, n_snp, nrhs, precision, device, stream, 0);
    if (st != DPCA_OK) {
        free_all(&hh->h);
        delete hh;
        return st;
    }
    *out = hh;
    return DPCA_OK;
}

dpca_status dpca_create_streamed(dpca_handle **out, int n_ind, int n_snp, int nrhs, int precision, int device,
                                 void *stream, int block_snps) {
    clear_error();
    if (!out) return DPCA_ERR_INVALID;
    *out = nullptr;
    if (block_snps <= 0) {
        set_error("dpca_create_streamed: block_snps must be positive");
        return DPCA_ERR_INVALID;
    }
    dpca_handle *hh = new (std::nothrow) dpca_handle();
    if (!hh) return DPCA_ERR_NOMEM;
    dpca_status st = create_impl(&hh->h, n_ind, n_snp, nrhs, precision, device, stream, block_snps);
    if (st != DPCA_OK) {
        free_all(&hh->h);
        delete hh;
        return st;
    }
    *out = hh;
    return DPCA_OK;
}

dpca_status dpca_qr_device(int device, int n, int k, double *a, int separate) {
    clear_error();
    if (n < 1 || k < 1 || k > kMaxNrhs || !a) {
        set_error("dpca_qr_device: need n >= 1, 1 <= k <= %d and a non-null array", kMaxNrhs);
        return DPCA_ERR_INVALID;
    }
    dpca_handle *hh = nullptr;
    DPCA_TRY(dpca_create(&hh, n, 1, k, DPCA_PREC_FP64, device, nullptr));
    Handle *h = &hh->h;
    if (separate) h->qr_coresident = -1;
    const size_t bytes = (size_t)n * k * sizeof(double);
    dpca_status st = DPCA_OK;
    cudaError_t e = cudaMemcpyAsync(h->omega, a, bytes, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) st = launch_qr(h, h->omega);
    if (e == cudaSuccess && st == DPCA_OK) e = cudaMemcpyAsync(a, h->omega, bytes, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess && st == DPCA_OK) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess && st == DPCA_OK) {
        set_error("dpca_qr_device: %s", cudaGetErrorString(e));
        st = DPCA_ERR_CUDA;
    }
    dpca_destroy(hh);
    return st;
}

dpca_status dpca_destroy(dpca_handle *hh) {
    if (!hh) return DPCA_OK;
    cudaSetDevice(hh->h.device);
    if (hh->h.stream) cudaStreamSynchronize(hh->h.stream);
    free_all(&hh->h);
    delete hh;
    return DPCA_OK;
}

dpca_status dpca_upload(dpca_handle *hh, const uint8_t *packed, int64_t row_stride) {
    clear_error();
    if (!hh || !packed) return DPCA_ERR_INVALID;
    Handle *h = &hh->h;
    if (row_stride < h->np) {
        set_error("row_stride %lld < ceil(n_ind/4) = %lld", (long long)row_stride, (long long)h->np);
        return DPCA_ERR_INVALID;
    }
    DPCA_CUDA(cudaSetDevice(h->device));
    RowSource *src = new (std::nothrow) RowSource();
    if (!src) return DPCA_ERR_NOMEM;
    src->set_memory(packed, row_stride, h->np);
    return attach_source(h, src);
}

dpca_status dpca_upload_file(dpca_handle *hh, const char *bed_path) {
    clear_error();
    if (!hh || !bed_path) return DPCA_ERR_INVALID;
    Handle *h = &hh->h;
    DPCA_CUDA(cudaSetDevice(h->device));
    RowSource *src = new (std::nothrow) RowSource();
    if (!src) return DPCA_ERR_NOMEM;
    dpca_status st = src->open_file(bed_path, h->np);
    if (st != DPCA_OK) {
        delete src;
        return st;
    }
    return attach_source(h, src);
}

dpca_status dpca_upload_blocks(dpca_handle *hh, dpca_block_fn fn, void *ctx, int64_t max_row_stride) {
    clear_error();
    if (!hh || !fn) return DPCA_ERR_INVALID;
    Handle *h = &hh->h;
    if (max_row_stride < h->np) {
        set_error("max_row_stride %lld < ceil(n_ind/4) = %lld", (long long)max_row_stride, (long long)h->np);
        return DPCA_ERR_INVALID;
    }
    DPCA_CUDA(cudaSetDevice(h->device));
    RowSource *src = new (std::nothrow) RowSource();
    if (!src) return DPCA_ERR_NOMEM;
    src->set_blocks(fn, ctx, h->np, max_row_stride);
    return attach_source(h, src);
}

dpca_status dpca_synth_fill(dpca_handle *hh, uint64_t key, const uint8_t *pop, const uint32_t *miss_thr,
                            const uint32_t *snp_thr, int n_pop) {
    clear_error();
    if (!hh || !pop || !miss_thr || !snp_thr || n_pop <= 0) return DPCA_ERR_INVALID;
    Handle *h = &hh->h;
    if (h->streamed) {
        set_error("dpca_synth_fill: a streaming handle reads its rows from host memory (use dpca_upload)");
        return DPCA_ERR_UNSUPPORTED;
    }
    DPCA_CUDA(cudaSetDevice(h->device));
    uint8_t *d_pop = nullptr;
    uint32_t *d_miss = nullptr, *d_thr = nullptr;
    const size_t held = h->dev_bytes;
    dpca_status st = dalloc(h, &d_pop, (size_t)h->n_ind);
    if (st == DPCA_OK) st = dalloc(h, &d_miss, (size_t)h->n_ind);
    if (st == DPCA_OK) st = dalloc(h, &d_thr, (size_t)h->n_snp * n_pop);
    if (st != DPCA_OK) {
        dev_free(h, d_pop);
        dev_free(h, d_miss);
        h->dev_bytes = held;
        return st;
    }
    DPCA_CUDA(cudaMemcpyAsync(d_pop, pop, (size_t)h->n_ind, cudaMemcpyHostToDevice, h->stream));
    DPCA_CUDA(cudaMemcpyAsync(d_miss, miss_thr, (size_t)h->n_ind * 4, cudaMemcpyHostToDevice, h->stream));
    DPCA_CUDA(cudaMemcpyAsync(d_thr, snp_thr, (size_t)h->n_snp * n_pop * 4, cudaMemcpyHostToDevice, h->stream));
    st = launch_synth_fill(h, key, d_pop, d_miss, d_thr, n_pop);
    cudaStreamSynchronize(h->stream);  // the host tables may be freed once this returns
    dev_free(h, d_pop);
    dev_free(h, d_miss);
    dev_free(h, d_thr);
    h->dev_bytes = held;  // temporaries
    DPCA_TRY(st);
    DPCA_TRY(after_data(h));
    return DPCA_OK;
}

dpca_status dpca_download_packed(dpca_handle *hh, int s0, int s1, uint8_t *out) {
    clear_error();
    if (!hh || !out) return DPCA_ERR_INVALID;
    Handle *h = &hh->h;
    if (s0 < 0 || s1 > h->n_snp || s0 > s1) {
        set_error("SNP range [%d, %d) outside [0, %d)", s0, s1, h->n_snp);
        return DPCA_ERR_INVALID;
    }
    DPCA_CUDA(cudaSetDevice(h->device));
    if (h->streamed) {
        if (!h->src || h->src->kind == RowSource::kNone) {
            set_error("no genotype rows attached (call dpca_upload, dpca_upload_file or dpca_upload_blocks)");
            return DPCA_ERR_INVALID;
        }
        std::string err;
        dpca_status st = s1 > s0 ? h->src->read_into(s0, s1 - s0, out, &err) : DPCA_OK;
        if (st != DPCA_OK) set_error("%s", err.c_str());
        return st;
    }
    if (s1 > s0)
        DPCA_CUDA(cudaMemcpy2DAsync(out, h->np, h->P + (int64_t)s0 * h->pitch, h->pitch, h->np, s1 - s0,
                                    cudaMemcpyDeviceToHost, h->stream));
    DPCA_CUDA(cudaStreamSynchronize(h->stream));
    return DPCA_OK;
}

dpca_status dpca_snp_stats(dpca_handle *hh, int32_t *counts, double *avg, double *sd, double *lut) {
    clear_error();
    if (!hh) return DPCA_ERR_INVALID;
    Handle *h = &hh->h;
    if (!h->stats_ready) {
        set_error("no genotype data on the device");
        return DPCA_ERR_INVALID;
    }
    DPCA_CUDA(cudaSetDevice(h->device));
    size_t n = (size_t)h->n_snp;
    if (counts) DPCA_CUDA(cudaMemcpyAsync(counts, h->counts, 4 * n * 4, cudaMemcpyDeviceToHost, h->stream));
    if (avg) DPCA_CUDA(cudaMemcpyAsync(avg, h->avg, n * 8, cudaMemcpyDeviceToHost, h->stream));
    if (sd) DPCA_CUDA(cudaMemcpyAsync(sd, h->sd, n * 8, cudaMemcpyDeviceToHost, h->stream));
    if (lut) DPCA_CUDA(cudaMemcpyAsync(lut, h->lut, 4 * n * 8, cudaMemcpyDeviceToHost, h->stream));
    DPCA_CUDA(cudaStreamSynchronize(h->stream));
    return DPCA_OK;
}

dpca_status dpca_set_omega(dpca_handle *hh, const double *omega) {
    clear_error();
    if (!hh || !omega) return DPCA_ERR_INVALID;
    Handle *h = &hh->h;
    DPCA_CUDA(cudaSetDevice(h->device));
    DPCA_CUDA(cudaMemcpyAsync(h->omega, omega, (size_t)h->n_ind * h->k * 8, cudaMemcpyHostToDevice, h->stream));
    return DPCA_OK;
}

dpca_status dpca_pass(dpca_handle *hh) {
    clear_error();
    if (!hh) return DPCA_ERR_INVALID;
    DPCA_CUDA(cudaSetDevice(hh->h.device));
    return handle_pass(&hh->h);
}

dpca_status dpca_get_z(dpca_handle *hh, double *z) {
    clear_error();
    if (!hh || !z) return DPCA_ERR_INVALID;
    Handle *h = &hh->h;
    DPCA_CUDA(cudaSetDevice(h->device));
    DPCA_CUDA(cudaMemcpyAsync(z, h->z, (size_t)h->n_ind * h->k * 8, cudaMemcpyDeviceToHost, h->stream));
    DPCA_CUDA(cudaStreamSynchronize(h->stream));
    return check_device_flag(h);
}

dpca_status dpca_solve(dpca_handle *hh, const dpca_config *cfg, double *omega_inout, dpca_result *res) {
    clear_error();
    if (!hh) return DPCA_ERR_INVALID;
    DPCA_CUDA(cudaSetDevice(hh->h.device));
    return solve_impl(&hh->h, cfg, omega_inout, res);
}

dpca_status dpca_synchronize(dpca_handle *hh) {
    clear_error();
    if (!hh) return DPCA_ERR_INVALID;
    DPCA_CUDA(cudaSetDevice(hh->h.device));
    return check_device_flag(&hh->h);
}

dpca_status dpca_kernel_times(dpca_handle *hh, char *names, size_t cap_names, double *ms, int64_t *launches,
                              int *count, int cap) {
    clear_error();
    if (!hh || !count) return DPCA_ERR_INVALID;
    KernelClock &c = hh->h.clock;
    c.resolve();
    int n = (int)c.names.size();
    *count = n;
    std::string joined;
    for (int i = 0; i < n; ++i) {
        if (i) joined += ';';
        joined += c.names[i];
        if (i < cap) {
            if (ms) ms[i] = c.ms[i];
            if (launches) launches[i] = c.launches[i];
        }
    }
    if (names && cap_names) {
        strncpy(names, joined.c_str(), cap_names - 1);
        names[cap_names - 1] = 0;
    }
    return DPCA_OK;
}

dpca_status dpca_reset_kernel_times(dpca_handle *hh, int enable) {
    clear_error();
    if (!hh) return DPCA_ERR_INVALID;
    hh->h.clock.reset();
    hh->h.clock.enabled = enable != 0;
    return DPCA_OK;
}

dpca_status dpca_inject_fault(dpca_handle *hh, int fault, double wait_limit_ms) {
    clear_error();
    if (!hh || fault < 0 || fault > 1 || !(wait_limit_ms > 0.0) || wait_limit_ms > 10000.0) {
        set_error("dpca_inject_fault: fault must be 0 or 1 and the wait limit in (0, 10000] ms");
        return DPCA_ERR_INVALID;
    }
    Handle *h = &hh->h;
    if (h->precision != DPCA_PREC_MIXED) {
        set_error("dpca_inject_fault: the fault is in the mixed-precision product kernel");
        return DPCA_ERR_UNSUPPORTED;
    }
    int clock_khz = 0;
    DPCA_CUDA(cudaDeviceGetAttribute(&clock_khz, cudaDevAttrClockRate, h->device));
    h->inject_fault = fault;
    // cycles at the highest SM clock: the wait lasts at least the requested time
    h->inject_wait_cycles = (long long)(wait_limit_ms * (double)std::max(clock_khz, 1000));
    return DPCA_OK;
}

dpca_status dpca_decode_counts(const uint8_t *packed, int64_t row_stride, int n_ind, int n_snp, int32_t *counts,
                               double *avg, double *sd) {
    clear_error();
    // on the calling thread's current device (cudaSetDevice before the call picks another)
    int dev = 0;
    DPCA_CUDA(cudaGetDevice(&dev));
    dpca_handle *hh = nullptr;
    DPCA_TRY(dpca_create(&hh, n_ind, n_snp, 1, DPCA_PREC_FP64, dev, nullptr));
    dpca_status st = dpca_upload(hh, packed, row_stride);
    if (st == DPCA_OK) st = dpca_snp_stats(hh, counts, avg, sd, nullptr);
    dpca_destroy(hh);
    return st;
}

}  // extern "C"
