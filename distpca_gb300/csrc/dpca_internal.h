// Internal declarations shared by the host (.cpp) and device (.cu) parts of libdpca.
#pragma once

#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <condition_variable>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "dpca.h"

namespace dpca {

void set_error(const char *fmt, ...);
void clear_error();

#define DPCA_TRY(expr)                                 \
    do {                                               \
        dpca_status st_ = (expr);                      \
        if (st_ != DPCA_OK) return st_;                \
    } while (0)

#define DPCA_CUDA(call)                                                                                  \
    do {                                                                                                 \
        cudaError_t e_ = (call);                                                                         \
        if (e_ != cudaSuccess) {                                                                         \
            ::dpca::set_error("%s:%d: %s -> %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_));     \
            return e_ == cudaErrorMemoryAllocation ? DPCA_ERR_NOMEM : DPCA_ERR_CUDA;                     \
        }                                                                                                \
    } while (0)

// Largest subspace width the device kernels accept (tcgen05 N <= 256 holds 2*nrhs).
constexpr int kMaxNrhs = 128;

// Per-kernel CUDA-event timing on the handle's stream.
struct KernelClock {
    struct Pending {
        int slot;
        cudaEvent_t a, b;
    };
    bool enabled = false;
    std::vector<std::string> names;
    std::vector<double> ms;
    std::vector<int64_t> launches;
    std::vector<Pending> pending;
    std::vector<cudaEvent_t> pool;
    int slot(const char *name);
    cudaEvent_t get_event();
    void resolve();  // accumulate finished pairs (synchronizes on their end events)
    void reset();
    ~KernelClock();
};

// Scoped timing of one launch: records events around the enclosed launch when enabled, and counts
// `kernels` launches for it (the kernels the scope encloses).
struct ScopedLaunch {
    KernelClock *clk;
    cudaStream_t st;
    int slot = -1;
    int kernels = 1;
    cudaEvent_t a = nullptr, b = nullptr;
    ScopedLaunch(KernelClock *c, cudaStream_t s, const char *name, int kernels = 1);
    ~ScopedLaunch();
};

// Where a handle's packed SNP rows come from (rows.cpp): a .bed file read with positional reads,
// caller rows in host memory, or a caller callback that hands out each block's rows.
struct RowSource {
    enum Kind { kNone, kMemory, kBlocks, kFile } kind = kNone;
    const uint8_t *base = nullptr;  // memory: row r at base + r * stride
    int64_t stride = 0;
    bool pinned = false;
    dpca_block_fn fn = nullptr;     // blocks
    void *ctx = nullptr;
    int64_t max_stride = 0;         // blocks: the largest row stride fn returns
    int fd = -1;                    // file
    int64_t header = 0;
    std::string path;
    int64_t np = 0;                 // bytes per row as stored contiguously in a ring slot = ceil(n_ind / 4)
    RowSource() = default;
    RowSource(const RowSource &) = delete;
    RowSource &operator=(const RowSource &) = delete;
    ~RowSource();
    dpca_status open_file(const char *bed_path, int64_t row_bytes);
    void set_memory(const uint8_t *rows, int64_t row_stride, int64_t row_bytes);
    void set_blocks(dpca_block_fn f, void *c, int64_t row_bytes, int64_t max_row_stride);
    // Rows [s0, s0 + rows) in place (memory and blocks sources); *pin says whether the copy
    // engine can read them directly.
    dpca_status direct(int64_t s0, int rows, const uint8_t **ptr, int64_t *row_stride, bool *pin) const;
    // Rows [s0, s0 + rows) copied into dst, np bytes per row (several threads).
    dpca_status read_into(int64_t s0, int rows, uint8_t *dst, std::string *err) const;
    // Whether blocks go through the pinned ring (file rows; memory and callback rows are copied in place).
    bool use_ring = false;
    // Row stride of what the device receives: np out of the ring, else the source's own stride.
    int64_t copy_stride() const { return use_ring ? np : kind == kMemory ? stride : max_stride; }
};

// Pinned host staging slots filled by a reader thread ahead of the device (rows.cpp).
class HostRing {
  public:
    static constexpr int kSlots = 3;
    ~HostRing();
    // Begin a sweep over blocks ({first row, rows} each) of src; slots are (re)allocated to fit.
    dpca_status start(const RowSource *src, std::vector<std::pair<int64_t, int>> blocks);
    // Wait (bounded) until block i of the sweep sits in a slot; *ptr = its rows, np bytes apart.
    dpca_status acquire(int i, const uint8_t **ptr);
    // Block i's copy out of its slot is enqueued on `stream`: the slot is refilled after it.
    dpca_status release(int i, cudaStream_t stream);
    size_t slot_size() const { return slot_bytes; }

  private:
    enum State { kFree, kFilling, kReady, kInUse, kReleased };
    struct Slot {
        uint8_t *buf = nullptr;
        cudaEvent_t done = nullptr;
        State state = kFree;
        int block = -1;
    };
    dpca_status ensure(size_t bytes);
    void shutdown();
    void reader_main();
    std::mutex mu;
    std::condition_variable cv;
    std::thread reader;
    std::vector<Slot> slots;
    size_t slot_bytes = 0;
    bool stop = false;
    const RowSource *sweep_src = nullptr;
    std::vector<std::pair<int64_t, int>> sweep;
    int next_read = 0;
    uint64_t generation = 0;
    dpca_status failed = DPCA_OK;
    std::string fail_msg;
};

struct Handle {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int n_ind = 0, n_snp = 0, k = 0, precision = DPCA_PREC_MIXED;
    int64_t np = 0;       // packed bytes per SNP row = ceil(n_ind/4)
    int64_t pitch = 0;    // device row pitch of P (multiple of 128 B)
    int64_t npT = 0;      // packed bytes per individual row of P^T = ceil(n_snp/4)
    int64_t pitchT = 0;   // device row pitch of P^T
    int n_ind_pad = 0;    // n_ind rounded up to 128 (operand padding)
    int n_snp_pad = 0;    // n_snp rounded up to 128
    double inv_sqrt_nsnp = 0;

    uint8_t *P = nullptr;    // SNP-major packed matrix, n_snp x pitch
    uint8_t *PT = nullptr;   // individual-major packed matrix (mixed path), pitchT bytes per individual,
                             // stored in contiguous 128-individual x 128-byte tiles

    // per-SNP statistics
    int32_t *counts = nullptr;  // [n_snp][4] codes 00,01,10,11
    double *avg = nullptr, *sd = nullptr;
    double *lut = nullptr;      // [n_snp][4] standardized value per raw code (times 1/sqrt(n_snp))
    double *coef = nullptr;     // [n_snp][2] mixed path: X = b*g + a*nonmissing -> {b, a}
    bool stats_ready = false;

    // dense FP64 state, n_ind x k row-major unless noted
    double *omega = nullptr, *z = nullptr, *q = nullptr, *old = nullptr, *work = nullptr;
    double *y = nullptr;        // n_snp x k (X Omega)
    double *partial = nullptr;  // split-K partials
    size_t partial_elems = 0;
    double *small = nullptr;    // k x k matrices, eigenvalues, sigma, scalars (see SmallLayout)
    double *red = nullptr;      // reduction scratch
    size_t red_elems = 0;
    int *dflag = nullptr;       // device error / status flags
    double *host_small = nullptr; // pinned mirror of small results

    // mixed-precision operands
    void *mx = nullptr;         // MixedState (k_mixed.cu)

    // Streaming (the packed matrix stays in host memory and is copied in blocks each pass).
    // Device buffers then hold `rows_dev` = blk SNP rows instead of n_snp.
    bool streamed = false;
    int blk = 0, nblk = 0;            // SNP rows per block (multiple of 128), number of blocks
    int rows_dev = 0;                 // SNP rows resident at a time: n_snp, or blk when streamed
    RowSource *src = nullptr;         // where the rows come from (set by dpca_upload*, owned)
    HostRing *ring = nullptr;         // pinned staging for sources the copy engine cannot read in place
    uint8_t *Pb[2] = {nullptr, nullptr};   // block buffers, blk x pitch
    uint8_t *PTb[2] = {nullptr, nullptr};  // mixed: block transposes, pitchTb per individual, tiled as PT
    int64_t pitchTb = 0;
    size_t sb_bytes = 0;
    uint8_t *Sb[2] = {nullptr, nullptr};   // staging for one contiguous host copy per block (host rows
                                           // whose stride is not the device pitch), re-pitched on device
    cudaStream_t cstream = nullptr;        // copy stream
    cudaEvent_t copied[2] = {nullptr, nullptr}, consumed[2] = {nullptr, nullptr};
    cudaEvent_t staged_free[2] = {nullptr, nullptr};  // Sb[b] re-pitched (recorded on the compute stream)

    // Device allocations: cudaMalloc, or stream-ordered on `stream` (cudaMallocAsync / cudaFreeAsync)
    // for handles of the serving loop, so that creating and freeing one job's buffers never
    // synchronises the device under the other jobs' work.  dev_bytes counts what is held.
    // Test hook (dpca_inject_fault): a fault for the next mixed X Omega launch and its wait limit.
    int inject_fault = 0;
    long long inject_wait_cycles = 0;

    bool async_alloc = false;
    cudaMemPool_t pool = nullptr;  // the pool stream-ordered allocations come from (NULL: the device's default)
    size_t dev_bytes = 0;

    KernelClock clock;
    // Coarse timing of a solve's stages (a pass's two products, a QR, the eigensolve) when the
    // per-launch clock is off: a few events per outer iteration instead of two per launch.
    KernelClock *stage = nullptr;
    bool no_graphs = false;  // solves launch every iteration eagerly (serving handles)
    int qr_coresident = 0;  // blocks of the fused QR kernel that fit at once (0: not queried, -1: none)
};

// Raise a kernel's dynamic shared-memory limit to the current device's opt-in maximum, once
// per (kernel, CUDA context).  The limit is a process-wide function attribute: setting it to each
// launch's own size races between host threads that launch the same kernel with different
// sizes (the serving loop's workers), so it is set once, to the largest value.  It belongs to
// the context, so a context created later (after cudaDeviceReset) gets it set again.
dpca_status allow_max_smem(const void *func);
// Unique id (cuCtxGetId) of the calling thread's current CUDA context.
dpca_status current_context_id(unsigned long long *id);

dpca_status dev_alloc(Handle *h, void **p, size_t bytes);
void dev_free(Handle *h, void *p);
// Device bytes a resident handle of these sizes holds (what create_impl and mixed_prepare allocate).
size_t handle_footprint(int n_ind, int n_snp, int nrhs, int precision, int sm_count);
size_t mixed_footprint(int n_ind, int n_snp, int nrhs, int sm_count);
// Resident handle for the serving loop: stream-ordered allocations from `pool` on `stream`, pageable
// result mirror.
dpca_status create_serving_handle(dpca_handle **out, int n_ind, int n_snp, int nrhs, int precision, int device,
                                  cudaStream_t stream, cudaMemPool_t pool);

// Offsets (in doubles) inside Handle::small.
struct SmallLayout {
    int k;
    __host__ __device__ size_t B() const { return 0; }                    // k*k Rayleigh / Gram matrix
    __host__ __device__ size_t W() const { return (size_t)k * k; }        // k*k eigenvectors (descending)
    __host__ __device__ size_t w() const { return 2 * (size_t)k * k; }    // k eigenvalues (descending)
    __host__ __device__ size_t sigma() const { return w() + k; }          // k
    __host__ __device__ size_t sigma_old() const { return sigma() + k; }  // k
    __host__ __device__ size_t dots() const { return sigma_old() + k; }   // k MEV dot products
    __host__ __device__ size_t tau() const { return dots() + k; }         // k Householder scalars
    __host__ __device__ size_t crit() const { return tau() + k; }         // [0] criterion value, [1] stop flag, [2] sum sigma
    __host__ __device__ size_t total() const { return crit() + 8; }
};

// ---- launchers (device code in .cu files); all stream-ordered on h->stream ----
dpca_status launch_snp_stats(Handle *h);
dpca_status launch_synth_fill(Handle *h, uint64_t key, const uint8_t *d_pop, const uint32_t *d_miss,
                              const uint32_t *d_thr, int n_pop, const int *d_row_src = nullptr);
dpca_status launch_transpose_packed(Handle *h);
void launch_snp_stats_raw(const uint8_t *P, int64_t pitch, int n_ind, int n_snp, double inv_sqrt_nsnp,
                          int32_t *counts, double *avg, double *sd, double *lut, double *coef, cudaStream_t stream,
                          const double *row_inv_sqrt = nullptr);
void launch_transpose_raw(const uint8_t *P, int64_t pitch, uint8_t *PT, int64_t pitchT, int n_ind, int n_snp,
                          cudaStream_t stream, int s_base = 0);
// one streamed block: Z (+)= X_b^T (X_b Omega) over SNP rows [s0, s0 + ns) held in buffer b
dpca_status launch_fp64_block(Handle *h, int b, int s0, int ns, const double *omega, double *z, bool accumulate);
dpca_status mixed_omega_operand(Handle *h, const double *omega);
// -fullSVD: leading nsv singular values / left vectors (host, n_ind x nsv) of a resident FP64
// handle created with nrhs = 128
dpca_status full_svd_device(Handle *h, int nsv, double *sigma, double *u, int *info);
dpca_status mixed_block(Handle *h, int b, int s0, int ns, double *z, bool accumulate);
dpca_status launch_fp64_xw(Handle *h, const double *omega, double *y);
dpca_status launch_fp64_xty(Handle *h, const double *y, double *z);
dpca_status launch_qr(Handle *h, double *a);
dpca_status launch_atb(Handle *h, const double *a, const double *b, int n, double *out);  // k x k = A^T B
dpca_status launch_eig_desc(Handle *h);                                                   // small.B -> W, w
dpca_status host_sym_eig_desc(int k, const double *B, double *w, double *W);              // eig_host.cpp
dpca_status launch_apply_w(Handle *h, const double *q, double *out);                      // out = Q W
dpca_status launch_sigma_and_criterion(Handle *h, int nsv, int crit, double tol, int ii, const double *old,
                                       const double *omega);

// One mixed pass over W batched windows (k_mixed.cu mixed_win_pass): Z_w = X_w^T X_w Omega_w for
// every active window, on a mixed handle whose rows are the windows' SNPs, each window padded
// to whole 512-row blocks (padding rows have zero coefficients).
struct WinPass {
    int W = 0;
    const double *omega = nullptr;  // [W][n][k]
    double *z = nullptr;            // [W][n][k]
    const int *tile_win = nullptr;  // [rows / 128] window of each 128-row tile
    const int *win_kb0 = nullptr, *win_nkb = nullptr;  // [W] 64-SNP K-block range of each window
    const int *active = nullptr;    // [W] 0 = converged (skipped)
    __half *omega_s = nullptr;      // [W * 2 kp][n_pad] FP16 slices
    double *scales = nullptr;       // [W][4][k]
    unsigned int *colmax = nullptr; // [W][k]
    long long *colsumq = nullptr, *rq = nullptr;  // [W][k]
    double *partial = nullptr;      // [W][n][k]
    CUtensorMap *map_om = nullptr;  // B map over omega_s (built on first use)
    mutable bool map_ready = false;
};
dpca_status mixed_win_pass(Handle *h, const WinPass &p);

// mixed-precision pass (k_mixed.cu)
dpca_status mixed_prepare(Handle *h);
dpca_status mixed_release(Handle *h);
dpca_status launch_mixed_xw(Handle *h, const double *omega, double *y_out_or_null);
dpca_status launch_mixed_xty(Handle *h, double *z);

// host-side helpers shared between translation units
dpca_status handle_pass(Handle *h);
// Reads the device flags (synchronises the stream): DPCA_ERR_TIMEOUT when a bounded device wait
// gave up (flag 0), DPCA_ERR_NUMERIC when a device k x k solve did not converge (flag 1).
dpca_status check_device_flag(Handle *h);
bool env_flag(const char *name);

}  // namespace dpca

struct dpca_handle {
    dpca::Handle h;
};
