/*
 * dpca.h -- C ABI of libdpca, a GB300-native (sm_103a) drop-in for DistPCA's
 * randomized subspace-iteration PCA on PLINK SNP-major .bed genotypes.
 *
 * Conventions
 *   - Every entry point returns dpca_status; nothing calls exit().  The text
 *     of the last failure on the calling thread is in dpca_last_error().
 *   - Host buffers are caller-owned.  Device state hangs off an opaque
 *     dpca_handle that one host thread drives; work is ordered on one CUDA
 *     stream (the handle's own, or one the caller passes in).
 *   - Matrices are row-major.  n_ind = individuals (.fam rows, the
 *     reference's M), n_snp = markers (.bim rows, the reference's N),
 *     nrhs = subspace width k.  Omega and the Ritz block are n_ind x nrhs.
 *   - There is no CPU fallback: entry points that compute need a CUDA
 *     device and return DPCA_ERR_CUDA when none is usable.
 *
 * Reference interfaces replaced (paths relative to the DistPCA checkout):
 *   dpca_run / dpca_run_packed / dpca_solve
 *       BlockSubspaceIter_MPI_OOC_double_buffering  src/methods.h:49, src/methods.cpp:702
 *       SubspaceIteration_MPI (bsize >= n_snp)      src/methods.h:48, src/methods.cpp:24
 *   dpca_pass
 *       the pass lambda _compute_matvec_buff         src/methods.cpp:786-936
 *   dpca_snp_stats / dpca_decode_counts
 *       decode_plink_sse2 + standardize + LUT cache  src/utilities.cpp:272-306, 351-480;
 *                                                    src/methods.cpp:819-843
 *   dpca_start_block
 *       start-block RNG loop                         src/distpca.cpp:384-394, src/gennorm.c:21-72
 *   dpca_config_init / dpca_parse_args / dpca_resolve_config
 *       initialize_structure, findarg, main's clamps src/utilities.cpp:195-232, src/io.c:24-67,
 *                                                    src/distpca.cpp:83-352
 *   dpca_probe_bfile
 *       .fam/.bim line counting                      src/distpca.cpp:102-189
 *   dpca_write_outputs / dpca_print_statistics
 *       -fwrite writer and statistics block          src/methods.cpp:1077-1118, src/utilities.cpp:147-193
 */
#ifndef DPCA_H
#define DPCA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    DPCA_OK = 0,
    DPCA_ERR_INVALID = 1,     /* bad argument or inconsistent sizes */
    DPCA_ERR_IO = 2,          /* file missing, unreadable or short */
    DPCA_ERR_FORMAT = 3,      /* .bed magic/mode wrong or size does not match .fam/.bim */
    DPCA_ERR_CUDA = 4,        /* CUDA runtime/driver error or no device */
    DPCA_ERR_NOMEM = 5,       /* host or device allocation failed */
    DPCA_ERR_UNSUPPORTED = 6, /* shape outside the kernels' limits (e.g. nrhs > 128) */
    DPCA_ERR_TIMEOUT = 7,     /* a bounded device-side wait gave up */
    DPCA_ERR_NUMERIC = 8      /* non-finite values in the iteration */
} dpca_status;

typedef enum {
    DPCA_PREC_FP64 = 0,  /* plain path: FP64 standardized values, FP64 products */
    DPCA_PREC_MIXED = 1  /* exact 0/1/2 genotypes x hi+lo FP16 operands on tcgen05, FP32 accumulate */
} dpca_precision;

/* Run configuration: the DistPCA.exe flags plus device knobs. */
typedef struct {
    int nsv;           /* -nsv     sought PCs (default 10) */
    int nrhs;          /* -nrhs    subspace width (default 20) */
    int power;         /* -power   passes per outer iteration minus one (default 1) */
    int crit;          /* -crit    0 trace, 1 per-sigma (default), 2 MEV */
    int miter;         /* -miter   outer iterations (default 100) */
    int bsize;         /* -bsize   SNPs per block; <= 0 picks one from -memory/RAM like the reference */
    int verbose;       /* -verbose (default 1) */
    int fwrite;        /* -fwrite  write the two result files (default 0) */
    int full_svd;      /* -fullSVD accuracy check against a dense SVD (default 0) */
    double tol;        /* -tol     (default 1e-3) */
    double memory_gb;  /* -memory  host memory budget used by the block-size rule (0 = RAM/10) */
    char prefix[1024]; /* -prefix  output prefix (default "noprefix") */
    int precision;     /* dpca_precision (default DPCA_PREC_MIXED) */
    int device;        /* CUDA device ordinal (default 0) */
    double hbm_budget_gb; /* -hbm: device bytes (GB) the resident packed matrix may use; above it (or,
                             when 0, above 85% of the free device memory) dpca_run streams the rows
                             from host memory in blocks */
} dpca_config;

/* Results and the reference's timers (seconds).  sigma and u are caller-owned. */
typedef struct {
    int n_ind, n_snp, nsv, nrhs;
    int rows_fetched;   /* block size after the reference's clamps */
    int total_its;      /* outer iterations performed */
    int passes;         /* applications of X^T X */
    int in_core;        /* 1 when the in-core variant's Gram-form Rayleigh quotient was used */
    int streamed;       /* 1 when packed blocks were streamed from host memory each pass */
    double *sigma;      /* [nsv]            singular values (sqrt of Ritz values) */
    double *u;          /* [n_ind * nsv]    left singular vectors, row-major */
    double *delta_iter; /* [miter] or NULL  sum of sigma per iteration */
    double time_generate_rhs, time_load_matrix, time_mm, time_mm_a, time_mm_a_t;
    double time_gs, time_projected_svd, time_other, time_total;
    /* -fullSVD results as the statistics block reports them (distpca.cpp's TIME_2_TRUE_SVD,
     * frob_norm_angle, cos_error); zero until dpca_full_svd fills a dpca_fullsvd */
    double time_true_svd, frob_norm_angle, cos_error;
} dpca_result;

/* The -fullSVD accuracy check: the dense SVD of the standardized matrix compared with a result.
 * Arrays are caller-owned; true_u and vec_relerr may be NULL. */
typedef struct {
    int info;              /* 0 on success (the eigensolver's info otherwise) */
    double time_true_svd;  /* seconds for the dense decomposition */
    double frob_norm_angle;/* ||(Uhat^T U) with |diagonal| - I||_F */
    double cos_error;      /* ||(Uhat^T U) with |diagonal| - I||_2 */
    double *true_sigma;    /* [nsv] leading singular values */
    double *true_u;        /* [n_ind * nsv] leading left singular vectors, row-major */
    double *sigma_relerr;  /* [nsv] |sigma_true - sigma| / sigma_true */
    double *vec_relerr;    /* [n_ind * nsv] ||u_true| - |u|| / (|u_true| + 1e-12) */
    double *cosines;       /* [nsv] diagonal of Uhat^T U */
} dpca_fullsvd;

typedef struct dpca_handle dpca_handle;

/* ---- host-side configuration (no device needed) ---- */
const char *dpca_status_string(dpca_status s);
const char *dpca_last_error(void);
const char *dpca_version(void);
void dpca_config_init(dpca_config *cfg);
/* findarg semantics: "-name value", first match wins, atoi/atof. bfile gets -bfile. */
dpca_status dpca_parse_args(int argc, char **argv, dpca_config *cfg, char *bfile, size_t bfile_cap);
/* n_ind/n_snp from .fam/.bim line counts; checks .bed exists, magic 6C 1B 01 and size. */
dpca_status dpca_probe_bfile(const char *bfile, int *n_ind, int *n_snp);
/* The reference's clamps on nsv/nrhs/bsize (distpca.cpp:239-352); writes the final block size. */
dpca_status dpca_resolve_config(dpca_config *cfg, int n_ind, int n_snp, int *rows_fetched);
/* Start block, bit-identical to the reference RNG loop: n_ind x k row-major. */
dpca_status dpca_start_block(int n_ind, int k, double *out);
/* The Rayleigh-Ritz eigenproblem (LAPACKE_dsyev 'V','U' and the column reversal,
 * src/methods.cpp:981-1000) on the host: b is k x k row-major (upper triangle used); w gets the
 * eigenvalues in descending order, W (k x k row-major) the eigenvectors as columns.  Householder
 * tridiagonalization + implicit symmetric QR with Wilkinson shifts, dsyev's method.  A host-side
 * utility: the solve itself runs this step on the device (dpca_sym_eig_device). */
dpca_status dpca_sym_eig(int k, const double *b, double *w, double *W);
/* The same eigenproblem with the device kernel every outer iteration of a solve uses (one block,
 * parallel cyclic Jacobi in FP64, k <= 128), on `device`; b, w, W are host arrays as above.
 * DPCA_ERR_NUMERIC when it does not converge. */
dpca_status dpca_sym_eig_device(int device, int k, const double *b, double *w, double *W);
/* The thin QR every solve runs on its n x k panels (dgeqrf + dorgqr in the reference,
 * src/methods.cpp:947-961; here shifted CholeskyQR3 on the device), on `device`: a is an n x k
 * row-major host array, n >= 1, 1 <= k <= the nrhs limit, overwritten by Q.  separate = 1 runs
 * the step as separate kernels instead of the one cooperative launch the solve takes when it
 * fits; both give the same bits. */
dpca_status dpca_qr_device(int device, int n, int k, double *a, int separate);

/* ---- whole runs (device) ---- */
/* Read <bfile>.bed/.bim/.fam and run.  omega_inout: start block in, final Ritz block out. */
dpca_status dpca_run(const dpca_config *cfg, const char *bfile, double *omega_inout, dpca_result *res);
/* Same from packed rows already in host memory (row_stride bytes apart, >= ceil(n_ind/4)). */
dpca_status dpca_run_packed(const dpca_config *cfg, const uint8_t *packed, int64_t row_stride, int n_ind,
                            int n_snp, double *omega_inout, dpca_result *res);
/* Write <prefix>_singularValues.txt and <prefix>_leftSingularVectors.txt (IIDs from <bfile>.fam). */
dpca_status dpca_write_outputs(const dpca_config *cfg, const char *bfile, const dpca_result *res);
void dpca_print_statistics(const dpca_config *cfg, const dpca_result *res);
/* -fullSVD (distpca.cpp:449-635, computeCosineError utilities.cpp:234-270): the dense SVD of the
 * standardized matrix on the device -- the FP64 Gram matrix X^T X (n_ind x n_ind) from the packed
 * rows and its symmetric eigendecomposition -- compared with res (sigma, u).  Rows come from
 * packed (host, row_stride apart) or, when packed is NULL, from <bfile>.bed.  n_ind is limited
 * to 20,000 (DPCA_ERR_UNSUPPORTED above).  With verbose > 1 it prints the reference's lines. */
dpca_status dpca_full_svd(const dpca_config *cfg, const char *bfile, const uint8_t *packed, int64_t row_stride,
                          int n_ind, int n_snp, const dpca_result *res, dpca_fullsvd *out);
/* The four -fullSVD -fwrite files: <prefix>_realLeftSingularVectors.txt, _realSingularValues.txt,
 * _singvecs_accuracy.txt, _cosineValues.txt (timestamped names without a prefix). */
dpca_status dpca_write_fullsvd(const dpca_config *cfg, const char *bfile, int n_ind, int nsv,
                               const dpca_fullsvd *f);

/* ---- device-resident handle ---- */
/* stream: a cudaStream_t to order work on, or NULL for a handle-owned stream. */
dpca_status dpca_create(dpca_handle **h, int n_ind, int n_snp, int nrhs, int precision, int device, void *stream);
/* Streaming handle (the out-of-core block reader, src/methods.cpp:795-811, 873-874): the device
 * holds two blocks of block_snps SNP rows (rounded up to 128) and, on the mixed path, their
 * transposes.  dpca_upload then only records the host rows, which must stay valid and unchanged
 * until the handle is destroyed (pinned memory copies at full speed), and computes the per-SNP
 * statistics in one sweep; every pass copies the blocks in on a side stream, double-buffered,
 * and accumulates Z over them.  dpca_synth_fill is not available on such a handle. */
dpca_status dpca_create_streamed(dpca_handle **h, int n_ind, int n_snp, int nrhs, int precision, int device,
                                 void *stream, int block_snps);
dpca_status dpca_destroy(dpca_handle *h);
/* Copy packed rows (host, pinned or pageable) to the device and compute per-SNP statistics. */
dpca_status dpca_upload(dpca_handle *h, const uint8_t *packed, int64_t row_stride);
/* The rows of <bed_path> (a SNP-major .bed; its magic is checked), read with positional reads of
 * whole SNP blocks at 3 + ceil(n_ind/4) * first_snp (the block reader of src/methods.cpp:795-811,
 * 873-874), through a ring of three pinned staging blocks that a reader thread fills ahead of the
 * device.  A resident handle reads the file once; a streaming handle reads every block from the
 * file in every pass and never holds the whole matrix in host memory.  A read that comes up short
 * returns DPCA_ERR_IO. */
dpca_status dpca_upload_file(dpca_handle *h, const char *bed_path);
/* Rows handed out block by block by a caller callback (a decompressor, a network receiver, a
 * synthetic generator): fn(ctx, first_snp, n_rows, &rows, &row_stride) stores the host address of
 * SNP rows [first_snp, first_snp + n_rows) and their stride (>= ceil(n_ind/4), <= max_row_stride)
 * and returns 0 (non-zero: the call that needed the rows fails with DPCA_ERR_IO).  The rows are
 * copied to the device in place (at full speed when pinned) by stream-ordered copies, so they must
 * stay valid and unchanged until the work that reads them has finished (dpca_synchronize,
 * dpca_get_z, or the return of dpca_solve).  A streaming handle calls fn for every block of every
 * pass; a resident handle once per 256 MB chunk. */
typedef int (*dpca_block_fn)(void *ctx, int64_t first_snp, int n_rows, const uint8_t **rows, int64_t *row_stride);
dpca_status dpca_upload_blocks(dpca_handle *h, dpca_block_fn fn, void *ctx, int64_t max_row_stride);
/* Fill the device matrix with a seeded Balding-Nichols cohort (tables as in distpca_gb300/synth.py):
 * pop[n_ind] uint8, miss_thr[n_ind] uint32, snp_thr[n_snp * n_pop] uint32 (host arrays). */
dpca_status dpca_synth_fill(dpca_handle *h, uint64_t key, const uint8_t *pop, const uint32_t *miss_thr,
                            const uint32_t *snp_thr, int n_pop);
/* Download packed rows [s0, s1) (row-major, ceil(n_ind/4) bytes per row). */
dpca_status dpca_download_packed(dpca_handle *h, int s0, int s1, uint8_t *out);
/* Per-SNP statistics: counts[4*n_snp] = {hom A1 (00), missing (01), het (10), hom A2 (11)},
 * avg/sd as standardize() computes them, lut[4*n_snp] = standardized value per raw code. */
dpca_status dpca_snp_stats(dpca_handle *h, int32_t *counts, double *avg, double *sd, double *lut);
dpca_status dpca_set_omega(dpca_handle *h, const double *omega);
/* One pass Z = X^T X Omega on the device, stream-ordered (no host sync). */
dpca_status dpca_pass(dpca_handle *h);
dpca_status dpca_get_z(dpca_handle *h, double *z);
/* Full solve on the resident matrix. */
dpca_status dpca_solve(dpca_handle *h, const dpca_config *cfg, double *omega_inout, dpca_result *res);
dpca_status dpca_synchronize(dpca_handle *h);
/* Per-kernel device time (ms) and launch counts accumulated since the last reset, via CUDA events
 * recorded on the handle's stream around each launch.  names: ';'-separated list. */
dpca_status dpca_kernel_times(dpca_handle *h, char *names, size_t names_cap, double *ms, int64_t *launches,
                              int *count, int cap);
dpca_status dpca_reset_kernel_times(dpca_handle *h, int enable);
/* Autotuner of the mixed-precision product kernels (no counterpart in the reference, whose
 * products are MKL calls): measures, on this handle's resident matrix and current Omega, the
 * cluster width of both products (CTAs sharing each dense-operand stage by multicast), X^T Y's
 * grid mode (persistent or one CTA per work item) and K-split count, and both ring depths, one
 * choice after another, with CUDA events; keeps the fastest for this handle and remembers it for
 * the handle's shape class (individual tiles, SNP blocks and padded nrhs, one octave per class),
 * which handles created later in the process start from.  report (may be NULL) gets a JSON
 * object with the default and tuned times in ms and the choices. */
dpca_status dpca_autotune(dpca_handle *h, char *report, size_t report_cap);

/* ---- test hook: device-side failure detection without a GPU fault ----
 * Every barrier wait in the product kernels is bounded; when one runs out the kernel records the
 * site in a device flag, waits (bounded) for its own copies and MMAs in flight, frees its tensor
 * memory and returns, and the next call that reads results reports DPCA_ERR_TIMEOUT with the
 * handle still usable.  fault = 1 makes the next mixed X Omega launch of this handle withhold one
 * load (its first CTA's first batch never arrives), so that the MMA issuer's wait for it runs out
 * after wait_limit_ms (the normal limit is ~4 s); the setting applies to that one launch.
 * fault = 0 clears it.  A mixed-precision handle only (DPCA_ERR_UNSUPPORTED otherwise). */
dpca_status dpca_inject_fault(dpca_handle *h, int fault, double wait_limit_ms);

/* ---- unit-parity entry: decode + counts for packed rows in host memory, on the calling
 * thread's current CUDA device ---- */
dpca_status dpca_decode_counts(const uint8_t *packed, int64_t row_stride, int n_ind, int n_snp, int32_t *counts,
                               double *avg, double *sd);

/* ---- allocation-free pass (no counterpart in the reference) ----
 * One plain FP64 pass Z = X^T (X Omega) -- per-SNP statistics, then both products, the same
 * kernels as a DPCA_PREC_FP64 handle's dpca_pass -- on device buffers the caller owns, without
 * allocating any device or host memory.  It is for callers that cannot let a library call
 * cudaMalloc: applications that hand out all device memory from their own fixed-budget pool,
 * and latency-sensitive loops in which an allocation, which can synchronise the device, is not
 * acceptable.
 *   packed  device pointer, 16-byte aligned: n_snp SNP-major rows of ceil(n_ind/4) .bed bytes,
 *           row_stride bytes apart (a multiple of 16, at least ceil(n_ind/4) rounded up to 32)
 *   omega   device pointer, n_ind x nrhs row-major FP64 (nrhs <= 128)
 *   z       device pointer, n_ind x nrhs row-major FP64, written
 *   stream  cudaStream_t to launch on (NULL: the default stream); the call returns without
 *           waiting for the work
 * Its working buffers live in one static device array of 32 MiB that every GPU which loads the
 * library holds until the process exits; inputs whose statistics, Y and one split of partial
 * sums do not fit (about 64 + 8*nrhs bytes per SNP plus 8*nrhs bytes per individual) are
 * rejected with DPCA_ERR_UNSUPPORTED before any work is queued.  The first call on a device
 * looks up the array's device address (cudaGetSymbolAddress) and raises the shared-memory limit
 * of every kernel the entry point may launch, so make that first call before any stream
 * capture.  The address belongs to the CUDA context current at that call; a call in a different
 * context (another context the caller made current, or the device's new primary context after
 * cudaDeviceReset) repeats the set-up, so the first call after such a change also belongs
 * outside capture.  All calls share the array: calls whose work overlaps on the GPU race on
 * it, so serialise them (one stream, or events between streams). */
dpca_status dpca_pass_fp64_noalloc(const uint8_t *packed, int64_t row_stride, int n_ind, int n_snp,
                                   const double *omega, int nrhs, double *z, void *stream);

/* ---- batched local PCA over SNP windows ----
 * The reference runs one PCA per invocation (src/distpca.cpp:83-405).  A dpca_windows object
 * holds W independent PCA problems that share the individuals: window w is the next win_snps[w]
 * SNP rows of one packed matrix (consecutive windows, sum(win_snps) rows), standardized on its
 * own (1/sqrt(win_snps[w]) in place of 1/sqrt(n_snp), src/utilities.cpp:294-305).  dpca_windows_solve
 * runs the subspace iteration of dpca_solve on every window at once -- mixed precision, a full
 * pass for the Rayleigh quotient (bsize < n_snp) -- with one launch of each kernel per step for
 * all windows still iterating; a window stops at its own convergence test (cfg->crit, tol,
 * miter) and keeps its result.  nrhs <= 48, at most 65,535 windows. */
typedef struct dpca_windows dpca_windows;
dpca_status dpca_windows_create(dpca_windows **w, int n_ind, int n_win, const int *win_snps, int nrhs, int device,
                                void *stream);
dpca_status dpca_windows_destroy(dpca_windows *w);
/* Packed host rows of all windows in order (row_stride >= ceil(n_ind/4) bytes apart). */
dpca_status dpca_windows_upload(dpca_windows *w, const uint8_t *packed, int64_t row_stride);
/* A seeded Balding-Nichols cohort over sum(win_snps) SNPs (the dpca_synth_fill tables). */
dpca_status dpca_windows_synth_fill(dpca_windows *w, uint64_t key, const uint8_t *pop, const uint32_t *miss_thr,
                                    const uint32_t *snp_thr, int n_pop);
/* omega0: n_ind x nrhs start block for every window (NULL: dpca_start_block's).  Outputs:
 * sigma[n_win * nsv]; u[n_win * n_ind * nsv] or NULL; its[n_win] outer iterations or NULL. */
dpca_status dpca_windows_solve(dpca_windows *w, const dpca_config *cfg, const double *omega0, double *sigma,
                               double *u, int *its);
/* The handle the windows run on, for dpca_kernel_times / dpca_reset_kernel_times. */
dpca_handle *dpca_windows_handle(dpca_windows *w);

/* ---- serving loop: many independent PCA jobs on one GPU ----
 * The reference runs one PCA per MPI job: main reads one .bed and calls the solver once
 * (src/distpca.cpp:83-405 -> BlockSubspaceIter_MPI_OOC_double_buffering, src/methods.h:49).
 * A dpca_server accepts such jobs as they arrive -- different cohorts, SNP sets, nsv and nrhs --
 * and runs up to `slots` of them at once on one device, each on its own stream and host worker
 * thread.  Admission: in arrival order, when a slot is free and the job's device footprint fits
 * the memory budget beside the jobs in flight; a later job that fits may pass one that does not
 * fit yet, at most 2*slots times for that job.  A job's packed genotypes and subspace state stay
 * on the device until it finishes.  Its buffers are stream-ordered allocations from the device's
 * memory pool, so admitting and retiring jobs never synchronises the device under the other
 * jobs' work.  A job's result is the one dpca_solve gives for the same inputs alone: the kernels
 * are deterministic and jobs share no device state.  Jobs larger than the whole budget fail with
 * DPCA_ERR_NOMEM at submission. */
typedef struct dpca_server dpca_server;

typedef struct {
    int device;
    int slots;            /* jobs in flight at once, 1..64 (0: 4) */
    double hbm_budget_gb; /* device memory the jobs in flight may hold (<= 0: 85% of the free memory) */
} dpca_serve_config;

typedef struct {
    int n_ind, n_snp;
    /* nsv, nrhs, power, crit, tol, miter, precision; bsize >= n_snp selects the in-core variant.
     * verbose, fwrite, full_svd, prefix, memory_gb, device and hbm_budget_gb are not used. */
    dpca_config cfg;
    /* Genotypes: packed host rows (SNP-major, .bed bytes, row_stride >= ceil(n_ind/4) apart), or,
     * when packed is NULL, a seeded Balding-Nichols cohort filled on the device from the
     * dpca_synth_fill tables.  Every array must stay valid until the job is done. */
    const uint8_t *packed;
    int64_t row_stride;
    uint64_t synth_key;
    const uint8_t *synth_pop;        /* [n_ind] */
    const uint32_t *synth_miss_thr;  /* [n_ind] */
    const uint32_t *synth_snp_thr;   /* [n_snp * synth_n_pop] */
    int synth_n_pop;
    const double *omega;  /* start block n_ind x nrhs, or NULL for dpca_start_block's */
    double *sigma;        /* [nsv], written when the job is done */
    double *u;            /* [n_ind * nsv] or NULL, written when the job is done */
} dpca_job;

typedef struct {
    int status;           /* dpca_status of the job */
    int total_its, passes;
    double t_submit, t_start, t_done;  /* seconds since dpca_serve_create */
    double device_gb;     /* footprint admitted against the budget */
    char error[256];
} dpca_job_info;

dpca_status dpca_serve_create(dpca_server **out, const dpca_serve_config *cfg);
/* Queue a job; thread-safe.  The dpca_job is copied, the arrays it points to are not. */
dpca_status dpca_serve_submit(dpca_server *s, const dpca_job *job, int64_t *job_id);
/* Non-blocking: *done = 1 and *info (may be NULL) filled once the job has finished. */
dpca_status dpca_serve_poll(dpca_server *s, int64_t job_id, int *done, dpca_job_info *info);
/* Block until the job has finished (DPCA_ERR_TIMEOUT after timeout_s seconds; < 0 waits forever). */
dpca_status dpca_serve_wait(dpca_server *s, int64_t job_id, double timeout_s, dpca_job_info *info);
/* Jobs finished, most jobs in flight at once, most device bytes admitted at once, the budget. */
dpca_status dpca_serve_stats(dpca_server *s, int64_t *done, int *max_in_flight, double *peak_gb, double *budget_gb);
/* Finish every submitted job, stop the workers and free the server. */
dpca_status dpca_serve_shutdown(dpca_server *s);

#ifdef __cplusplus
}
#endif

#endif /* DPCA_H */
