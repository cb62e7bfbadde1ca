// Host side of libdpca: error reporting, the DistPCA.exe configuration rules, .bed/.bim/.fam
// probing and reading, the start-block RNG, whole runs and the result writers.
#include <cuda_runtime.h>
#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "dpca_internal.h"

namespace dpca {

static thread_local std::string g_last_error;

void set_error(const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
}

void clear_error() { g_last_error.clear(); }

static double wall_now() {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

// Lines terminated by '\n', counted the way distpca.cpp:137-147 counts them (a final line
// without a newline is not counted); tokens[col] of each counted line is collected.
static dpca_status read_lines(const std::string &path, int col, std::vector<std::string> *tokens, int *count) {
    std::ifstream in(path.c_str(), std::ios::in);
    if (!in) {
        set_error("Error reading file '%s': %s", path.c_str(), strerror(errno));
        return DPCA_ERR_IO;
    }
    int n = 0;
    while (in) {
        std::string line;
        std::getline(in, line);
        if (!in.eof()) {
            if (tokens) {
                std::stringstream ss(line);
                std::string t;
                std::vector<std::string> toks;
                while (ss >> t) toks.push_back(t);
                tokens->push_back((int)toks.size() > col ? toks[col] : std::string());
            }
            n++;
        }
    }
    *count = n;
    return DPCA_OK;
}

static int ram_kb() {
    FILE *f = fopen("/proc/meminfo", "r");
    if (!f) return -1;
    char line[256];
    int kb = -1;
    while (fgets(line, sizeof(line), f))
        if (sscanf(line, "MemTotal: %d kB", &kb) == 1) break;
    fclose(f);
    return kb;
}

static std::string construct_filename(const std::string &pure, const char *type) {
    time_t raw;
    time(&raw);
    struct tm *ti = localtime(&raw);
    char mon[16];
    // utilities.cpp:137-140: zero-padded only while month+1 < 9
    if (ti->tm_mon + 1 < 9) snprintf(mon, sizeof(mon), "0%d", ti->tm_mon + 1);
    else snprintf(mon, sizeof(mon), "%d", ti->tm_mon + 1);
    char buf[512];
    snprintf(buf, sizeof(buf), "%s_%d%s%d_%d-%d-%d_%s.txt", pure.c_str(), 1900 + ti->tm_year, mon, ti->tm_mday,
             ti->tm_hour, ti->tm_min, ti->tm_sec, type);
    return buf;
}

static std::string pure_name(const std::string &full) {
    size_t slash = full.find_last_of("/\\");
    std::string base = full.substr(slash == std::string::npos ? 0 : slash + 1);
    size_t dot = base.find_last_of('.');
    return dot == std::string::npos ? base : base.substr(0, dot);
}

// Largest singular value of a small square matrix C (k x k, row-major): sqrt of the largest
// eigenvalue of C^T C by cyclic Jacobi.  Used by the -fullSVD report (computeCosineError takes
// the first singular value of (Uhat^T U with |diagonal| - I), utilities.cpp:262-265).
static double largest_singular_value(const std::vector<double> &C, int k) {
    std::vector<double> A((size_t)k * k, 0.0);
    for (int i = 0; i < k; ++i)
        for (int j = 0; j < k; ++j) {
            double s = 0;
            for (int r = 0; r < k; ++r) s += C[(size_t)r * k + i] * C[(size_t)r * k + j];
            A[(size_t)i * k + j] = s;
        }
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0;
        for (int p = 0; p < k; ++p)
            for (int q = p + 1; q < k; ++q) off += A[(size_t)p * k + q] * A[(size_t)p * k + q];
        if (off < 1e-30) break;
        for (int p = 0; p < k; ++p)
            for (int q = p + 1; q < k; ++q) {
                const double apq = A[(size_t)p * k + q];
                if (apq == 0.0) continue;
                const double app = A[(size_t)p * k + p], aqq = A[(size_t)q * k + q];
                const double theta = (aqq - app) / (2 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1));
                const double c = 1 / std::sqrt(t * t + 1), sn = t * c;
                for (int r = 0; r < k; ++r) {
                    const double arp = A[(size_t)r * k + p], arq = A[(size_t)r * k + q];
                    A[(size_t)r * k + p] = c * arp - sn * arq;
                    A[(size_t)r * k + q] = sn * arp + c * arq;
                }
                for (int r = 0; r < k; ++r) {
                    const double apr = A[(size_t)p * k + r], aqr = A[(size_t)q * k + r];
                    A[(size_t)p * k + r] = c * apr - sn * aqr;
                    A[(size_t)q * k + r] = sn * apr + c * aqr;
                }
            }
    }
    double mx = 0;
    for (int i = 0; i < k; ++i) mx = std::max(mx, A[(size_t)i * k + i]);
    return std::sqrt(std::max(mx, 0.0));
}

static dpca_status run_common(const dpca_config *cfg_in, const char *bfile, const uint8_t *packed_host,
                              int64_t row_stride, int n_ind, int n_snp, double *omega_inout, dpca_result *res) {
    if (!cfg_in || !omega_inout || !res) {
        set_error("null argument");
        return DPCA_ERR_INVALID;
    }
    dpca_config cfg = *cfg_in;
    int rows = 0;
    DPCA_TRY(dpca_resolve_config(&cfg, n_ind, n_snp, &rows));
    cfg.bsize = rows;
    res->rows_fetched = rows;
    double t0 = wall_now();
    // Resident or streamed: the packed matrix (twice on the mixed path, which also keeps its
    // individual-major transpose) must fit the device budget -- -hbm GB, else 85% of the free
    // device memory -- or it is streamed from host memory in blocks of at most 2 GB, two in
    // flight.
    const int64_t np = (n_ind + 3) / 4;
    const size_t pitch = ((size_t)np + 127) / 128 * 128;
    const size_t per_row = pitch * (cfg.precision == DPCA_PREC_MIXED ? 2 : 1);
    size_t budget = 0;
    if (cfg.hbm_budget_gb > 0) {
        budget = (size_t)(cfg.hbm_budget_gb * 1e9);
    } else {
        size_t fr = 0, tot = 0;
        if (cudaSetDevice(cfg.device) == cudaSuccess && cudaMemGetInfo(&fr, &tot) == cudaSuccess)
            budget = (size_t)(0.85 * (double)fr);
        else
            cudaGetLastError();
    }
    int block_snps = 0;
    if (budget > 0 && per_row * (size_t)n_snp > budget) {
        size_t rows = std::min<size_t>((size_t)2000000000 / pitch, budget / (2 * per_row));
        block_snps = (int)std::max<size_t>(128, rows / 128 * 128);
    }
    dpca_handle *hh = nullptr;
    if (block_snps > 0 && block_snps < n_snp)
        DPCA_TRY(dpca_create_streamed(&hh, n_ind, n_snp, cfg.nrhs, cfg.precision, cfg.device, nullptr, block_snps));
    else
        DPCA_TRY(dpca_create(&hh, n_ind, n_snp, cfg.nrhs, cfg.precision, cfg.device, nullptr));
    dpca_status st = DPCA_OK;
    if (packed_host) {
        st = dpca_upload(hh, packed_host, row_stride);
    } else {
        // the .bed rows through the handle's block reader: read once for a resident matrix, every
        // pass for a streamed one -- never the whole file in host memory at once
        std::string bed = std::string(bfile) + ".bed";
        st = dpca_upload_file(hh, bed.c_str());
    }
    if (st == DPCA_OK) st = dpca_synchronize(hh);
    double t1 = wall_now();
    res->time_load_matrix = t1 - t0;
    if (st == DPCA_OK) st = dpca_solve(hh, &cfg, omega_inout, res);
    dpca_destroy(hh);
    res->time_total = wall_now() - t0 + res->time_generate_rhs;
    return st;
}

}  // namespace dpca

using namespace dpca;

extern "C" {

const char *dpca_status_string(dpca_status s) {
    switch (s) {
        case DPCA_OK: return "ok";
        case DPCA_ERR_INVALID: return "invalid argument";
        case DPCA_ERR_IO: return "I/O error";
        case DPCA_ERR_FORMAT: return "bad input format";
        case DPCA_ERR_CUDA: return "CUDA error";
        case DPCA_ERR_NOMEM: return "out of memory";
        case DPCA_ERR_UNSUPPORTED: return "unsupported shape";
        case DPCA_ERR_TIMEOUT: return "device wait timed out";
        case DPCA_ERR_NUMERIC: return "numerical failure";
    }
    return "unknown status";
}

const char *dpca_last_error(void) { return g_last_error.c_str(); }

const char *dpca_version(void) { return "dpca 0.1.0 (sm_103a)"; }

void dpca_config_init(dpca_config *c) {
    // initialize_structure, utilities.cpp:195-232 (the code's defaults, not the README's)
    memset(c, 0, sizeof(*c));
    c->nsv = 10;
    c->nrhs = 20;
    c->power = 1;
    c->crit = 1;
    c->miter = 100;
    c->bsize = 0;
    c->verbose = 1;
    c->fwrite = 0;
    c->full_svd = 0;
    c->tol = 1e-3;
    c->memory_gb = 0.0;
    snprintf(c->prefix, sizeof(c->prefix), "noprefix");
    c->precision = DPCA_PREC_MIXED;
    c->device = 0;
    c->hbm_budget_gb = 0.0;
}

// findarg (io.c:24-67): scan argv for "-name"; first match wins; a flag given as the last
// argument leaves the default in place; values go through atoi/atof.
static int findarg(const char *name, int type, void *val, int argc, char **argv, size_t cap = 1024) {
    for (int i = 0; i < argc; i++) {
        if (!argv[i] || argv[i][0] != '-') continue;
        if (strcmp(name, argv[i] + 1) != 0) continue;
        if (type == 3) return 1;
        if (i + 1 >= argc) return 0;
        if (type == 0) *(int *)val = atoi(argv[i + 1]);
        else if (type == 1) *(double *)val = atof(argv[i + 1]);
        else snprintf((char *)val, cap, "%s", argv[i + 1]);
        return 1;
    }
    return 0;
}

dpca_status dpca_parse_args(int argc, char **argv, dpca_config *cfg, char *bfile, size_t bfile_cap) {
    clear_error();
    if (!cfg) return DPCA_ERR_INVALID;
    char prefix[1024] = {0}, bf[1024] = {0};
    int have_prefix = findarg("prefix", 2, prefix, argc, argv);
    findarg("bfile", 2, bf, argc, argv);
    findarg("nrhs", 0, &cfg->nrhs, argc, argv);
    findarg("nsv", 0, &cfg->nsv, argc, argv);
    findarg("memory", 1, &cfg->memory_gb, argc, argv);
    findarg("bsize", 0, &cfg->bsize, argc, argv);
    findarg("verbose", 0, &cfg->verbose, argc, argv);
    findarg("fwrite", 0, &cfg->fwrite, argc, argv);
    findarg("tol", 1, &cfg->tol, argc, argv);
    findarg("miter", 0, &cfg->miter, argc, argv);
    findarg("crit", 0, &cfg->crit, argc, argv);
    findarg("power", 0, &cfg->power, argc, argv);
    findarg("fullSVD", 0, &cfg->full_svd, argc, argv);
    // device-side extensions
    char prec[64] = {0};
    if (findarg("precision", 2, prec, argc, argv, sizeof(prec))) {
        if (!strcmp(prec, "fp64")) cfg->precision = DPCA_PREC_FP64;
        else if (!strcmp(prec, "mixed")) cfg->precision = DPCA_PREC_MIXED;
        else {
            set_error("-precision must be fp64 or mixed");
            return DPCA_ERR_INVALID;
        }
    }
    findarg("device", 0, &cfg->device, argc, argv);
    findarg("hbm", 1, &cfg->hbm_budget_gb, argc, argv);
    if (have_prefix) snprintf(cfg->prefix, sizeof(cfg->prefix), "%s", prefix);
    if (bfile && bfile_cap) snprintf(bfile, bfile_cap, "%s", bf);
    return DPCA_OK;
}

dpca_status dpca_probe_bfile(const char *bfile, int *n_ind, int *n_snp) {
    clear_error();
    if (!bfile || !n_ind || !n_snp) return DPCA_ERR_INVALID;
    std::string b(bfile);
    std::string bed = b + ".bed";
    struct stat stb;
    if (stat(bed.c_str(), &stb) != 0) {
        set_error("[Data::read_bed] Error reading file %s", bed.c_str());
        return DPCA_ERR_IO;
    }
    int m = 0, n = 0;
    DPCA_TRY(read_lines(b + ".fam", 0, nullptr, &m));
    DPCA_TRY(read_lines(b + ".bim", 0, nullptr, &n));
    if (m <= 0 || n <= 0) {
        set_error("M and/or N were either zero or negative");
        return DPCA_ERR_FORMAT;
    }
    uint8_t magic[3] = {0, 0, 0};
    FILE *f = fopen(bed.c_str(), "rb");
    if (!f) {
        set_error("[Data::read_bed] Error reading file %s", bed.c_str());
        return DPCA_ERR_IO;
    }
    size_t got = fread(magic, 1, 3, f);
    fclose(f);
    if (got != 3 || magic[0] != 0x6C || magic[1] != 0x1B) {
        set_error("%s is not a PLINK .bed file (magic %02x %02x)", bed.c_str(), magic[0], magic[1]);
        return DPCA_ERR_FORMAT;
    }
    if (magic[2] != 0x01) {
        set_error("%s is individual-major (mode byte %02x); only SNP-major .bed is supported", bed.c_str(), magic[2]);
        return DPCA_ERR_FORMAT;
    }
    int64_t need = 3 + (int64_t)((m + 3) / 4) * n;
    if ((int64_t)stb.st_size < need) {
        set_error("%s holds %lld bytes; %d individuals x %d SNPs need %lld", bed.c_str(), (long long)stb.st_size, m,
                  n, (long long)need);
        return DPCA_ERR_FORMAT;
    }
    *n_ind = m;
    *n_snp = n;
    return DPCA_OK;
}

dpca_status dpca_resolve_config(dpca_config *c, int M, int N, int *rows_fetched) {
    clear_error();
    if (!c) return DPCA_ERR_INVALID;
    const int local_N = N;  // one process drives one device: a single SNP range
    int rows = c->bsize;
    if (rows <= 0) {
        // distpca.cpp:218-222, 239-269
        double mem = c->memory_gb;
        if (mem == 0.0) mem = ((double)ram_kb() / 1000000.0) / 10.0;
        const double B = 8.0, G = 1e9, SAFETY = 2048.0 * 100000.0;
        double membuff = (3.0 * local_N * B) + ((double)M * c->nsv * B) + (2.0 * local_N * c->nrhs) + (3.0 * M * B) +
                         SAFETY;
        double avail = mem * G - membuff;
        double blk = avail > 0.0 ? avail / (B * M) : (membuff + (double)M * B) / 1e7;
        rows = (int)blk;
        if (rows <= 0) rows = c->nsv;
        if (rows >= local_N) rows = local_N;
    } else if (rows > local_N) {
        if (c->verbose > 0)
            printf("\nWarning: Specified block size (%d) exceeds local SNPs (%d). Adjusting to local_N.\n", rows,
                   local_N);
        rows = local_N;
    }
    if (M <= 0 || N <= 0) {
        set_error("M and/or N were either zero or negative. Aborting...");
        return DPCA_ERR_INVALID;
    }
    if (c->nsv <= 0) {
        set_error("NSV was either zero or negative. Aborting...");
        return DPCA_ERR_INVALID;
    }
    int mn = std::min(M, N);
    if (c->nsv > mn) c->nsv = mn;
    if (c->nrhs <= 0) c->nrhs = std::min(2 * c->nsv, mn);
    if (c->nrhs > mn) c->nrhs = mn;
    if (c->nrhs < c->nsv) c->nrhs = std::min(2 * c->nsv, mn);
    if (c->nrhs > kMaxNrhs) {
        set_error("nrhs=%d exceeds the device limit of %d", c->nrhs, kMaxNrhs);
        return DPCA_ERR_UNSUPPORTED;
    }
    if (rows_fetched) *rows_fetched = rows;
    return DPCA_OK;
}

// rand_val / norm2 (gennorm.c:21-72) with PI = 3.14159265 (gennorm.h:23) and the reseeding
// loop of distpca.cpp:389-394: entry (j, c) calls rand_val(j*M + c) with 32-bit wraparound;
// positive seeds reset the Park-Miller state, others advance it.
dpca_status dpca_start_block(int n_ind, int k, double *out) {
    clear_error();
    if (n_ind <= 0 || k <= 0 || !out) return DPCA_ERR_INVALID;
    const long a = 16807, m = 2147483647, q = 127773, r = 2836;
    long x = 0;
    auto next = [&]() -> double {
        long hi = x / q, lo = x % q;
        long nx = a * lo - r * hi;
        x = nx > 0 ? nx : nx + m;
        return (double)x / m;
    };
    for (int j = 0; j < n_ind; ++j)
        for (int c = 0; c < k; ++c) {
            int seed = (int)((uint32_t)j * (uint32_t)n_ind + (uint32_t)c);
            if (seed > 0) x = seed;
            else next();
            double u = 0.0;
            while (u == 0.0) u = next();
            double rr = sqrt(-2.0 * log(u));
            double th = 0.0;
            while (th == 0.0) th = 2.0 * 3.14159265 * next();
            double v = rr * cos(th);
            out[(size_t)j * k + c] = v * 1.0 + 0.0;
        }
    return DPCA_OK;
}

dpca_status dpca_run(const dpca_config *cfg, const char *bfile, double *omega_inout, dpca_result *res) {
    clear_error();
    if (!bfile) return DPCA_ERR_INVALID;
    int m = 0, n = 0;
    DPCA_TRY(dpca_probe_bfile(bfile, &m, &n));
    return run_common(cfg, bfile, nullptr, 0, m, n, omega_inout, res);
}

dpca_status dpca_run_packed(const dpca_config *cfg, const uint8_t *packed, int64_t row_stride, int n_ind, int n_snp,
                            double *omega_inout, dpca_result *res) {
    clear_error();
    if (!packed) return DPCA_ERR_INVALID;
    return run_common(cfg, nullptr, packed, row_stride, n_ind, n_snp, omega_inout, res);
}

dpca_status dpca_write_outputs(const dpca_config *cfg, const char *bfile, const dpca_result *res) {
    clear_error();
    if (!cfg || !res || !res->sigma || !res->u) return DPCA_ERR_INVALID;
    std::vector<std::string> iids;
    int m = 0;
    if (bfile) DPCA_TRY(read_lines(std::string(bfile) + ".fam", 1, &iids, &m));
    iids.resize(res->n_ind);
    std::string prefix(cfg->prefix);
    std::string pure = pure_name(bfile ? bfile : "noprefix");
    std::string fv = prefix.empty() ? construct_filename(pure, "singularValues") : prefix + "_singularValues.txt";
    FILE *f = fopen(fv.c_str(), "w");
    if (!f) {
        set_error("fopen singularValues: %s", strerror(errno));
        return DPCA_ERR_IO;
    }
    for (int i = 0; i < res->nsv; ++i) fprintf(f, "%2.13lf\n", res->sigma[i]);
    fclose(f);
    std::string fu =
        prefix.empty() ? construct_filename(pure, "leftSingularVectors") : prefix + "_leftSingularVectors.txt";
    f = fopen(fu.c_str(), "w");
    if (!f) {
        set_error("fopen leftSingularVectors: %s", strerror(errno));
        return DPCA_ERR_IO;
    }
    fprintf(f, "FID");
    for (int j = 0; j < res->nsv; ++j) fprintf(f, "\tPC%d", j);
    fprintf(f, "\n");
    for (int i = 0; i < res->n_ind; ++i) {
        fprintf(f, "%8s", iids[i].c_str());
        for (int j = 0; j < res->nsv; ++j) fprintf(f, "\t%2.13f", res->u[(size_t)i * res->nsv + j]);
        fprintf(f, "\n");
    }
    fclose(f);
    return DPCA_OK;
}

dpca_status dpca_full_svd(const dpca_config *cfg, const char *bfile, const uint8_t *packed, int64_t row_stride,
                          int n_ind, int n_snp, const dpca_result *res, dpca_fullsvd *out) {
    clear_error();
    if (!cfg || !res || !out || !res->sigma || !res->u || !out->true_sigma || !out->sigma_relerr || !out->cosines ||
        n_ind <= 0 || n_snp <= 0 || (!packed && !bfile)) {
        set_error("dpca_full_svd: null argument or empty matrix");
        return DPCA_ERR_INVALID;
    }
    const int nsv = res->nsv;
    if (n_ind > 20000) {
        set_error("-fullSVD: the dense check supports up to 20000 individuals (got %d)", n_ind);
        return DPCA_ERR_UNSUPPORTED;
    }
    if (nsv < 1 || nsv > std::min(n_ind, n_snp)) {
        set_error("-fullSVD: nsv %d outside [1, min(n_ind, n_snp)]", nsv);
        return DPCA_ERR_INVALID;
    }
    dpca_handle *hh = nullptr;
    DPCA_TRY(dpca_create(&hh, n_ind, n_snp, 128, DPCA_PREC_FP64, cfg->device, nullptr));
    dpca_status st = packed ? dpca_upload(hh, packed, row_stride)
                            : dpca_upload_file(hh, (std::string(bfile) + ".bed").c_str());
    std::vector<double> tu((size_t)n_ind * nsv);
    const double t0 = wall_now();
    if (st == DPCA_OK) st = full_svd_device(&hh->h, nsv, out->true_sigma, tu.data(), &out->info);
    out->time_true_svd = wall_now() - t0;
    dpca_destroy(hh);
    DPCA_TRY(st);
    // comparisons as distpca.cpp:522-557 and computeCosineError (utilities.cpp:234-270)
    for (int i = 0; i < nsv; ++i) {
        const double denom = out->true_sigma[i] ? out->true_sigma[i] : 1.0;
        out->sigma_relerr[i] = std::fabs(out->true_sigma[i] - res->sigma[i]) / denom;
    }
    if (out->true_u) memcpy(out->true_u, tu.data(), tu.size() * sizeof(double));
    if (out->vec_relerr)
        for (size_t e = 0; e < tu.size(); ++e)
            out->vec_relerr[e] = std::fabs(std::fabs(tu[e]) - std::fabs(res->u[e])) / (std::fabs(tu[e]) + 1e-12);
    std::vector<double> C((size_t)nsv * nsv, 0.0);  // Uhat^T U
    for (int i = 0; i < n_ind; ++i)
        for (int a = 0; a < nsv; ++a) {
            const double ua = res->u[(size_t)i * nsv + a];
            for (int b = 0; b < nsv; ++b) C[(size_t)a * nsv + b] += ua * tu[(size_t)i * nsv + b];
        }
    double frob = 0;
    for (int a = 0; a < nsv; ++a)
        for (int b = 0; b < nsv; ++b) {
            const double v = C[(size_t)a * nsv + b];
            frob += a == b ? (std::fabs(v) - 1.0) * (std::fabs(v) - 1.0) : v * v;
        }
    out->frob_norm_angle = std::sqrt(frob);
    for (int a = 0; a < nsv; ++a) {
        out->cosines[a] = C[(size_t)a * nsv + a];
        C[(size_t)a * nsv + a] = std::fabs(C[(size_t)a * nsv + a]) - 1.0;
    }
    out->cos_error = largest_singular_value(C, nsv);
    if (cfg->verbose > 1) {
        printf("\nFULL SVD computed in %lf sec, info = %d\n\n", out->time_true_svd, out->info);
        for (int i = 0; i < nsv; ++i) printf("RelError Sigma(%d): %e\n", i, out->sigma_relerr[i]);
        for (int i = 0; i < nsv; ++i) printf("Cosine(%d): %lf\n", i, out->cosines[i]);
    }
    return DPCA_OK;
}

dpca_status dpca_write_fullsvd(const dpca_config *cfg, const char *bfile, int n_ind, int nsv,
                               const dpca_fullsvd *fs) {
    clear_error();
    if (!cfg || !fs || !fs->true_sigma || !fs->true_u || !fs->vec_relerr || !fs->cosines) {
        set_error("dpca_write_fullsvd: the check's vectors are needed (true_u, vec_relerr)");
        return DPCA_ERR_INVALID;
    }
    std::string prefix(cfg->prefix);
    std::string pure = pure_name(bfile ? bfile : "noprefix");
    auto name = [&](const char *type) {
        return prefix.empty() ? construct_filename(pure, type) : prefix + "_" + type + ".txt";
    };
    FILE *fvec = fopen(name("realLeftSingularVectors").c_str(), "w");
    FILE *fval = fopen(name("realSingularValues").c_str(), "w");
    FILE *ferr = fopen(name("singvecs_accuracy").c_str(), "w");
    FILE *fcos = fopen(name("cosineValues").c_str(), "w");
    if (!fvec || !fval || !ferr || !fcos) {
        for (FILE *f : {fvec, fval, ferr, fcos})
            if (f) fclose(f);
        set_error("File error");
        return DPCA_ERR_IO;
    }
    for (int i = 0; i < n_ind; ++i) {
        for (int j = 0; j < nsv; ++j) fprintf(fvec, "%2.13f ", fs->true_u[(size_t)i * nsv + j]);
        fprintf(fvec, "\n");
    }
    for (int i = 0; i < nsv; ++i) fprintf(fval, "%2.13f\n", fs->true_sigma[i]);
    for (size_t i = 0; i < (size_t)n_ind * nsv; ++i) fprintf(ferr, "%2.13lf\n", fs->vec_relerr[i]);
    for (int i = 0; i < nsv; ++i) fprintf(fcos, "%2.13lf\n", fs->cosines[i]);
    for (FILE *f : {fvec, fval, ferr, fcos}) fclose(f);
    return DPCA_OK;
}

// print_statistics (utilities.cpp:147-193), same lines and formats.
void dpca_print_statistics(const dpca_config *cfg, const dpca_result *r) {
    time_t raw;
    time(&raw);
    int threads = 1;
    if (getenv("OMP_NUM_THREADS")) threads = atoi(getenv("OMP_NUM_THREADS"));
    int kb = ram_kb();
    printf("----------------------------------------------------------\n");
    printf("DistPCA software package, Version: 1.0.0\n");
    printf("Current local time and date: %s", asctime(localtime(&raw)));
    printf("Total number of threads exploited: %d\n", threads);
    printf("RAM size in KBs: %d\n", kb);
    printf("RAM size in GBs: %lf\n", (double)kb / 1000000.0);
    printf("Total number of matrix rows: %d\n", r->n_ind);
    printf("Total number of matrix columns: %d\n", r->n_snp);
    printf("Total number of singular pairs sought: %d\n", r->nsv);
    printf("Total number of right-hand sides used: %d\n", r->nrhs);
    printf("Value of power: %d\n", cfg->power);
    printf("Total number of rows fetched from the disk per block: %d\n", r->rows_fetched);
    if (r->rows_fetched < r->n_snp) {
        int fetched = r->total_its * (cfg->power + 1);
        printf("Total number of times which the data matrix was fetched from the memory: %d\n", fetched);
        printf("Average amount of time elapsed per matrix fetching: %lf\n", r->time_load_matrix / fetched);
    }
    double total = r->time_projected_svd + r->time_generate_rhs + r->time_load_matrix + r->time_mm + r->time_gs +
                   r->time_other;
    double noload = total - r->time_load_matrix;
    const double hs[2] = {1.0, 3600.0};
    const char *unit[2] = {"seconds", "hours"};
    for (int u = 0; u < 2; ++u) {
        double d = hs[u];
        printf("\n[The following times are listed in %s]\n\n", unit[u]);
        printf("Time to generate the right-hand sides matrix: %02.13f\n", r->time_generate_rhs / d);
        printf("Time to load the data matrix: %02.13f\n", r->time_load_matrix / d);
        printf("Time to perform the MM products (overall): %02.13f\n", r->time_mm / d);
        printf("Time to perform the MM products (with A): %02.13f\n", r->time_mm_a / d);
        printf("Time to perform the MM products (with A^T): %02.13f\n", r->time_mm_a_t / d);
        printf("Time to perform the orthonormalization: %02.13f\n", r->time_gs / d);
        printf("Time to solve the projection eigenvalue problem: %02.13f\n", r->time_projected_svd / d);
        printf("\nTotal wall-clock time elapsed: %02.13f\n", total / d);
        if (u == 0)
            printf("Total wall-clock time elapsed (without including the amount of time spent on loading the "
                   "matrix): %02.13f\n",
                   noload / d);
        else
            printf("Total wall-clock time elapsed (without including the time spent on loading the matrix): "
                   "%02.13f\n",
                   noload / d);
    }
    // utilities.cpp:187-191: printed for in-core runs with -fullSVD; the reference prints these
    // before the check runs, so they read zero unless a caller filled them in first
    if (cfg && cfg->full_svd == 1 && r->rows_fetched == r->n_snp) {
        printf("\nTotal wall-clock time to compute the full ('econ') SVD: %02.13f\n", r->time_true_svd);
        printf("||Uhat^TU - I||_F: %02.13f\n", r->frob_norm_angle);
        printf("||Uhat^TU - I||_2: %02.13f\n", r->cos_error);
    }
}

}  // extern "C"
