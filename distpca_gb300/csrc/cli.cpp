// dpca: command line compatible with DistPCA.exe (distpca.cpp:47-644).
//
//   dpca -bfile P [-nsv 10] [-nrhs 20] [-power 1] [-crit 1] [-tol 1e-3] [-bsize B] [-miter 100]
//        [-verbose 1] [-fwrite 0] [-prefix noprefix] [-memory GB] [-fullSVD 0]
//        [-precision mixed|fp64] [-device 0]
//
// Prints the reference's progress and statistics lines and writes the same -fwrite files.
// Exit status is 0 on success and 1 on any error (the message is printed, as the reference
// does before exiting).
#include <cmath>
#include <cstdio>
#include <fstream>
#include <sstream>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <algorithm>
#include <vector>

#include "dpca.h"

static std::string stamp() {
    time_t t = time(nullptr);
    char *s = asctime(localtime(&t));
    std::string str(s);
    if (!str.empty() && str.back() == '\n') str.pop_back();
    return "[" + str + "] ";
}

// IIDs (.fam column 2) of the newline-terminated lines, as GetFamInfo collects them.
static std::vector<std::string> read_iids(const std::string &fam) {
    std::vector<std::string> ids;
    std::ifstream in(fam.c_str());
    while (in) {
        std::string line;
        std::getline(in, line);
        if (in.eof()) break;
        std::stringstream ss(line);
        std::string a, b;
        ss >> a >> b;
        ids.push_back(b);
    }
    return ids;
}

static int fail(dpca_status st) {
    printf("\n%s (%s)\n", dpca_last_error(), dpca_status_string(st));
    return 1;
}

int main(int argc, char **argv) {
    for (int i = 1; i < argc; ++i)
        if (!strcmp(argv[i], "-about") || !strcmp(argv[i], "-help")) {
            printf("\nDistPCA\nDistributed Out-of-Core Principal Component Analysis (PCA) for Tera-Scale Genomic "
                   "Data\n\n%s\n",
                   dpca_version());
            return 0;
        }
    dpca_config cfg;
    dpca_config_init(&cfg);
    char bfile[1024];
    dpca_status st = dpca_parse_args(argc, argv, &cfg, bfile, sizeof(bfile));
    if (st != DPCA_OK) return fail(st);
    int M = 0, N = 0;
    printf("%sReading .fam file: %s.fam\n", stamp().c_str(), bfile);
    st = dpca_probe_bfile(bfile, &M, &N);
    if (st != DPCA_OK) return fail(st);
    printf("\n%sNumber of individuals (M): %d\n", stamp().c_str(), M);
    printf("\n%sReading .bim file: %s.bim\n", stamp().c_str(), bfile);
    printf("\n%sNumber of markers (N): %d\n", stamp().c_str(), N);
    printf("\n%sNumber of devices: 1 (GB300, one process per GPU)\n", stamp().c_str());
    int rows = 0;
    st = dpca_resolve_config(&cfg, M, N, &rows);
    if (st != DPCA_OK) return fail(st);
    printf("\n%sBlock size (SNPs per block): %d\n", stamp().c_str(), rows);
    cfg.bsize = rows;
    std::vector<double> omega((size_t)M * cfg.nrhs), sigma(cfg.nsv), u((size_t)M * cfg.nsv);
    std::vector<double> delta(cfg.miter > 0 ? cfg.miter : 1);
    dpca_result res;
    memset(&res, 0, sizeof(res));
    res.sigma = sigma.data();
    res.u = u.data();
    res.delta_iter = delta.data();
    struct timespec a, b;
    clock_gettime(CLOCK_MONOTONIC, &a);
    st = dpca_start_block(M, cfg.nrhs, omega.data());
    clock_gettime(CLOCK_MONOTONIC, &b);
    if (st != DPCA_OK) return fail(st);
    res.time_generate_rhs = (b.tv_sec - a.tv_sec) + 1e-9 * (b.tv_nsec - a.tv_nsec);
    st = dpca_run(&cfg, bfile, omega.data(), &res);
    if (st != DPCA_OK) return fail(st);
    if (cfg.fwrite == 1) {
        st = dpca_write_outputs(&cfg, bfile, &res);
        if (st != DPCA_OK) return fail(st);
    }
    if (cfg.verbose > 1) {
        // distpca.cpp:409-439
        printf("\nApproximate eigenvalues:\n");
        for (int j = 0; j < res.nsv; ++j) printf("λ_%d = %.13f\n", j, sigma[j] * sigma[j]);
        printf("\nFirst 5 individuals' eigenvectors:\n\n");
        printf("%-20s", "FID");
        for (int j = 0; j < res.nsv; ++j) printf("%-15s", ("PC" + std::to_string(j)).c_str());
        printf("\n%s\n", std::string(20 + 15 * res.nsv, '-').c_str());
        std::vector<std::string> iids = read_iids(std::string(bfile) + ".fam");
        for (int i = 0; i < std::min(5, M); ++i) {
            printf("%-20s", i < (int)iids.size() ? iids[i].c_str() : "");
            for (int j = 0; j < res.nsv; ++j) printf("%-15.6f", u[(size_t)i * res.nsv + j]);
            printf("\n");
        }
    }
    if (cfg.verbose > 0) dpca_print_statistics(&cfg, &res);
    if (cfg.full_svd == 1) {
        // distpca.cpp:449-635: after the statistics block, the dense check and its files
        std::vector<double> ts(res.nsv), tu((size_t)M * res.nsv), se(res.nsv), ve((size_t)M * res.nsv), cs(res.nsv);
        dpca_fullsvd fs;
        memset(&fs, 0, sizeof(fs));
        fs.true_sigma = ts.data();
        fs.true_u = tu.data();
        fs.sigma_relerr = se.data();
        fs.vec_relerr = ve.data();
        fs.cosines = cs.data();
        st = dpca_full_svd(&cfg, bfile, nullptr, 0, M, N, &res, &fs);
        if (st != DPCA_OK) return fail(st);
        if (cfg.fwrite == 1) {
            st = dpca_write_fullsvd(&cfg, bfile, M, res.nsv, &fs);
            if (st != DPCA_OK) return fail(st);
        }
    }
    return 0;
}
