/*
 * Golden-vector harness around the reference's own, unmodified decode,
 * standardize and RNG routines (test infrastructure only; built by
 * oracle/build_ref.sh into oracle/_ref/ref_harness).
 *
 *   ref_harness stats <bfile> <n_ind> <n_snp> <out.bin>
 *       For every SNP row of <bfile>.bed: decode_plink_sse2
 *       (utilities.cpp:351) then standardize (utilities.cpp:272).  Writes,
 *       per SNP, avg and sd (2 doubles), then the n_ind standardized doubles,
 *       then the n_ind decoded codes (bytes).
 *   ref_harness omega <n_ind> <k> <out.bin>
 *       The start block exactly as distpca.cpp:389-394 builds it
 *       (rand_val(jj*M+kk) then norm2(0,1), gennorm.c:21-72): n_ind*k doubles.
 */
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <vector>

#include "gennorm.h"
#include "utilities.h"

static int do_stats(const char *bfile, int n_ind, int n_snp, const char *out) {
    std::string bed = std::string(bfile) + ".bed";
    FILE *f = fopen(bed.c_str(), "rb");
    if (!f) { perror("bed"); return 1; }
    FILE *o = fopen(out, "wb");
    if (!o) { perror("out"); return 1; }
    unsigned np = (unsigned)((n_ind + 3) / 4);
    std::vector<unsigned char> row(np), dec((size_t)np * 4);
    std::vector<double> norm(n_ind);
    double inv_sqrtN = 1.0 / sqrt((double)n_snp);
    fseek(f, 3, SEEK_SET);
    for (int s = 0; s < n_snp; ++s) {
        if (fread(row.data(), 1, np, f) != np) { fprintf(stderr, "short read\n"); return 1; }
        decode_plink_sse2(dec.data(), row.data(), np);
        double avg = 0, sd = 0;
        standardize(norm.data(), dec.data(), n_ind, avg, sd, inv_sqrtN);
        fwrite(&avg, 8, 1, o);
        fwrite(&sd, 8, 1, o);
        fwrite(norm.data(), 8, (size_t)n_ind, o);
        fwrite(dec.data(), 1, (size_t)n_ind, o);
    }
    fclose(f);
    fclose(o);
    return 0;
}

static int do_omega(int M, int NRHS, const char *out) {
    std::vector<double> rhs((size_t)M * NRHS);
    for (int jj = 0; jj < M; jj++)
        for (int kk = 0; kk < NRHS; kk++) {
            rand_val(jj * M + kk);
            rhs[(size_t)jj * NRHS + kk] = (double)norm2(0.0, 1.0);
        }
    FILE *o = fopen(out, "wb");
    if (!o) { perror("out"); return 1; }
    fwrite(rhs.data(), 8, rhs.size(), o);
    fclose(o);
    return 0;
}

int main(int argc, char **argv) {
    if (argc == 6 && !strcmp(argv[1], "stats")) return do_stats(argv[2], atoi(argv[3]), atoi(argv[4]), argv[5]);
    if (argc == 5 && !strcmp(argv[1], "omega")) return do_omega(atoi(argv[2]), atoi(argv[3]), argv[4]);
    fprintf(stderr, "usage: ref_harness stats <bfile> <n_ind> <n_snp> <out> | omega <n_ind> <k> <out>\n");
    return 2;
}
