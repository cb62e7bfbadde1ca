/* openblas_set_num_threads for the aarch64 branch of the reference oracle build
 * (distpca.cpp declares it extern "C"); forwards to scipy's prefixed export.
 * Test infrastructure only. */
void scipy_openblas_set_num_threads(int);
void openblas_set_num_threads(int n) { scipy_openblas_set_num_threads(n); }
