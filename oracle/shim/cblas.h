/* CBLAS names for the reference oracle build on aarch64 (test infrastructure only). */
#include "dpca_blas_shim.h"
