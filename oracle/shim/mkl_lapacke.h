/* LAPACKE names for the reference oracle build (test infrastructure only). */
#include "dpca_blas_shim.h"
