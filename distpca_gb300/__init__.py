"""distpca_gb300: GB300-native randomized subspace-iteration PCA on PLINK .bed genotypes.

The product is libdpca.so (C++ host code + sm_103a CUDA kernels behind the C ABI in
include/dpca.h) and the dpca command line, flag-compatible with DistPCA.exe.  This
package holds the sources (csrc/), the build recipe (build.py), a ctypes mirror of the
solver interface (api.py) and the seeded cohort generator (synth.py).
"""
from .api import *  # noqa: F401,F403
