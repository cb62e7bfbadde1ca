// Mixed-precision pass (tcgen05).  Placeholder until the tensor-core kernels land.
#include "dpca_internal.h"

namespace dpca {

dpca_status mixed_prepare(Handle *) { return DPCA_OK; }
dpca_status mixed_release(Handle *) { return DPCA_OK; }
dpca_status launch_mixed_xw(Handle *, const double *, double *) {
    set_error("mixed precision pass not built yet");
    return DPCA_ERR_UNSUPPORTED;
}
dpca_status launch_mixed_xty(Handle *, double *) {
    set_error("mixed precision pass not built yet");
    return DPCA_ERR_UNSUPPORTED;
}

}  // namespace dpca
