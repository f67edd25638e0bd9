// Fast multipole evaluation of the demagnetising potential (built in a later step).
#include "fg_internal.h"

namespace fg {
int fmm_build(Ctx &c) {
    c.err = "FMM demag is not built in this library version";
    return FG_EINVAL;
}
void fmm_free(Ctx &) {}
cudaError_t fmm_eval(Ctx &) { return cudaErrorNotSupported; }
cudaError_t launch_mixed(Ctx &, double, double) { return cudaErrorNotSupported; }
}  // namespace fg
