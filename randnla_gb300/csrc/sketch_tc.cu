// Tensor-core (tcgen05) digit-sliced products.  Placeholder until the
// sm_103a kernel lands: every entry point reports RNLA_ERR_UNSUPPORTED.
#include "rnla_internal.h"

namespace rnla {

bool tc_available(Ctx&) { return false; }

void tc_sketch_apply(Ctx&, const RngKey&, const void*, bool, int64_t, int64_t, int64_t, int64_t, int,
                     double*, int64_t) {
    fail(RNLA_ERR_UNSUPPORTED, "tensor-core sketch not built");
}

void tc_gemm_tn(Ctx&, const double*, int64_t, int64_t, int64_t, const double*, int64_t, int64_t, int,
                int, double*, int64_t) {
    fail(RNLA_ERR_UNSUPPORTED, "tensor-core GEMM not built");
}

}  // namespace rnla
