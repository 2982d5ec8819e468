// split_stub.cu -- placeholder until the tensor-core split-precision path is built:
// requesting AEROS_PREC_SPLIT reports AEROS_ERR_UNSUPPORTED (no silent fallback).
#include "split.h"

namespace aeros {

struct SplitCtx {};

int split_create(const Geometry &, const DevTables &, int, SplitCtx **out) {
    *out = nullptr;
    set_error("split-precision Legendre path not built");
    return AEROS_ERR_UNSUPPORTED;
}
void split_destroy(SplitCtx *) {}
int split_leg_synth(SplitCtx *, const Ctx &, const SynPlan &, double2 *, int) { return AEROS_ERR_UNSUPPORTED; }
int split_leg_anal(SplitCtx *, const Ctx &, const AnaCol *, int, const double2 *, int) {
    return AEROS_ERR_UNSUPPORTED;
}

}  // namespace aeros
