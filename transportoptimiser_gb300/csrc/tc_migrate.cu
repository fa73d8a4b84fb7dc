// tc_migrate.cu - tensor-core (tcgen05, kind::tf32, 3xTF32) migration step.
#include "to_internal.cuh"
#include "to_pop.cuh"

namespace to_k {
to_status mte_tc(to_ctx ctx, to_mte_args a, int n_rs) {
    (void)a; (void)n_rs;
    return to_set_error(ctx, TO_ERR_UNSUPPORTED, "tensor-core migration not built");
}
}  // namespace to_k
