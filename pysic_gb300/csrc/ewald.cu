// ewald.cu -- reciprocal-space Ewald sum (placeholder until the k-space kernels land).
#include "common.cuh"

namespace pg {

void ewald_prepare(pg_context* ctx) {
    require(false, PG_ERR_UNSUPPORTED, "k-space Ewald is not available in this build");
    (void)ctx;
}

int ewald_partial_slots(pg_context* ctx) {
    (void)ctx;
    return 0;
}

void launch_ewald_kspace(pg_context* ctx, int precision, int flags, bool first_f, bool first_chi, double* partial) {
    (void)ctx; (void)precision; (void)flags; (void)first_f; (void)first_chi; (void)partial;
}

}  // namespace pg
