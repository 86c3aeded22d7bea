// relax.cu -- device-resident damped charge dynamics (placeholder).
#include "common.cuh"

namespace pg {

void relax_charges(pg_context* ctx, int precision, int n_steps, double dt, double inertia, double friction,
                   double tolerance, double* rates, double* charges, int* steps, double* error, double* max_dq) {
    (void)ctx; (void)precision; (void)n_steps; (void)dt; (void)inertia; (void)friction; (void)tolerance;
    (void)rates; (void)charges; (void)steps; (void)error; (void)max_dq;
    require(false, PG_ERR_UNSUPPORTED, "charge relaxation is not available in this build");
}

}  // namespace pg
