// persist_f64_spec.cu -- the FP64, single-species Tersoff (parameters as arguments) instantiations of the persistent
// batch kernel (persist.cuh), in a translation unit of their own so that the
// four variants compile in parallel.
#include "persist.cuh"

namespace pg {

int launch_persistent_f64_spec(const PersistArgs& P, int pg_lanes, int bg_lanes, int sms, cudaStream_t st) {
    return launch_persistent_impl<double, true>(P, pg_lanes, bg_lanes, sms, st);
}

}  // namespace pg
