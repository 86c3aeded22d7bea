// persist_f32_table.cu -- the FP32 (mixed-precision), table-driven Tersoff instantiations of the persistent
// batch kernel (persist.cuh), in a translation unit of their own so that the
// four variants compile in parallel.
#include "persist.cuh"

namespace pg {

int launch_persistent_f32_table(const PersistArgs& P, int pg_lanes, int bg_lanes, int sms, cudaStream_t st) {
    return launch_persistent_impl<float, false>(P, pg_lanes, bg_lanes, sms, st);
}

}  // namespace pg
