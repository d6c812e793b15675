// fp64 instantiation of the engine. Built with -fmad=false so that every
// product and sum is rounded like MCell4's CPU build (no fused multiply-add).
#include "mcg_engine.cuh"

namespace mcg {
DeviceEngine* make_engine_f64() { return new DeviceEngineT<double>(); }
// the countdown is shared by every engine of the process (one inline definition)
void set_alloc_failure(long long after) { alloc_failure_countdown().store(after < 0 ? -1 : after); }
}  // namespace mcg
