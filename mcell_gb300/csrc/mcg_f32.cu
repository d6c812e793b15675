// fp32 instantiation of the engine (positions and ray geometry in fp32,
// reaction probabilities and times in fp64).
#include "mcg_engine.cuh"

namespace mcg {
DeviceEngine* make_engine_f32() { return new DeviceEngineT<float>(); }
}  // namespace mcg
