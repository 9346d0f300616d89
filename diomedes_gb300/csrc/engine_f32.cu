// engine_f32.cu -- instantiates the engine for <P, R> = <float,float>.
#include "engine_impl.cuh"

namespace dio {
EngineBase* make_engine_f32(const DioCapacity& cap, cudaStream_t s, const DioConfig& cfg) {
    return make_engine_t<float,float>(cap, s, cfg);
}
}  // namespace dio
