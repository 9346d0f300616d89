// engine_split.cu -- instantiates the engine for <P, R> = <double,float>.
#include "engine_impl.cuh"

namespace dio {
EngineBase* make_engine_split(const DioCapacity& cap, cudaStream_t s, const DioConfig& cfg) {
    return make_engine_t<double,float>(cap, s, cfg);
}
}  // namespace dio
