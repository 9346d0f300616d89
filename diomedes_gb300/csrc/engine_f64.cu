// engine_f64.cu -- instantiates the engine for <P, R> = <double,double>.
#include "engine_impl.cuh"

namespace dio {
EngineBase* make_engine_f64(const DioCapacity& cap, cudaStream_t s, const DioConfig& cfg) {
    return make_engine_t<double,double>(cap, s, cfg);
}
}  // namespace dio
