// engine_2d_f32.cu - instantiation of the 2D FP32-compensated engines for every
// smoothing kernel (one translation unit per dimension and form, so the
// build compiles them in parallel).
#include "engine_impl.cuh"

namespace tg {

std::unique_ptr<EngineBase> make_engine_2d_f32(int kernel) {
  return make_engine<2, TG_FP32C>(kernel);
}

}  // namespace tg
