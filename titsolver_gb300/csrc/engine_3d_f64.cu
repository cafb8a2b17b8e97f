// engine_3d_f64.cu - instantiation of the 3D FP64 engines for every
// smoothing kernel (one translation unit per dimension and form, so the
// build compiles them in parallel).
#include "engine_impl.cuh"

namespace tg {

std::unique_ptr<EngineBase> make_engine_3d_f64(int kernel) {
  return make_engine<3, TG_FP64>(kernel);
}

}  // namespace tg
