// engine_inst.cu - one engine template instance per object file. The build
// compiles this file once for every (dimension, form, smoothing kernel) with
// TG_INST_DIM, TG_INST_FORM and TG_INST_KERNEL defined, so the instances
// compile in parallel.
#include "engine_impl.cuh"

#if !defined(TG_INST_DIM) || !defined(TG_INST_FORM) || !defined(TG_INST_KERNEL)
#error "engine_inst.cu needs TG_INST_DIM, TG_INST_FORM and TG_INST_KERNEL"
#endif

namespace tg {

template std::unique_ptr<EngineBase>
make_engine_instance<TG_INST_DIM, TG_INST_FORM, TG_INST_KERNEL>();

}  // namespace tg
