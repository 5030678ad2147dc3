// FP32 instantiation of the engine.
#include "ffs_engine.cuh"
namespace ffsgpu {
EngineBase* make_engine_f32() { return new Engine<float>(); }
}  // namespace ffsgpu
