// FP32 instantiation of the engine.
#include "ffs_engine.cuh"
namespace ffsgpu {
EngineBase* make_engine_f32() { return new Engine<float>(); }
int64_t estimate_bytes_f32(const ffs_params& p) { return Engine<float>::estimate_bytes(p); }
}  // namespace ffsgpu
