// FP64 instantiation of the engine.
#include "ffs_engine.cuh"
namespace ffsgpu {
EngineBase* make_engine_f64() { return new Engine<double>(); }
}  // namespace ffsgpu
