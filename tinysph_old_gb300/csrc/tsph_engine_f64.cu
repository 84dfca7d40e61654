// FP64 throughout, compiled with -fmad=false: the error-study build whose
// arithmetic rounds like the reference's C++ (no fused multiply-add).
#include "tsph_engine.cuh"

namespace tsph {
EngineBase *make_engine_f64() { return new Engine<double>(); }
}  // namespace tsph
