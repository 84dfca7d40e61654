// FP32 pair math with FP64 positions (the production build).
#include "tsph_engine.cuh"

namespace tsph {
EngineBase *make_engine_f32() { return new Engine<float>(); }
}  // namespace tsph
