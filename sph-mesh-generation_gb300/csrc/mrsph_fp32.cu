// mrsph_fp32.cu — FP32-split engine instantiation: positions are an integer
// anchor cell plus an FP32 offset, pair arithmetic and accumulation in FP32,
// the dt / max|v| grid reductions exact in FP64.
#include "engine.cuh"

namespace mrsph {
EngineBase* make_engine_fp32(const EngineConfig& cfg) {
  if (cfg.prm.dim == 2) return new Engine<2, float>(cfg);
  return new Engine<3, float>(cfg);
}
}  // namespace mrsph
