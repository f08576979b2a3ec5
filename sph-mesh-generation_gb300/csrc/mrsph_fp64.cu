// mrsph_fp64.cu — FP64-plain engine instantiation.  Compiled with
// -fmad=false so every multiply and add rounds separately, as in the
// reference's FP64 arithmetic (Makefile.in:29, glbcls.h:138-144).
#include "engine.cuh"

namespace mrsph {
EngineBase* make_engine_fp64(const EngineConfig& cfg) {
  if (cfg.prm.dim == 2) return new Engine<2, double>(cfg);
  return new Engine<3, double>(cfg);
}
}  // namespace mrsph
