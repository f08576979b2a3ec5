// handle.h — the opaque mrsph_handle of the C ABI (internal).
#pragma once
#include <string>
#include <vector>

#include "engine_iface.h"

struct mrsph_batch;

struct mrsph_handle {
  mrsph_params prm{};
  std::string err;
  cudaStream_t stream = nullptr;
  mrsph::CellGeo geo{};
  mrsph::LsSet ls{};
  int nls = 0;
  long long ls_ntot[mrsph::MAX_LS] = {0, 0, 0, 0};
  std::vector<void*> ls_allocs;
  mrsph::EngineBase* eng = nullptr;
  // the geometry's singularity points and segments (mrsph_set_characteristics)
  std::vector<double> sing, seg;
  // the batches that hold this handle (mrsph_batch_create); mrsph_destroy
  // detaches the handle from them first
  std::vector<mrsph_batch*> batches;
};

// Waits for the batch's queued work and takes handle h out of it; the batch
// then refuses to step (mrsph_batch.cu).
void mrsph_batch_detach(mrsph_batch* b, mrsph_handle* h);
