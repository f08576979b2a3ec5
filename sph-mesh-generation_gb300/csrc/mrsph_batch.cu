// mrsph_batch.cu — batched relaxation of independent geometries.
//
// The reference relaxes one geometry per run (SPH_mesh_generation::
// SPH_run_mesh_generation, sph_mesh_generation.cpp:1371-1463); relaxing many
// means one run after another.  Here every handle keeps the CUDA graph of its
// own step (12 kernels) and a batch step launches each handle's graph on the
// handle's own stream, back to back from one host thread: the geometries run
// concurrently on the GPU, so small ones fill it together, and each handle's
// results are those of stepping it alone (the same graph on the same
// stream).  A single parent graph with one child node per handle was the
// first design; its host launch cost grew faster than the node count (about
// 60 ms per launch for 512 handles, three times the GPU time of the step).
//
// Ordering: everything runs on the handles' own streams, so work queued on a
// handle before a batch call runs first and work queued afterwards runs
// after the batch's steps.  Every 32 steps the batch waits for each handle's
// stream and makes its neighbour-list capacity check (which may rebuild the
// handle's graphs).
#include <cuda_runtime.h>

#include <cstring>
#include <string>
#include <vector>

#include "handle.h"

struct mrsph_batch {
  std::vector<mrsph_handle*> hs;
  std::vector<cudaEvent_t> ev;  // per handle: end of its part of a timed region
  cudaStream_t stream = nullptr;  // timing stream
  int countdown = 32;             // steps until the next capacity check
  int device = 0;
  std::string err;
};

namespace {

int bfail(mrsph_batch* b, int code, const std::string& msg) {
  b->err = msg;
  return code;
}

// wait for every handle's stream, then run the capacity checks
int check_caps(mrsph_batch* b) {
  for (size_t k = 0; k < b->hs.size(); k++) {
    mrsph::EngineBase* e = b->hs[k]->eng;
    if (cudaStreamSynchronize(b->hs[k]->stream) != cudaSuccess)
      return bfail(b, MRSPH_ERR_CUDA, "handle " + std::to_string(k) + ": step failed");
    int rc = e->check_capacity();
    if (rc) return bfail(b, rc, "handle " + std::to_string(k) + ": " + e->err);
  }
  return 0;
}

int run_steps(mrsph_batch* b, int nsteps, bool checks) {
  for (int s = 0; s < nsteps; s++) {
    for (size_t k = 0; k < b->hs.size(); k++) {
      mrsph::EngineBase* e = b->hs[k]->eng;
      int rc = e->step_batched();
      if (rc) return bfail(b, rc, "handle " + std::to_string(k) + ": " + e->err);
    }
    if (checks && --b->countdown <= 0) {
      b->countdown = 32;
      int rc = check_caps(b);
      if (rc) return rc;
    }
  }
  return 0;
}

}  // namespace

extern "C" int mrsph_batch_create(mrsph_handle* const* handles, int count, mrsph_batch** out) {
  if (!out || !handles || count < 1) return MRSPH_ERR_ARG;
  *out = nullptr;
  mrsph_batch* b = new mrsph_batch();
  b->device = handles[0] ? handles[0]->prm.device : 0;
  for (int k = 0; k < count; k++) {
    mrsph_handle* h = handles[k];
    if (!h || !h->eng || h->eng->num_particles() <= 0) {
      delete b;
      return MRSPH_ERR_STATE;
    }
    if (h->prm.device != b->device) {
      delete b;
      return MRSPH_ERR_ARG;
    }
    for (int q = 0; q < k; q++)
      if (handles[q] == h) {
        delete b;
        return MRSPH_ERR_ARG;
      }
    b->hs.push_back(h);
  }
  if (cudaSetDevice(b->device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete b;
    return MRSPH_ERR_CUDA;
  }
  b->ev.assign(count, nullptr);
  for (int k = 0; k < count; k++)
    if (cudaEventCreateWithFlags(&b->ev[k], cudaEventDisableTiming) != cudaSuccess) {
      for (int q = 0; q < k; q++) cudaEventDestroy(b->ev[q]);
      cudaStreamDestroy(b->stream);
      delete b;
      return MRSPH_ERR_CUDA;
    }
  *out = b;
  return 0;
}

extern "C" int mrsph_batch_destroy(mrsph_batch* b) {
  if (!b) return 0;
  cudaSetDevice(b->device);
  for (auto* h : b->hs) cudaStreamSynchronize(h->stream);
  for (auto e : b->ev) cudaEventDestroy(e);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return 0;
}

extern "C" int mrsph_batch_last_error(mrsph_batch* b, char* buf, size_t len) {
  if (!b || !buf || len == 0) return MRSPH_ERR_ARG;
  std::strncpy(buf, b->err.c_str(), len - 1);
  buf[len - 1] = 0;
  return 0;
}

extern "C" int mrsph_batch_step(mrsph_batch* b, int nsteps) {
  if (!b) return MRSPH_ERR_ARG;
  if (nsteps <= 0) return 0;
  if (cudaSetDevice(b->device) != cudaSuccess) return bfail(b, MRSPH_ERR_CUDA, "cudaSetDevice failed");
  return run_steps(b, nsteps, true);
}

extern "C" int mrsph_batch_step_timed(mrsph_batch* b, int nsteps, double* ms) {
  if (!b || !ms) return MRSPH_ERR_ARG;
  if (cudaSetDevice(b->device) != cudaSuccess) return bfail(b, MRSPH_ERR_CUDA, "cudaSetDevice failed");
  // settle capacities and build every graph outside the timed region
  int rc = check_caps(b);
  for (size_t k = 0; !rc && k < b->hs.size(); k++) {
    rc = b->hs[k]->eng->prepare_steps();
    if (rc) rc = bfail(b, rc, "handle " + std::to_string(k) + ": " + b->hs[k]->eng->err);
  }
  if (rc) return rc;
  cudaEvent_t t0, t1;
  if (cudaEventCreate(&t0) != cudaSuccess) return bfail(b, MRSPH_ERR_CUDA, "cudaEventCreate failed");
  if (cudaEventCreate(&t1) != cudaSuccess) {
    cudaEventDestroy(t0);
    return bfail(b, MRSPH_ERR_CUDA, "cudaEventCreate failed");
  }
  // t0 on the timing stream; every handle's steps start after it and the
  // timing stream records t1 after every handle's last step
  if (cudaEventRecord(t0, b->stream) != cudaSuccess) rc = bfail(b, MRSPH_ERR_CUDA, "event record failed");
  for (auto* h : b->hs)
    if (!rc && cudaStreamWaitEvent(h->stream, t0, 0) != cudaSuccess)
      rc = bfail(b, MRSPH_ERR_CUDA, "event ordering failed");
  if (!rc) rc = run_steps(b, nsteps, false);
  for (size_t k = 0; !rc && k < b->hs.size(); k++)
    if (cudaEventRecord(b->ev[k], b->hs[k]->stream) != cudaSuccess ||
        cudaStreamWaitEvent(b->stream, b->ev[k], 0) != cudaSuccess)
      rc = bfail(b, MRSPH_ERR_CUDA, "event ordering failed");
  if (!rc && cudaEventRecord(t1, b->stream) != cudaSuccess) rc = bfail(b, MRSPH_ERR_CUDA, "event record failed");
  if (!rc) {
    if (cudaEventSynchronize(t1) != cudaSuccess) rc = bfail(b, MRSPH_ERR_CUDA, "batch step failed");
    float f = 0.f;
    if (!rc && cudaEventElapsedTime(&f, t0, t1) == cudaSuccess) *ms = f;
  }
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  return rc;
}

extern "C" int mrsph_batch_sync(mrsph_batch* b) {
  if (!b) return MRSPH_ERR_ARG;
  if (cudaSetDevice(b->device) != cudaSuccess) return bfail(b, MRSPH_ERR_CUDA, "cudaSetDevice failed");
  for (auto* h : b->hs)
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) return bfail(b, MRSPH_ERR_CUDA, "handle stream failed");
  return 0;
}
