// mrsph_batch.cu — batched relaxation of independent geometries.
//
// The reference relaxes one geometry per run (SPH_mesh_generation::
// SPH_run_mesh_generation, sph_mesh_generation.cpp:1371-1463); relaxing many
// means one run after another.  Three ways to step a batch here:
//
// * persistent (default when every handle is FP32-split): one cooperative
//   launch of the persistent batch kernel (mrsph_persist.cu) runs up to 32
//   whole steps of every geometry, replayed from a CUDA graph per step count
//   where the capture of a cooperative launch is available.
// * phases: the same work lists, one launch per phase (12 per step).
// * streams: every handle keeps the CUDA graph of its own step and a batch
//   step launches each handle's graph on the handle's own stream, back to
//   back from one host thread (about 8.5 ms of host launch cost per step for
//   512 handles).  FP64-plain handles always step this way.
//
// Either way each handle's results are those of stepping it alone (the same
// device code on the same state).  Ordering: the batch kernels run on the
// batch's own stream after the work queued on every handle's stream and
// before the work queued on them afterwards (events).  Every 32 steps the
// batch waits for the GPU, turns a raised device error bit into
// MRSPH_ERR_DEVICE and makes each handle's neighbour-list capacity check.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "handle.h"

namespace mrsph {  // mrsph_persist.cu
struct Persist;
Persist* persist_create(int device, int kk, int ng);
void persist_destroy(Persist* S);
bool persist_resident(const Persist* S);
int persist_refresh(Persist* S, EngineBase* const* engines, cudaStream_t s);
int persist_steps(Persist* S, int nsteps, int step0, bool persistent, cudaStream_t s);
int persist_check(Persist* S, cudaStream_t s);
bool persist_graph_captured(const Persist* S);
const std::string& persist_error(const Persist* S);
int persist_barrier_selftest(int device, double limit_ms);
}  // namespace mrsph

struct mrsph_batch {
  std::vector<mrsph_handle*> hs;
  std::vector<mrsph::EngineBase*> engines;
  std::vector<cudaEvent_t> ev;  // per handle: end of its queued work / of its part of a timed region
  cudaEvent_t done = nullptr;   // end of the batch's own work
  cudaStream_t stream = nullptr;  // the batch kernels and the timing events run here
  int countdown = 32;             // steps until the next capacity check
  int device = 0;
  int mode = MRSPH_BATCH_STREAMS;
  bool fp32 = true;
  mrsph::Persist* P = nullptr;
  std::string err;
  bool detached = false;  // a handle was destroyed while the batch held it
};

void mrsph_batch_detach(mrsph_batch* b, mrsph_handle* h) {
  cudaSetDevice(b->device);
  cudaStreamSynchronize(b->stream);
  for (size_t k = 0; k < b->hs.size(); k++)
    if (b->hs[k] == h) {
      b->hs[k] = nullptr;
      b->engines[k] = nullptr;
      b->detached = true;
    }
  auto& v = h->batches;
  v.erase(std::remove(v.begin(), v.end(), b), v.end());
}

namespace {

int bfail(mrsph_batch* b, int code, const std::string& msg) {
  b->err = msg;
  return code;
}

// the batch stream waits for every handle's queued work
int batch_after_handles(mrsph_batch* b) {
  for (size_t k = 0; k < b->hs.size(); k++)
    if (cudaEventRecord(b->ev[k], b->hs[k]->stream) != cudaSuccess ||
        cudaStreamWaitEvent(b->stream, b->ev[k], 0) != cudaSuccess)
      return bfail(b, MRSPH_ERR_CUDA, "event ordering failed");
  return 0;
}

// every handle's later work waits for the batch stream
int handles_after_batch(mrsph_batch* b) {
  if (cudaEventRecord(b->done, b->stream) != cudaSuccess) return bfail(b, MRSPH_ERR_CUDA, "event record failed");
  for (auto* h : b->hs)
    if (cudaStreamWaitEvent(h->stream, b->done, 0) != cudaSuccess)
      return bfail(b, MRSPH_ERR_CUDA, "event ordering failed");
  return 0;
}

// wait for every handle's stream, then run the capacity checks
int check_caps(mrsph_batch* b) {
  for (size_t k = 0; k < b->hs.size(); k++) {
    mrsph::EngineBase* e = b->engines[k];
    if (cudaStreamSynchronize(b->hs[k]->stream) != cudaSuccess)
      return bfail(b, MRSPH_ERR_CUDA, "handle " + std::to_string(k) + ": step failed");
    int rc = e->check_capacity();
    if (rc) return bfail(b, rc, "handle " + std::to_string(k) + ": " + e->err);
  }
  return 0;
}

int run_streams(mrsph_batch* b, int nsteps, bool checks) {
  for (int s = 0; s < nsteps; s++) {
    for (size_t k = 0; k < b->hs.size(); k++) {
      mrsph::EngineBase* e = b->engines[k];
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

// persistent / phases: chunks of at most 32 steps (up to the next capacity
// check) on the batch stream
int run_kernels(mrsph_batch* b, int nsteps, bool checks) {
  const bool persistent = b->mode == MRSPH_BATCH_PERSISTENT;
  int rc = batch_after_handles(b);
  while (!rc && nsteps > 0) {
    const int chunk = nsteps < b->countdown ? nsteps : b->countdown;
    rc = mrsph::persist_refresh(b->P, b->engines.data(), b->stream);
    if (!rc) rc = mrsph::persist_steps(b->P, chunk, 0, persistent, b->stream);
    if (rc) return bfail(b, rc, mrsph::persist_error(b->P));
    for (auto* e : b->engines) e->batch_advance(chunk);
    nsteps -= chunk;
    b->countdown -= chunk;
    if (b->countdown <= 0) {
      b->countdown = 32;
      if (checks) {
        rc = mrsph::persist_check(b->P, b->stream);
        if (rc) return bfail(b, rc, mrsph::persist_error(b->P));
        rc = handles_after_batch(b);
        if (!rc) rc = check_caps(b);
        if (!rc) rc = batch_after_handles(b);
      }
    }
  }
  if (!rc) rc = handles_after_batch(b);
  return rc;
}

int run_steps(mrsph_batch* b, int nsteps, bool checks) {
  return b->mode == MRSPH_BATCH_STREAMS ? run_streams(b, nsteps, checks) : run_kernels(b, nsteps, checks);
}

}  // namespace

extern "C" int mrsph_batch_create(mrsph_handle* const* handles, int count, mrsph_batch** out) {
  if (!out || !handles || count < 1) return MRSPH_ERR_ARG;
  *out = nullptr;
  mrsph_batch* b = new mrsph_batch();
  b->device = handles[0] ? handles[0]->prm.device : 0;
  bool wen = true;
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
    b->engines.push_back(h->eng);
    if (h->prm.precision != MRSPH_FP32_SPLIT) b->fp32 = false;
    if (h->prm.kernel != mrsph::K_WEN) wen = false;
  }
  if (cudaSetDevice(b->device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete b;
    return MRSPH_ERR_CUDA;
  }
  b->ev.assign(count, nullptr);
  bool ok = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming) == cudaSuccess;
  for (int k = 0; ok && k < count; k++)
    ok = cudaEventCreateWithFlags(&b->ev[k], cudaEventDisableTiming) == cudaSuccess;
  if (!ok) {
    for (auto e : b->ev)
      if (e) cudaEventDestroy(e);
    if (b->done) cudaEventDestroy(b->done);
    cudaStreamDestroy(b->stream);
    delete b;
    return MRSPH_ERR_CUDA;
  }
  if (b->fp32) {
    b->P = mrsph::persist_create(b->device, wen ? mrsph::K_WEN : -1, count);
    if (b->P) b->mode = mrsph::persist_resident(b->P) ? MRSPH_BATCH_PERSISTENT : MRSPH_BATCH_PHASES;
  }
  for (auto* h : b->hs) h->batches.push_back(b);
  *out = b;
  return 0;
}

extern "C" int mrsph_batch_destroy(mrsph_batch* b) {
  if (!b) return 0;
  cudaSetDevice(b->device);
  cudaStreamSynchronize(b->stream);
  for (auto* h : b->hs) {
    if (!h) continue;  // destroyed before the batch
    cudaStreamSynchronize(h->stream);
    auto& v = h->batches;
    v.erase(std::remove(v.begin(), v.end(), b), v.end());
  }
  mrsph::persist_destroy(b->P);
  for (auto e : b->ev) cudaEventDestroy(e);
  if (b->done) cudaEventDestroy(b->done);
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

extern "C" int mrsph_batch_set_mode(mrsph_batch* b, int mode) {
  if (!b) return MRSPH_ERR_ARG;
  if (mode == MRSPH_BATCH_STREAMS) {
    b->mode = mode;
    return 0;
  }
  if (mode != MRSPH_BATCH_PERSISTENT && mode != MRSPH_BATCH_PHASES) return bfail(b, MRSPH_ERR_ARG, "unknown batch mode");
  if (!b->fp32 || !b->P) return bfail(b, MRSPH_ERR_ARG, "the batch kernels take FP32-split handles only");
  if (mode == MRSPH_BATCH_PERSISTENT && !mrsph::persist_resident(b->P))
    return bfail(b, MRSPH_ERR_STATE, "the persistent batch kernel cannot be resident on this device");
  b->mode = mode;
  return 0;
}

extern "C" int mrsph_batch_get_mode(mrsph_batch* b, int* mode, int* graph_captured) {
  if (!b || !mode) return MRSPH_ERR_ARG;
  *mode = b->mode;
  if (graph_captured) *graph_captured = mrsph::persist_graph_captured(b->P) ? 1 : 0;
  return 0;
}

// a batch whose handle was destroyed steps no more
static int batch_usable(mrsph_batch* b) {
  return b->detached ? bfail(b, MRSPH_ERR_STATE, "a handle of the batch was destroyed") : 0;
}

extern "C" int mrsph_batch_step(mrsph_batch* b, int nsteps) {
  if (!b) return MRSPH_ERR_ARG;
  if (int rc = batch_usable(b)) return rc;
  if (nsteps <= 0) return 0;
  if (cudaSetDevice(b->device) != cudaSuccess) return bfail(b, MRSPH_ERR_CUDA, "cudaSetDevice failed");
  return run_steps(b, nsteps, true);
}

extern "C" int mrsph_batch_step_timed(mrsph_batch* b, int nsteps, double* ms) {
  if (!b || !ms) return MRSPH_ERR_ARG;
  if (int rc = batch_usable(b)) return rc;
  if (cudaSetDevice(b->device) != cudaSuccess) return bfail(b, MRSPH_ERR_CUDA, "cudaSetDevice failed");
  // settle capacities and build every graph outside the timed region
  int rc = check_caps(b);
  for (size_t k = 0; !rc && k < b->hs.size(); k++) {
    rc = b->engines[k]->prepare_steps();
    if (rc) rc = bfail(b, rc, "handle " + std::to_string(k) + ": " + b->engines[k]->err);
  }
  if (rc) return rc;
  if (b->mode != MRSPH_BATCH_STREAMS) b->countdown = 32;  // no capacity check inside the timed steps
  cudaEvent_t t0, t1;
  if (cudaEventCreate(&t0) != cudaSuccess) return bfail(b, MRSPH_ERR_CUDA, "cudaEventCreate failed");
  if (cudaEventCreate(&t1) != cudaSuccess) {
    cudaEventDestroy(t0);
    return bfail(b, MRSPH_ERR_CUDA, "cudaEventCreate failed");
  }
  if (b->mode == MRSPH_BATCH_STREAMS) {
    // t0 on the timing stream; every handle's steps start after it and the
    // timing stream records t1 after every handle's last step
    if (cudaEventRecord(t0, b->stream) != cudaSuccess) rc = bfail(b, MRSPH_ERR_CUDA, "event record failed");
    for (auto* h : b->hs)
      if (!rc && cudaStreamWaitEvent(h->stream, t0, 0) != cudaSuccess)
        rc = bfail(b, MRSPH_ERR_CUDA, "event ordering failed");
    if (!rc) rc = run_streams(b, nsteps, false);
    for (size_t k = 0; !rc && k < b->hs.size(); k++)
      if (cudaEventRecord(b->ev[k], b->hs[k]->stream) != cudaSuccess ||
          cudaStreamWaitEvent(b->stream, b->ev[k], 0) != cudaSuccess)
        rc = bfail(b, MRSPH_ERR_CUDA, "event ordering failed");
    if (!rc && cudaEventRecord(t1, b->stream) != cudaSuccess) rc = bfail(b, MRSPH_ERR_CUDA, "event record failed");
  } else {
    // untimed warm-up of the launch form (graph capture, slot upload) first
    rc = batch_after_handles(b);
    if (!rc && cudaEventRecord(t0, b->stream) != cudaSuccess) rc = bfail(b, MRSPH_ERR_CUDA, "event record failed");
    if (!rc) rc = run_kernels(b, nsteps, false);
    if (!rc && cudaEventRecord(t1, b->stream) != cudaSuccess) rc = bfail(b, MRSPH_ERR_CUDA, "event record failed");
  }
  if (!rc) {
    if (cudaEventSynchronize(t1) != cudaSuccess) rc = bfail(b, MRSPH_ERR_CUDA, "batch step failed");
    float f = 0.f;
    if (!rc && cudaEventElapsedTime(&f, t0, t1) == cudaSuccess) *ms = f;
  }
  if (!rc && b->mode != MRSPH_BATCH_STREAMS) {
    rc = mrsph::persist_check(b->P, b->stream);
    if (rc) bfail(b, rc, mrsph::persist_error(b->P));
  }
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  return rc;
}

extern "C" int mrsph_batch_sync(mrsph_batch* b) {
  if (!b) return MRSPH_ERR_ARG;
  if (int rc = batch_usable(b)) return rc;
  if (cudaSetDevice(b->device) != cudaSuccess) return bfail(b, MRSPH_ERR_CUDA, "cudaSetDevice failed");
  if (cudaStreamSynchronize(b->stream) != cudaSuccess) return bfail(b, MRSPH_ERR_CUDA, "batch stream failed");
  for (auto* h : b->hs)
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) return bfail(b, MRSPH_ERR_CUDA, "handle stream failed");
  if (b->mode != MRSPH_BATCH_STREAMS) {
    int rc = mrsph::persist_check(b->P, b->stream);
    if (rc) return bfail(b, rc, mrsph::persist_error(b->P));
  }
  return 0;
}

extern "C" int mrsph_batch_barrier_selftest(int device, double limit_ms, int* raised) {
  if (!raised || !(limit_ms > 0) || limit_ms > 10000.0) return MRSPH_ERR_ARG;
  int r = mrsph::persist_barrier_selftest(device, limit_ms);
  if (r < 0) return MRSPH_ERR_CUDA;
  *raised = r;
  return 0;
}
