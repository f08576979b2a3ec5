// mrsph_batch.cu — batched relaxation of independent geometries.
//
// The reference relaxes one geometry per run (SPH_mesh_generation::
// SPH_run_mesh_generation, sph_mesh_generation.cpp:1371-1463); relaxing many
// means one run after another.  Here every handle keeps the CUDA graph of
// its own step (12 kernels), and a batch adds one child-graph node per handle
// to a parent graph, one per buffer parity.  One launch of the parent graph
// advances every geometry one step; the child graphs are independent
// branches, so geometries of uneven size run concurrently and small ones fill
// the GPU together.  Each handle's results are those of stepping it alone:
// the child graph is the handle's own step graph.
//
// Ordering with the handles' own streams: work already queued on a handle's
// stream (seeding, state injection) completes before the batch's first step,
// and work queued afterwards on a handle's stream (stats, taps) waits for the
// batch's last step.  Every 32 steps the batch waits for its stream and
// makes the neighbour-list capacity check of each handle, rebuilding the
// parent graphs if a handle's step graph changed.
#include <cuda_runtime.h>

#include <cstring>
#include <string>
#include <vector>

#include "handle.h"

struct mrsph_batch {
  std::vector<mrsph_handle*> hs;
  std::vector<cudaEvent_t> ev;
  std::vector<unsigned> versions;
  std::vector<int> parity;  // each handle's buffer parity when the parent graphs were built
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  cudaGraphExec_t exec[2] = {nullptr, nullptr};
  int phase = 0;       // steps since the parent graphs were built, mod 2
  int countdown = 32;  // steps until the next capacity check
  int device = 0;
  std::string err;
};

namespace {

int bfail(mrsph_batch* b, int code, const std::string& msg) {
  b->err = msg;
  return code;
}

void drop_exec(mrsph_batch* b) {
  for (int p = 0; p < 2; p++)
    if (b->exec[p]) { cudaGraphExecDestroy(b->exec[p]); b->exec[p] = nullptr; }
}

int build_exec(mrsph_batch* b) {
  drop_exec(b);
  for (int p = 0; p < 2; p++) {
    cudaGraph_t parent = nullptr;
    if (cudaGraphCreate(&parent, 0) != cudaSuccess) return bfail(b, MRSPH_ERR_CUDA, "cudaGraphCreate failed");
    for (size_t k = 0; k < b->hs.size(); k++) {
      mrsph::EngineBase* e = b->hs[k]->eng;
      cudaGraph_t g = nullptr;
      int rc = e->step_graph(p, &g);
      if (rc) {
        cudaGraphDestroy(parent);
        return bfail(b, rc, "handle " + std::to_string(k) + ": " + e->err);
      }
      cudaGraphNode_t node;
      if (cudaGraphAddChildGraphNode(&node, parent, nullptr, 0, g) != cudaSuccess) {
        cudaGraphDestroy(parent);
        return bfail(b, MRSPH_ERR_CUDA, "cudaGraphAddChildGraphNode failed");
      }
      b->versions[k] = e->graph_version();
      b->parity[k] = e->parity();
    }
    cudaError_t ce = cudaGraphInstantiate(&b->exec[p], parent, 0);
    cudaGraphDestroy(parent);
    if (ce != cudaSuccess) return bfail(b, MRSPH_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ce));
  }
  b->phase = 0;
  return 0;
}

// wait for every handle's stream, then run the capacity checks
int check_caps(mrsph_batch* b) {
  if (cudaStreamSynchronize(b->stream) != cudaSuccess) return bfail(b, MRSPH_ERR_CUDA, "batch step failed");
  bool stale = false;
  for (size_t k = 0; k < b->hs.size(); k++) {
    mrsph::EngineBase* e = b->hs[k]->eng;
    int rc = e->check_capacity();
    if (rc) return bfail(b, rc, "handle " + std::to_string(k) + ": " + e->err);
    stale = stale || e->graph_version() != b->versions[k];
  }
  if (stale) drop_exec(b);
  return 0;
}

int sync_in(mrsph_batch* b) {
  // a handle stepped alone since the last batch call, or whose step graph
  // was rebuilt, needs new parent graphs
  for (size_t k = 0; k < b->hs.size(); k++) {
    mrsph::EngineBase* e = b->hs[k]->eng;
    if (b->exec[0] && (e->graph_version() != b->versions[k] || e->parity() != (b->parity[k] ^ b->phase))) {
      drop_exec(b);
      break;
    }
  }
  for (size_t k = 0; k < b->hs.size(); k++) {
    if (cudaEventRecord(b->ev[k], b->hs[k]->stream) != cudaSuccess ||
        cudaStreamWaitEvent(b->stream, b->ev[k], 0) != cudaSuccess)
      return bfail(b, MRSPH_ERR_CUDA, "event ordering failed");
  }
  return 0;
}

int sync_out(mrsph_batch* b) {
  if (cudaEventRecord(b->done, b->stream) != cudaSuccess) return bfail(b, MRSPH_ERR_CUDA, "event record failed");
  for (auto* h : b->hs)
    if (cudaStreamWaitEvent(h->stream, b->done, 0) != cudaSuccess)
      return bfail(b, MRSPH_ERR_CUDA, "event ordering failed");
  return 0;
}

int run_steps(mrsph_batch* b, int nsteps, bool checks) {
  for (int s = 0; s < nsteps; s++) {
    if (!b->exec[0]) {
      int rc = build_exec(b);
      if (rc) return rc;
    }
    if (cudaGraphLaunch(b->exec[b->phase], b->stream) != cudaSuccess)
      return bfail(b, MRSPH_ERR_CUDA, "cudaGraphLaunch failed");
    b->phase ^= 1;
    for (auto* h : b->hs) h->eng->batch_advanced(1);
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
      cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming) != cudaSuccess) {
    delete b;
    return MRSPH_ERR_CUDA;
  }
  b->ev.assign(count, nullptr);
  b->versions.assign(count, 0);
  b->parity.assign(count, 0);
  for (int k = 0; k < count; k++)
    if (cudaEventCreateWithFlags(&b->ev[k], cudaEventDisableTiming) != cudaSuccess) {
      for (int q = 0; q < k; q++) cudaEventDestroy(b->ev[q]);
      cudaEventDestroy(b->done);
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
  cudaStreamSynchronize(b->stream);
  drop_exec(b);
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

extern "C" int mrsph_batch_step(mrsph_batch* b, int nsteps) {
  if (!b) return MRSPH_ERR_ARG;
  if (nsteps <= 0) return 0;
  if (cudaSetDevice(b->device) != cudaSuccess) return bfail(b, MRSPH_ERR_CUDA, "cudaSetDevice failed");
  int rc = sync_in(b);
  if (!rc) rc = run_steps(b, nsteps, true);
  if (!rc) rc = sync_out(b);
  return rc;
}

extern "C" int mrsph_batch_step_timed(mrsph_batch* b, int nsteps, double* ms) {
  if (!b || !ms) return MRSPH_ERR_ARG;
  if (cudaSetDevice(b->device) != cudaSuccess) return bfail(b, MRSPH_ERR_CUDA, "cudaSetDevice failed");
  int rc = sync_in(b);
  if (!rc) rc = check_caps(b);  // settle capacities and graphs outside the timed region
  if (!rc && !b->exec[0]) rc = build_exec(b);
  if (rc) return rc;
  cudaEvent_t t0, t1;
  if (cudaEventCreate(&t0) != cudaSuccess) return bfail(b, MRSPH_ERR_CUDA, "cudaEventCreate failed");
  if (cudaEventCreate(&t1) != cudaSuccess) {
    cudaEventDestroy(t0);
    return bfail(b, MRSPH_ERR_CUDA, "cudaEventCreate failed");
  }
  cudaEventRecord(t0, b->stream);
  rc = run_steps(b, nsteps, false);
  cudaEventRecord(t1, b->stream);
  if (!rc) {
    if (cudaEventSynchronize(t1) != cudaSuccess) rc = bfail(b, MRSPH_ERR_CUDA, "batch step failed");
    float f = 0.f;
    if (!rc && cudaEventElapsedTime(&f, t0, t1) == cudaSuccess) *ms = f;
  }
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  if (!rc) rc = sync_out(b);
  return rc;
}

extern "C" int mrsph_batch_sync(mrsph_batch* b) {
  if (!b) return MRSPH_ERR_ARG;
  if (cudaSetDevice(b->device) != cudaSuccess) return bfail(b, MRSPH_ERR_CUDA, "cudaSetDevice failed");
  if (cudaStreamSynchronize(b->stream) != cudaSuccess) return bfail(b, MRSPH_ERR_CUDA, "batch step failed");
  for (auto* h : b->hs)
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) return bfail(b, MRSPH_ERR_CUDA, "handle stream failed");
  return 0;
}
