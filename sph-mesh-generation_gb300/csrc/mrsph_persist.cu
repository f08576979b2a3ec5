// mrsph_persist.cu — many FP32-split geometries relaxed together by batch
// kernels whose work lists span every geometry.
//
// The reference relaxes one geometry per run (SPH_run_mesh_generation,
// sph_mesh_generation.cpp:1371-1463, driven by Solver::SPH_Mesh_Generation_
// Solver, solver.cpp:257-321).  Here each phase of a step (begin, map, the
// three scan passes, scatter, rank, reorder, density, its fix-up, the two
// force stages with their spilled particles) is a work list of (geometry,
// block) items over all geometries of a batch: blocks of 256 particles,
// blocks of 4096 cells for the scans, or one item per geometry.  Every item
// runs the same block function as the handle's own kernel (engine.cuh,
// mrsph_sort.cuh) on the geometry's BatchSlot, which a block copies into
// shared memory when it moves to another geometry, so each geometry's results
// are those of stepping its handle alone (bit for bit).
//
// Two launch forms over the same items:
//   * persistent: ONE cooperative launch runs up to 32 whole steps of every
//     geometry; the grid (every block resident) walks each phase's list with a
//     stride of its size, and grid-wide barriers separate the phases.  A
//     barrier waits at most BatchPlan::limit_ns for the other blocks; past it
//     the block sets bit 0 of *err and returns, and every other block leaves
//     at its next barrier (the host turns the flag into MRSPH_ERR_DEVICE).
//     Buffers read in one phase were written by other blocks earlier in the
//     same launch, so the persistent kernel reads through coherent loads
//     (LdPlain), never the read-only path.
//   * phases: one launch per phase (14 per step) with one block per item,
//     each phase its own kernel (own register allocation, read-only loads).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "engine.cuh"
#include "mrsph_sort.cuh"

namespace mrsph {

// resident 256-thread blocks per SM of the persistent kernel, i.e. its
// register budget (2: 128 registers, where the fused phases do not spill;
// 4: 64, with spills in the rare paths but twice the warps; measured on a
// GB300 with 512 geometries: 45, 37 and 32 ms per step at 2, 3 and 4)
#ifndef MRSPH_BATCH_MIN_BLOCKS
#define MRSPH_BATCH_MIN_BLOCKS 4
#endif
constexpr int kBatchThreads = 256;
constexpr int kBatchScanCells = kBatchThreads * SCAN_ITEMS;  // cells per scan item

enum BatchPhase {
  BP_BEGIN = 0, BP_MAP, BP_SCAN_REDUCE, BP_SCAN_TOP, BP_SCAN_DOWN, BP_SCATTER, BP_RANK, BP_REORDER,
  BP_DENSITY, BP_FIX, BP_FORCE1, BP_SPILL1, BP_FORCE2, BP_SPILL2, BP_COUNT
};

// A force stage's listed and spilled particles are independent of each
// other, so the persistent kernel runs the spilled ones without a barrier
// between.
__host__ __device__ inline bool barrier_after(int ph) { return ph != BP_FORCE1 && ph != BP_FORCE2; }

// resident blocks per SM the per-phase kernels' register budgets allow: the
// per-handle kernels' tuning
__host__ __device__ constexpr int phase_min_blocks(int ph) {
  return ph == BP_MAP ? MRSPH_MAP_MIN_BLOCKS
         : ph == BP_DENSITY ? MRSPH_DENSITY_MIN_BLOCKS
         : ph == BP_FORCE1 ? MRSPH_FORCE_MIN_BLOCKS
         : ph == BP_FORCE2 ? MRSPH_FORCE2_MIN_BLOCKS : 1;
}

// item lists: 0 one item per geometry, 1 particle blocks, 2 scan blocks,
// 3 queue blocks (the density fix-up and the spilled force stages, whose
// queues hold a few per cent of a geometry's particles at most: one item per
// MRSPH_BATCH_QUEUE_DIV particle blocks, at least one per geometry, each
// striding over the geometry's queue)
constexpr int kBatchLists = 4;
#ifndef MRSPH_BATCH_QUEUE_DIV
#define MRSPH_BATCH_QUEUE_DIV 16
#endif
__host__ __device__ inline int phase_list(int ph) {
  return (ph == BP_BEGIN || ph == BP_SCAN_TOP) ? 0
         : (ph == BP_SCAN_REDUCE || ph == BP_SCAN_DOWN) ? 2
         : (ph == BP_FIX || ph == BP_SPILL1 || ph == BP_SPILL2) ? 3 : 1;
}

// items a block claims at a time from a phase's work queue
#ifndef MRSPH_BATCH_CHUNK
#define MRSPH_BATCH_CHUNK 2
#endif

struct BatchPlan {
  const BatchSlot* slots;  // [ng]
  const long long* off;    // kBatchLists prefix tables of [ng + 1] items
  long long nitems[kBatchLists];
  int ng;
  int nsteps;
  int step0;                // steps of this launch sequence already run (buffer parity)
  unsigned* bar;            // barrier arrivals (zeroed before each persistent launch)
  unsigned* err;            // error bits
  unsigned long long* queue;  // per (step, phase): items claimed (zeroed before each persistent launch)
  unsigned long long limit_ns;
};

__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Grid-wide barrier number epoch (1, 2, ...): arrivals count up to epoch x
// gridDim.x.  Returns false when the wait ran out (this block raised the
// error bit) or another block had raised it.
__device__ bool grid_barrier(unsigned* bar, unsigned* err, unsigned epoch, unsigned long long limit_ns) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(bar, 1u);
    const unsigned target = epoch * gridDim.x;
    const unsigned long long t0 = now_ns();
    int ok = 1;
    while (true) {
      if (*(volatile unsigned*)bar >= target) break;
      if (*(volatile unsigned*)err) { ok = 0; break; }
      if (now_ns() - t0 > limit_ns) {
        atomicOr(err, 1u);
        ok = 0;
        break;
      }
      __nanosleep(64);
    }
    __threadfence();
    if (*(volatile unsigned*)err) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// geometry of item it of a prefix table (binary search)
__device__ __forceinline__ int item_geometry(const long long* off, int ng, long long it) {
  int lo = 0, hi = ng - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (off[mid] <= it) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// the block's copy of the slot of geometry g (all threads call it)
__device__ inline void load_slot(const BatchPlan& P, int g, BatchSlot& s_slot, int& s_g) {
  if (s_g == g) return;
  __syncthreads();
  const int* src = reinterpret_cast<const int*>(P.slots + g);
  int* dst = reinterpret_cast<int*>(&s_slot);
  for (int k = threadIdx.x; k < (int)(sizeof(BatchSlot) / sizeof(int)); k += blockDim.x) dst[k] = src[k];
  __syncthreads();
  if (threadIdx.x == 0) s_g = g;
  __syncthreads();
}

template <int D, int KK, class LD>
__device__ inline void run_item_d(const BatchSlot& S, int ph, long long blk, long long nblk, int cur) {
  const Buf<float>& b0 = S.buf[cur];      // the step's state before the reorder
  const Buf<float>& b1 = S.buf[cur ^ 1];  // after it
  switch (ph) {
    case BP_BEGIN: {
      if (threadIdx.x == 0) begin_step_body(S.c.sc, 1);
      const long long nl = S.c.geo.nc0 * S.c.geo.ncl;
      for (long long k = threadIdx.x; k < nl; k += blockDim.x) S.w.lhmax[k] = 0u;
      break;
    }
    case BP_MAP: map_block<D, float>(S.c, b0, S.w.counts, S.w.lhmax, MAP_STEP, 1000000u, blk); break;
    case BP_SCAN_REDUCE: scan_reduce_block(S.w.counts, S.ncells, S.w.blocksums, blk); break;
    case BP_SCAN_TOP: scan_top_block(S.w.blocksums, (S.ncells + kBatchScanCells - 1) / kBatchScanCells); break;
    case BP_SCAN_DOWN: scan_down_block(S.w.counts, S.ncells, S.w.blocksums, S.w.cstart, (int)S.c.n, blk); break;
    case BP_SCATTER: scatter_block(b0.cellkey, S.w.counts, S.w.cstart, S.w.perm, S.c.n, blk); break;
    case BP_RANK: rank_block(b0.cellkey, S.w.cstart, S.w.perm, b0.id, S.w.perm2, S.c.n, blk); break;
    case BP_REORDER: reorder_block<D, float>(b0, b1, S.c, S.w.perm2, S.w.slot_of_id, S.c.n, 0, blk); break;
    case BP_DENSITY: density_block<D, float, KK, LD>(S.c, b1, S.w, blk); break;
    case BP_FIX: density_fix_items<D, KK, LD>(S.c, b1, S.w, blk, nblk); break;
    case BP_FORCE1:
      if (blk == 0 && threadIdx.x == 0) accum_pairs_body(S.c.sc);
      force_block<D, float, 1, KK, LD>(S.c, b1, S.w, blk);
      break;
    case BP_SPILL1: force_spill_items<D, float, 1, KK, LD>(S.c, b1, S.w, blk, nblk); break;
    case BP_FORCE2: force_block<D, float, 2, KK, LD>(S.c, b1, S.w, blk); break;
    case BP_SPILL2: force_spill_items<D, float, 2, KK, LD>(S.c, b1, S.w, blk, nblk); break;
  }
}

template <int KK, class LD>
__device__ inline void run_item(const BatchPlan& P, int ph, long long it, int step, BatchSlot& s_slot, int& s_g) {
  const int list = phase_list(ph);
  const long long* off = P.off + list * (P.ng + 1);
  const int g = item_geometry(off, P.ng, it);
  load_slot(P, g, s_slot, s_g);
  const long long blk = it - off[g];
  const long long nblk = off[g + 1] - off[g];
  const int cur = (s_slot.cur + step) & 1;
  // in a batch of mixed smoothing kernels (KK = -1) a Wendland geometry takes
  // the Wendland-specialised block functions, as its own handle's kernels do,
  // so its results stay those of stepping it alone
  const bool wen = KK < 0 && s_slot.c.prm.kernel == K_WEN;
  if (s_slot.dim == 2) {
    if (wen) run_item_d<2, K_WEN, LD>(s_slot, ph, blk, nblk, cur);
    else run_item_d<2, KK, LD>(s_slot, ph, blk, nblk, cur);
  } else {
    if (wen) run_item_d<3, K_WEN, LD>(s_slot, ph, blk, nblk, cur);
    else run_item_d<3, KK, LD>(s_slot, ph, blk, nblk, cur);
  }
}

template <int KK>
__global__ void __launch_bounds__(kBatchThreads, MRSPH_BATCH_MIN_BLOCKS) k_batch_persist(BatchPlan P) {
  __shared__ BatchSlot s_slot;
  __shared__ int s_g;
  if (threadIdx.x == 0) s_g = -1;
  __syncthreads();
  __shared__ long long s_it;
  unsigned epoch = 0;
  for (int st = 0; st < P.nsteps; st++) {
    for (int ph = 0; ph < BP_COUNT; ph++) {
      // the phase's work queue: a block claims MRSPH_BATCH_CHUNK consecutive
      // items at a time (mostly of one geometry, so its slot copy is reused)
      const long long n = P.nitems[phase_list(ph)];
      unsigned long long* q = P.queue + (long long)st * BP_COUNT + ph;
      while (true) {
        if (threadIdx.x == 0) s_it = (long long)atomicAdd(q, (unsigned long long)MRSPH_BATCH_CHUNK);
        __syncthreads();
        const long long it0 = s_it;
        __syncthreads();
        if (it0 >= n) break;
        const long long it1 = it0 + MRSPH_BATCH_CHUNK < n ? it0 + MRSPH_BATCH_CHUNK : n;
        for (long long it = it0; it < it1; it++) run_item<KK, LdPlain>(P, ph, it, P.step0 + st, s_slot, s_g);
      }
      if (barrier_after(ph) && !grid_barrier(P.bar, P.err, ++epoch, P.limit_ns)) return;
    }
  }
}

template <int KK, int PH>
__global__ void __launch_bounds__(kBatchThreads, phase_min_blocks(PH)) k_batch_phase(BatchPlan P) {
  __shared__ BatchSlot s_slot;
  __shared__ int s_g;
  if (threadIdx.x == 0) s_g = -1;
  __syncthreads();
  run_item<KK, LdNC>(P, PH, blockIdx.x, P.step0, s_slot, s_g);
}

// A barrier that one block never reaches: the others give up after limit_ns.
__global__ void k_barrier_selftest(unsigned* bar, unsigned* err, unsigned long long limit_ns) {
  if (blockIdx.x == 0) return;
  grid_barrier(bar, err, 1, limit_ns);
}

// ------------------------------------------------------------------- host
struct Persist {
  int device = 0;
  int kk = -1;     // K_WEN when every geometry uses the Wendland kernel
  int grid = 0;    // resident blocks of the persistent kernel
  int ng = 0;
  BatchSlot* d_slots = nullptr;
  long long* d_off = nullptr;
  unsigned* d_flags = nullptr;  // [0] barrier arrivals, [1] error bits
  unsigned long long* d_queue = nullptr;  // work-queue counters, 32 steps x BP_COUNT phases
  std::vector<BatchSlot> h_slots;
  std::vector<long long> h_off;
  long long nitems[kBatchLists] = {0, 0, 0, 0};
  std::vector<std::pair<int, cudaGraphExec_t>> graphs;  // persistent launch per step count
  bool capture_ok = true;
  std::string err;
};

namespace {

template <int KK>
cudaError_t launch_persist(const BatchPlan& P, int grid, cudaStream_t s) {
  BatchPlan q = P;
  void* args[] = {&q};
  return cudaLaunchCooperativeKernel((const void*)k_batch_persist<KK>, dim3(grid), dim3(kBatchThreads), args, 0, s);
}

template <int KK>
cudaError_t launch_phases(const BatchPlan& P, cudaStream_t s) {
  auto L = [&](auto kern, int ph) -> cudaError_t {
    const long long n = P.nitems[phase_list(ph)];
    if (n <= 0) return cudaSuccess;
    kern<<<(unsigned)n, kBatchThreads, 0, s>>>(P);
    return cudaGetLastError();
  };
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = L(k_batch_phase<KK, BP_BEGIN>, BP_BEGIN);
  if (e == cudaSuccess) e = L(k_batch_phase<KK, BP_MAP>, BP_MAP);
  if (e == cudaSuccess) e = L(k_batch_phase<KK, BP_SCAN_REDUCE>, BP_SCAN_REDUCE);
  if (e == cudaSuccess) e = L(k_batch_phase<KK, BP_SCAN_TOP>, BP_SCAN_TOP);
  if (e == cudaSuccess) e = L(k_batch_phase<KK, BP_SCAN_DOWN>, BP_SCAN_DOWN);
  if (e == cudaSuccess) e = L(k_batch_phase<KK, BP_SCATTER>, BP_SCATTER);
  if (e == cudaSuccess) e = L(k_batch_phase<KK, BP_RANK>, BP_RANK);
  if (e == cudaSuccess) e = L(k_batch_phase<KK, BP_REORDER>, BP_REORDER);
  if (e == cudaSuccess) e = L(k_batch_phase<KK, BP_DENSITY>, BP_DENSITY);
  if (e == cudaSuccess) e = L(k_batch_phase<KK, BP_FIX>, BP_FIX);
  if (e == cudaSuccess) e = L(k_batch_phase<KK, BP_FORCE1>, BP_FORCE1);
  if (e == cudaSuccess) e = L(k_batch_phase<KK, BP_SPILL1>, BP_SPILL1);
  if (e == cudaSuccess) e = L(k_batch_phase<KK, BP_FORCE2>, BP_FORCE2);
  if (e == cudaSuccess) e = L(k_batch_phase<KK, BP_SPILL2>, BP_SPILL2);
  return e;
}

BatchPlan plan_of(const Persist& S, int nsteps, int step0) {
  BatchPlan P{};
  P.slots = S.d_slots;
  P.off = S.d_off;
  for (int k = 0; k < kBatchLists; k++) P.nitems[k] = S.nitems[k];
  P.ng = S.ng;
  P.nsteps = nsteps;
  P.step0 = step0;
  P.bar = S.d_flags;
  P.err = S.d_flags + 1;
  P.limit_ns = 1000000000ull;  // one second per barrier wait
  P.queue = S.d_queue;
  return P;
}

}  // namespace

// Resident blocks of the persistent kernel on the device (0 if it cannot run).
int persist_grid(int kk, int device) {
  int sms = 0, bps = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 0;
  int coop = 0;
  if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device) != cudaSuccess || !coop) return 0;
  cudaError_t e = (kk == K_WEN)
                      ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_batch_persist<K_WEN>, kBatchThreads, 0)
                      : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_batch_persist<-1>, kBatchThreads, 0);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return bps * sms;
}

Persist* persist_create(int device, int kk, int ng) {
  Persist* S = new Persist();
  S->device = device;
  S->kk = kk;
  S->ng = ng;
  S->grid = persist_grid(kk, device);
  if (cudaMalloc(&S->d_slots, sizeof(BatchSlot) * ng) != cudaSuccess ||
      cudaMalloc(&S->d_off, sizeof(long long) * kBatchLists * (ng + 1)) != cudaSuccess ||
      cudaMalloc(&S->d_flags, sizeof(unsigned) * 2) != cudaSuccess ||
      cudaMalloc(&S->d_queue, sizeof(unsigned long long) * 32 * BP_COUNT) != cudaSuccess ||
      cudaMemset(S->d_flags, 0, sizeof(unsigned) * 2) != cudaSuccess) {
    cudaGetLastError();
    if (S->d_slots) cudaFree(S->d_slots);
    if (S->d_off) cudaFree(S->d_off);
    if (S->d_flags) cudaFree(S->d_flags);
    if (S->d_queue) cudaFree(S->d_queue);
    delete S;
    return nullptr;
  }
  return S;
}

void persist_destroy(Persist* S) {
  if (!S) return;
  for (auto& g : S->graphs) cudaGraphExecDestroy(g.second);
  cudaFree(S->d_slots);
  cudaFree(S->d_off);
  cudaFree(S->d_flags);
  cudaFree(S->d_queue);
  delete S;
}

bool persist_resident(const Persist* S) { return S && S->grid > 0; }

// The slots and item tables from the engines' current state, copied on s
// (behind the work already queued there).
int persist_refresh(Persist* S, EngineBase* const* engines, cudaStream_t s) {
  const int ng = S->ng;
  S->h_slots.assign(ng, BatchSlot{});
  S->h_off.assign(kBatchLists * (ng + 1), 0);
  for (int g = 0; g < ng; g++) {
    int rc = engines[g]->batch_slot(&S->h_slots[g]);
    if (rc) {
      S->err = "geometry " + std::to_string(g) + ": " + engines[g]->err;
      return rc;
    }
  }
  for (int g = 0; g < ng; g++) {
    const BatchSlot& b = S->h_slots[g];
    S->h_off[0 * (ng + 1) + g + 1] = g + 1;
    S->h_off[1 * (ng + 1) + g + 1] = S->h_off[1 * (ng + 1) + g] + (b.c.n + kBatchThreads - 1) / kBatchThreads;
    S->h_off[2 * (ng + 1) + g + 1] = S->h_off[2 * (ng + 1) + g] + (b.ncells + kBatchScanCells - 1) / kBatchScanCells;
    const long long pb = (b.c.n + kBatchThreads - 1) / kBatchThreads;
    S->h_off[3 * (ng + 1) + g + 1] =
        S->h_off[3 * (ng + 1) + g] + std::max(1LL, (pb + MRSPH_BATCH_QUEUE_DIV - 1) / MRSPH_BATCH_QUEUE_DIV);
  }
  for (int k = 0; k < kBatchLists; k++) S->nitems[k] = S->h_off[k * (ng + 1) + ng];
  // the host vectors are pageable: the copies return once staged
  if (cudaMemcpyAsync(S->d_slots, S->h_slots.data(), sizeof(BatchSlot) * ng, cudaMemcpyHostToDevice, s) !=
          cudaSuccess ||
      cudaMemcpyAsync(S->d_off, S->h_off.data(), sizeof(long long) * kBatchLists * (ng + 1), cudaMemcpyHostToDevice,
                      s) !=
          cudaSuccess) {
    S->err = "batch slot upload failed";
    return MRSPH_ERR_CUDA;
  }
  return 0;
}

// nsteps steps (<= 32) of every geometry on s.  persistent: one cooperative
// launch (replayed from a CUDA graph per step count when capture works);
// otherwise the per-phase kernels.  step0 = steps since the last refresh.
int persist_steps(Persist* S, int nsteps, int step0, bool persistent, cudaStream_t s) {
  if (!persistent) {
    for (int k = 0; k < nsteps; k++) {
      const BatchPlan P = plan_of(*S, 1, step0 + k);
      cudaError_t e = (S->kk == K_WEN) ? launch_phases<K_WEN>(P, s) : launch_phases<-1>(P, s);
      if (e != cudaSuccess) {
        S->err = std::string("batch phase launch: ") + cudaGetErrorString(e);
        return MRSPH_ERR_CUDA;
      }
    }
    return 0;
  }
  if (S->grid <= 0) {
    S->err = "the persistent batch kernel cannot be resident on this device";
    return MRSPH_ERR_STATE;
  }
  if (nsteps < 1 || nsteps > 32) {
    S->err = "a persistent batch launch runs 1 to 32 steps";
    return MRSPH_ERR_ARG;
  }
  const BatchPlan P = plan_of(*S, nsteps, step0);
  auto enqueue = [&](cudaStream_t st) -> cudaError_t {
    cudaError_t e = cudaMemsetAsync(S->d_flags, 0, sizeof(unsigned), st);  // barrier arrivals
    if (e == cudaSuccess) e = cudaMemsetAsync(S->d_queue, 0, sizeof(unsigned long long) * 32 * BP_COUNT, st);
    if (e == cudaSuccess) e = (S->kk == K_WEN) ? launch_persist<K_WEN>(P, S->grid, st) : launch_persist<-1>(P, S->grid, st);
    return e;
  };
  // the plan (step0) changes between launches, so a graph per step count is
  // only reused while step0 is even-aligned the same way: capture per
  // (nsteps, parity of step0)
  const int key = nsteps * 2 + (step0 & 1);
  cudaGraphExec_t ge = nullptr;
  for (auto& g : S->graphs)
    if (g.first == key) ge = g.second;
  if (!ge && S->capture_ok) {
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      cudaError_t e2 = enqueue(s);
      e = cudaStreamEndCapture(s, &graph);
      if (e2 != cudaSuccess) e = e2;
    }
    if (e == cudaSuccess && graph) e = cudaGraphInstantiate(&ge, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      // capture of the cooperative launch not available: launch it directly
      cudaGetLastError();
      S->capture_ok = false;
      ge = nullptr;
    } else {
      S->graphs.push_back({key, ge});
    }
  }
  cudaError_t e = ge ? cudaGraphLaunch(ge, s) : enqueue(s);
  if (e != cudaSuccess) {
    S->err = std::string("persistent batch launch: ") + cudaGetErrorString(e);
    return MRSPH_ERR_CUDA;
  }
  return 0;
}

// The device error bits of the batch (synchronises s); clears them.
int persist_check(Persist* S, cudaStream_t s) {
  unsigned f[2] = {0, 0};
  if (cudaMemcpyAsync(f, S->d_flags, sizeof(f), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess) {
    S->err = "persistent batch kernel failed";
    return MRSPH_ERR_CUDA;
  }
  if (f[1]) {
    cudaMemsetAsync(S->d_flags + 1, 0, sizeof(unsigned), s);
    S->err = "a grid barrier of the persistent batch kernel gave up waiting";
    return MRSPH_ERR_DEVICE;
  }
  return 0;
}

bool persist_graph_captured(const Persist* S) { return S && S->capture_ok && !S->graphs.empty(); }
const std::string& persist_error(const Persist* S) { return S->err; }

// Self-test of the bounded barrier wait: one block of a two-block cooperative
// launch never arrives; the other gives up after limit_ms and raises the
// error bit.  Returns 1 if the flag was raised, 0 if not, < 0 on a CUDA error.
int persist_barrier_selftest(int device, double limit_ms) {
  if (cudaSetDevice(device) != cudaSuccess) return -1;
  unsigned* d = nullptr;
  if (cudaMalloc(&d, sizeof(unsigned) * 2) != cudaSuccess) return -1;
  int out = -1;
  if (cudaMemset(d, 0, sizeof(unsigned) * 2) == cudaSuccess) {
    unsigned* bar = d;
    unsigned* err = d + 1;
    unsigned long long lim = (unsigned long long)(limit_ms * 1.0e6);
    void* args[] = {&bar, &err, &lim};
    if (cudaLaunchCooperativeKernel((const void*)k_barrier_selftest, dim3(2), dim3(32), args, 0, 0) == cudaSuccess &&
        cudaDeviceSynchronize() == cudaSuccess) {
      unsigned f = 0;
      if (cudaMemcpy(&f, err, sizeof(unsigned), cudaMemcpyDeviceToHost) == cudaSuccess) out = f ? 1 : 0;
    }
  }
  cudaGetLastError();
  cudaFree(d);
  return out;
}

}  // namespace mrsph
