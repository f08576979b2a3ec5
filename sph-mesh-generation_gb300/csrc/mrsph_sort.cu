// mrsph_sort.cu — cell binning as a counting sort over the concatenated
// (level, cell) table, the GPU replacement of the reference's concurrent
// per-cell push_back (cell_list.cpp:88-91, level_infor.cpp:325-344) and of its
// optional radix path (_SCLL_: parallelfunc.h:40-97, cell_list.cpp:103-124).
//
//   counts[key]++            (atomic, inside the map kernel)
//   cstart = exclusive_scan(counts), cstart[ncells] = n
//   perm[cstart[key] + --counts[key]] = i   (atomic; leaves counts at zero)
//   rank inside each cell by particle id -> perm2 (canonical, deterministic)
//
// cstart doubles as the dense lower-bound table used by the neighbour scan:
// every (empty or not) cell has a start, so a run of cells in a row is one
// contiguous range [cstart[c0], cstart[c1 + 1]).
#include <cuda_runtime.h>

#include "engine_iface.h"

namespace mrsph {

namespace {
constexpr int SCAN_THREADS = 512;
constexpr int SCAN_ITEMS = 16;
constexpr int SCAN_CHUNK = SCAN_THREADS * SCAN_ITEMS;

__device__ inline int warp_incl_scan(int v) {
  int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// Exclusive block scan of one value per thread; returns the block total.
__device__ inline int block_excl_scan(int v, int* total) {
  __shared__ int wsum[32];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int inc = warp_incl_scan(v);
  if (lane == 31) wsum[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    int nw = blockDim.x >> 5;
    int x = lane < nw ? wsum[lane] : 0;
    int xi = warp_incl_scan(x);
    if (lane < nw) wsum[lane] = xi - x;
    if (lane == nw - 1) wsum[31] = xi;
  }
  __syncthreads();
  int res = inc - v + wsum[wid];
  if (total) *total = wsum[31];
  __syncthreads();
  return res;
}

// The 16 counts of a thread: four 16-byte loads when the group lies inside
// the table (base is a multiple of 16, so the loads are aligned).
__device__ inline void load16(const int* __restrict__ counts, long long base, long long n, int* v) {
  if (base + SCAN_ITEMS <= n) {
    const int4* p = reinterpret_cast<const int4*>(counts + base);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS / 4; k++) {
      const int4 t = __ldg(p + k);
      v[4 * k] = t.x; v[4 * k + 1] = t.y; v[4 * k + 2] = t.z; v[4 * k + 3] = t.w;
    }
  } else {
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) v[k] = (base + k < n) ? counts[base + k] : 0;
  }
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(const int* __restrict__ counts, long long n,
                                                             int* __restrict__ blocksums) {
  long long base = (long long)blockIdx.x * SCAN_CHUNK + (long long)threadIdx.x * SCAN_ITEMS;
  int v[SCAN_ITEMS];
  load16(counts, base, n, v);
  int s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) s += v[k];
  int tot;
  block_excl_scan(s, &tot);
  if (threadIdx.x == 0) blocksums[blockIdx.x] = tot;
}

// single block, exclusive scan in place over nb entries (nb <= SCAN_CHUNK)
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_top(int* blocksums, int nb) {
  int base = threadIdx.x * SCAN_ITEMS;
  int v[SCAN_ITEMS];
  int s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) {
    v[k] = (base + k < nb) ? blocksums[base + k] : 0;
    s += v[k];
  }
  int off = block_excl_scan(s, nullptr);
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) {
    if (base + k < nb) blocksums[base + k] = off;
    off += v[k];
  }
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_down(int* __restrict__ counts, long long n,
                                                           const int* __restrict__ blocksums,
                                                           int* __restrict__ cstart, int ntotal) {
  long long base = (long long)blockIdx.x * SCAN_CHUNK + (long long)threadIdx.x * SCAN_ITEMS;
  int v[SCAN_ITEMS];
  load16(counts, base, n, v);
  int s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) s += v[k];
  int off = block_excl_scan(s, nullptr) + blocksums[blockIdx.x];
  if (base + SCAN_ITEMS <= n) {
    int4* p = reinterpret_cast<int4*>(cstart + base);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS / 4; k++) {
      int4 t;
      t.x = off; off += v[4 * k];
      t.y = off; off += v[4 * k + 1];
      t.z = off; off += v[4 * k + 2];
      t.w = off; off += v[4 * k + 3];
      p[k] = t;
    }
  } else {
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
      long long c = base + k;
      if (c < n) cstart[c] = off;
      off += v[k];
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) cstart[n] = ntotal;
}

__global__ void k_scatter(const int* __restrict__ cellkey, int* cursor, const int* __restrict__ cstart,
                          int* __restrict__ perm, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int c = cellkey[i];
  int slot = cstart[c] + atomicSub(&cursor[c], 1) - 1;
  if (slot >= 0 && slot < n) perm[slot] = (int)i;  // a histogram out of step with the keys cannot write outside
}

// Canonical order inside a cell: ascending particle id.
__global__ void k_rank(const int* __restrict__ cellkey, const int* __restrict__ cstart,
                       const int* __restrict__ perm, const int* __restrict__ id, int* __restrict__ perm2,
                       long long n) {
  long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  int o = perm[s];
  int c = cellkey[o];
  int b = cstart[c], e = cstart[c + 1];
  int my = id[o];
  int r = 0;
  for (int t = b; t < e; t++) r += (id[perm[t]] < my) ? 1 : 0;
  perm2[b + r] = o;
}
}  // namespace

long long scan_blocksums_size(long long ncells) { return (ncells + SCAN_CHUNK - 1) / SCAN_CHUNK + 1; }

void cell_scan(int* counts, int* cstart, int* blocksums, long long ncells, int ntotal, cudaStream_t s) {
  int nb = (int)((ncells + SCAN_CHUNK - 1) / SCAN_CHUNK);
  k_scan_reduce<<<nb, SCAN_THREADS, 0, s>>>(counts, ncells, blocksums);
  k_scan_top<<<1, SCAN_THREADS, 0, s>>>(blocksums, nb);
  k_scan_down<<<nb, SCAN_THREADS, 0, s>>>(counts, ncells, blocksums, cstart, ntotal);
}

void cell_scatter(const int* cellkey, int* cursor, const int* cstart, int* perm, long long n, cudaStream_t s) {
  int nb = (int)((n + 255) / 256);
  k_scatter<<<nb, 256, 0, s>>>(cellkey, cursor, cstart, perm, n);
}

void cell_rank(const int* cellkey, const int* cstart, const int* perm, const int* id, int* perm2, long long n,
               cudaStream_t s) {
  int nb = (int)((n + 255) / 256);
  k_rank<<<nb, 256, 0, s>>>(cellkey, cstart, perm, id, perm2, n);
}

}  // namespace mrsph
