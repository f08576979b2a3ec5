// mrsph_sort.cuh — the counting sort of the cell binning as block functions
// (one call = one 512- or 256-thread block of work, given as blk), shared by
// the per-handle kernels of mrsph_sort.cu and the batch kernels of
// mrsph_persist.cu.  The binning replaces the reference's concurrent
// per-cell push_back (cell_list.cpp:88-91, level_infor.cpp:325-344) and its
// optional radix path (_SCLL_: parallelfunc.h:40-97, cell_list.cpp:103-124):
//
//   counts[key]++            (atomic, inside the map kernel)
//   cstart = exclusive_scan(counts), cstart[ncells] = n
//   perm[cstart[key] + --counts[key]] = i   (atomic; leaves counts at zero)
//   rank inside each cell by particle id -> perm2 (canonical, deterministic)
//
// cstart doubles as the dense lower-bound table used by the neighbour scan:
// every (empty or not) cell has a start, so a run of cells in a row is one
// contiguous range [cstart[c0], cstart[c1 + 1]).
#pragma once
#include <cuda_runtime.h>

namespace mrsph {

constexpr int SCAN_THREADS = 512;  // per-handle scan kernels; the batch kernels scan with 256
constexpr int SCAN_ITEMS = 16;     // cells per thread; a block scans blockDim.x * SCAN_ITEMS cells
constexpr int SCAN_CHUNK = SCAN_THREADS * SCAN_ITEMS;
constexpr int SCAN_CHUNK_MIN = 256 * SCAN_ITEMS;  // the smallest chunk (sizes the block totals)

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

// SCAN_ITEMS consecutive counts of a thread, as 16-byte loads when the group
// lies inside the table (base is a multiple of 16, so the loads are aligned).
// The counts are written by other blocks of the same launch in the batch
// kernels, so the loads are plain (coherent) ones.
__device__ inline void load16(const int* counts, long long base, long long n, int* v) {
  if (base + SCAN_ITEMS <= n) {
    const int4* p = reinterpret_cast<const int4*>(counts + base);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS / 4; k++) {
      const int4 t = p[k];
      v[4 * k] = t.x; v[4 * k + 1] = t.y; v[4 * k + 2] = t.z; v[4 * k + 3] = t.w;
    }
  } else {
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) v[k] = (base + k < n) ? counts[base + k] : 0;
  }
}

// block blk: the total of cells [blk * chunk, +chunk), chunk = blockDim.x *
// SCAN_ITEMS, into blocksums[blk]
__device__ inline void scan_reduce_block(const int* counts, long long n, int* blocksums, long long blk) {
  long long base = blk * (long long)(blockDim.x * SCAN_ITEMS) + (long long)threadIdx.x * SCAN_ITEMS;
  int v[SCAN_ITEMS];
  load16(counts, base, n, v);
  int s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) s += v[k];
  int tot;
  block_excl_scan(s, &tot);
  if (threadIdx.x == 0) blocksums[blk] = tot;
}

// one block: exclusive scan in place over nb block totals, blockDim.x *
// SCAN_ITEMS of them per round, the rounds chained by a carry
__device__ inline void scan_top_block(int* blocksums, long long nb) {
  int carry = 0;
  for (long long r0 = 0; r0 < nb; r0 += (long long)blockDim.x * SCAN_ITEMS) {
    const long long base = r0 + (long long)threadIdx.x * SCAN_ITEMS;
    int v[SCAN_ITEMS];
    int s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
      v[k] = (base + k < nb) ? blocksums[base + k] : 0;
      s += v[k];
    }
    int tot;
    int off = block_excl_scan(s, &tot) + carry;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
      if (base + k < nb) blocksums[base + k] = off;
      off += v[k];
    }
    carry += tot;
  }
}

__device__ inline void scan_down_block(const int* counts, long long n, const int* blocksums, int* cstart, int ntotal,
                                       long long blk) {
  long long base = blk * (long long)(blockDim.x * SCAN_ITEMS) + (long long)threadIdx.x * SCAN_ITEMS;
  int v[SCAN_ITEMS];
  load16(counts, base, n, v);
  int s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) s += v[k];
  int off = block_excl_scan(s, nullptr) + blocksums[blk];
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
  if (blk == 0 && threadIdx.x == 0) cstart[n] = ntotal;
}

// 256-thread block blk of particles
__device__ inline void scatter_block(const int* cellkey, int* cursor, const int* cstart, int* perm, long long n,
                                     long long blk) {
  long long i = blk * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int c = cellkey[i];
  int slot = cstart[c] + atomicSub(&cursor[c], 1) - 1;
  if (slot >= 0 && slot < n) perm[slot] = (int)i;  // a histogram out of step with the keys cannot write outside
}

// Canonical order inside a cell: ascending particle id.
__device__ inline void rank_block(const int* cellkey, const int* cstart, const int* perm, const int* id, int* perm2,
                                  long long n, long long blk) {
  long long s = blk * blockDim.x + threadIdx.x;
  if (s >= n) return;
  int o = perm[s];
  int c = cellkey[o];
  int b = cstart[c], e = cstart[c + 1];
  int my = id[o];
  int r = 0;
  for (int t = b; t < e; t++) r += (id[perm[t]] < my) ? 1 : 0;
  perm2[b + r] = o;
}

}  // namespace mrsph
