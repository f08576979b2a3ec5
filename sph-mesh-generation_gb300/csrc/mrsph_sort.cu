// mrsph_sort.cu — the per-handle kernels of the cell binning's counting sort
// (block functions in mrsph_sort.cuh).
#include <cuda_runtime.h>

#include "engine_iface.h"
#include "mrsph_sort.cuh"

namespace mrsph {

namespace {
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(const int* __restrict__ counts, long long n,
                                                             int* __restrict__ blocksums) {
  scan_reduce_block(counts, n, blocksums, blockIdx.x);
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_top(int* blocksums, int nb) { scan_top_block(blocksums, nb); }

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_down(int* __restrict__ counts, long long n,
                                                           const int* __restrict__ blocksums,
                                                           int* __restrict__ cstart, int ntotal) {
  scan_down_block(counts, n, blocksums, cstart, ntotal, blockIdx.x);
}

__global__ void k_scatter(const int* __restrict__ cellkey, int* cursor, const int* __restrict__ cstart,
                          int* __restrict__ perm, long long n) {
  scatter_block(cellkey, cursor, cstart, perm, n, blockIdx.x);
}

__global__ void k_rank(const int* __restrict__ cellkey, const int* __restrict__ cstart,
                       const int* __restrict__ perm, const int* __restrict__ id, int* __restrict__ perm2,
                       long long n) {
  rank_block(cellkey, cstart, perm, id, perm2, n, blockIdx.x);
}
}  // namespace

// block totals of the smallest chunk (the batch kernels' 256-thread scans)
long long scan_blocksums_size(long long ncells) { return (ncells + SCAN_CHUNK_MIN - 1) / SCAN_CHUNK_MIN + 1; }

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
