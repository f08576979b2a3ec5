// mrsph_levelset.cu — level-set grid build on the GPU (row A15): normals,
// cut-cell tags, curvature and maximum phi from cell-centred phi, one thread
// per cell.  Restates Levelset::Calculate_level_set (level_set.cpp:238-307):
//   Levelset_package::Get_normal        lset_package.cpp:332-356 (interior)
//   Levelset_package::Get_BC_normal     lset_package.cpp:359-390 (margin packages)
//   Get_interface_tag / Is_cut_cell / Get_phi_at_corners  :450-470, 664-762
//   Get_curvature                       lset_package.cpp:393-434
//   Get_global_scale (maximum_phi)      lset_package.cpp:765-786
// Compiled with -fmad=false (FP64, reference operation order).
#include <cuda_runtime.h>

#include "engine_iface.h"

namespace mrsph {

namespace {

__device__ inline long long lidx(const LsBuildDesc& L, int gi, int gj, int gk) {
  long long a0 = gi + 4 * L.margin, a1 = gj + 4 * L.margin, a2 = (L.D == 3) ? gk + 4 * L.margin : 0;
  return (a2 * L.n[1] + a1) * L.n[0] + a0;
}

__device__ inline bool interior(const LsBuildDesc& L, int gi, int gj, int gk) {
  bool in = gi >= 0 && gi < 4 * L.num_pkg[0] && gj >= 0 && gj < 4 * L.num_pkg[1];
  if (L.D == 3) in = in && gk >= 0 && gk < 4 * L.num_pkg[2];
  return in;
}

__device__ inline int signum(double x) { return (0.0 < x) - (x < 0.0); }

__global__ void k_ls_normal(LsBuildDesc L, const double* __restrict__ phi, double4* __restrict__ g) {
  long long a = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long ntot = (long long)L.n[0] * L.n[1] * L.n[2];
  if (a >= ntot) return;
  int ai = (int)(a % L.n[0]);
  int aj = (int)((a / L.n[0]) % L.n[1]);
  int ak = (int)(a / ((long long)L.n[0] * L.n[1]));
  const int m4 = 4 * L.margin;
  int gi = ai - m4, gj = aj - m4, gk = (L.D == 3) ? ak - m4 : 0;
  auto P = [&](int i, int j, int k) { return phi[lidx(L, i, j, k)]; };
  double gr[3] = {0, 0, 0};
  if (interior(L, gi, gj, gk)) {
    gr[0] = 0.5 * (P(gi + 1, gj, gk) - P(gi - 1, gj, gk)) / L.dcell[0];
    gr[1] = 0.5 * (P(gi, gj + 1, gk) - P(gi, gj - 1, gk)) / L.dcell[1];
    if (L.D == 3) gr[2] = 0.5 * (P(gi, gj, gk + 1) - P(gi, gj, gk - 1)) / L.dcell[2];
  } else {
    int gg[3] = {gi, gj, gk};
    for (int d = 0; d < L.D; d++) {
      int loc = ((gg[d] % 4) + 4) % 4;
      int e[3] = {0, 0, 0};
      e[d] = 1;
      if (loc == 0)
        gr[d] = (P(gi + e[0], gj + e[1], gk + e[2]) - P(gi, gj, gk)) / L.dcell[d];
      else if (loc == 3)
        gr[d] = (P(gi, gj, gk) - P(gi - e[0], gj - e[1], gk - e[2])) / L.dcell[d];
      else
        gr[d] = 0.5 * (P(gi + e[0], gj + e[1], gk + e[2]) - P(gi - e[0], gj - e[1], gk - e[2])) / L.dcell[d];
    }
  }
  double dist = 0.0;
  dist += gr[0] * gr[0];
  dist += gr[1] * gr[1];
  if (L.D == 3) dist += gr[2] * gr[2];
  dist = sqrt(dist) + 1.e-12;
  double inv = 1. / dist;
  g[a] = make_double4(P(gi, gj, gk), gr[0] * inv, gr[1] * inv, (L.D == 3) ? gr[2] * inv : 0.0);
}

// corner vectors in the order of lset_package.cpp:726-733 (0 = minus, 1 = centre, 2 = plus)
__constant__ unsigned char c_cv[8][8][3] = {
    {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {1, 1, 0}, {0, 0, 1}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}},
    {{0, 0, 2}, {1, 0, 2}, {0, 1, 2}, {1, 1, 2}, {0, 0, 1}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}},
    {{1, 0, 2}, {2, 0, 2}, {1, 1, 2}, {2, 1, 2}, {1, 0, 1}, {2, 0, 1}, {1, 1, 1}, {2, 1, 1}},
    {{1, 0, 0}, {2, 0, 0}, {1, 1, 0}, {2, 1, 0}, {1, 0, 1}, {2, 0, 1}, {1, 1, 1}, {2, 1, 1}},
    {{0, 2, 0}, {1, 2, 0}, {0, 1, 0}, {1, 1, 0}, {0, 2, 1}, {1, 2, 1}, {0, 1, 1}, {1, 1, 1}},
    {{0, 2, 2}, {1, 2, 2}, {0, 1, 2}, {1, 1, 2}, {0, 2, 1}, {1, 2, 1}, {0, 1, 1}, {1, 1, 1}},
    {{1, 2, 2}, {2, 2, 2}, {1, 1, 2}, {2, 1, 2}, {1, 2, 1}, {2, 2, 1}, {1, 1, 1}, {2, 1, 1}},
    {{1, 2, 0}, {2, 2, 0}, {1, 1, 0}, {2, 1, 0}, {1, 2, 1}, {2, 2, 1}, {1, 1, 1}, {2, 1, 1}}};

__global__ void k_ls_tag_curv(LsBuildDesc L, const double* __restrict__ phi, uint8_t* __restrict__ tag,
                              double* __restrict__ curv, unsigned long long* __restrict__ max_phi_bits) {
  long long a = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long ntot = (long long)L.n[0] * L.n[1] * L.n[2];
  double my_max = 0.0, my_cmax = 0.0, my_cmin = 1.e20;
  if (a < ntot) {
    int ai = (int)(a % L.n[0]);
    int aj = (int)((a / L.n[0]) % L.n[1]);
    int ak = (int)(a / ((long long)L.n[0] * L.n[1]));
    const int m4 = 4 * L.margin;
    int gi = ai - m4, gj = aj - m4, gk = (L.D == 3) ? ak - m4 : 0;
    auto P = [&](int i, int j, int k) { return phi[lidx(L, i, j, k)]; };
    uint8_t t = 0;
    double cv = 0.0;
    if (interior(L, gi, gj, gk)) {
      double p0 = P(gi, gj, gk);
      if (p0 > 0.) my_max = fabs(p0);
      double v[3][3][3];
      for (int x = 0; x < 3; x++)
        for (int y = 0; y < 3; y++)
          for (int z = 0; z < 3; z++) {
            int kk = (L.D == 3) ? gk + z - 1 : 0;
            v[x][y][z] = P(gi + x - 1, gj + y - 1, kk);
          }
      double corner[8];
      for (int u = 0; u < 8; u++) {
        double w[8];
        for (int q = 0; q < 8; q++) {
          int cz = (L.D == 2) ? 1 : c_cv[u][q][2];
          w[q] = v[c_cv[u][q][0]][c_cv[u][q][1]][cz];
        }
        for (int p = 1; p < 8; p++) {  // ascending insertion sort
          double key = w[p];
          int q = p - 1;
          while (q >= 0 && w[q] > key) { w[q + 1] = w[q]; q--; }
          w[q + 1] = key;
        }
        double s = 0.0;
        for (int q = 0; q < 8; q++) s += w[q];
        corner[u] = s * 0.125;
      }
      bool cut = false;
      for (int c = 0; c < 8; c++)
        if (signum(corner[c]) != signum(corner[0])) cut = true;
      if (signum(v[1][1][1]) != signum(corner[0])) cut = true;
      t = cut ? 1 : 0;
      if (cut) {
        int i = gi, j = gj, k = gk;
        double px, py, pz = 0, pxx, pyy, pzz = 0, pxy, pyz = 0, pxz = 0;
        px = (8.0 * (P(i + 1, j, k) - P(i - 1, j, k)) - (P(i + 2, j, k) - P(i - 2, j, k))) / L.dcell[0] / 12.0;
        pxx = (P(i + 1, j, k) - 2 * P(i, j, k) + P(i - 1, j, k)) / L.dcell[0] / L.dcell[0];
        py = (8.0 * (P(i, j + 1, k) - P(i, j - 1, k)) - (P(i, j + 2, k) - P(i, j - 2, k))) / L.dcell[1] / 12.0;
        pyy = (P(i, j + 1, k) - 2 * P(i, j, k) + P(i, j - 1, k)) / L.dcell[1] / L.dcell[1];
        if (L.D == 3) {
          pz = (8.0 * (P(i, j, k + 1) - P(i, j, k - 1)) - (P(i, j, k + 2) - P(i, j, k - 2))) / L.dcell[2] / 12.0;
          pzz = (P(i, j, k + 1) - 2 * P(i, j, k) + P(i, j, k - 1)) / L.dcell[2] / L.dcell[2];
        }
        pxy = 0.25 * (P(i + 1, j + 1, k) - P(i - 1, j + 1, k) - P(i + 1, j - 1, k) + P(i - 1, j - 1, k)) / L.dcell[0] / L.dcell[1];
        if (L.D == 3) {
          pxz = 0.25 * (P(i + 1, j, k + 1) - P(i - 1, j, k + 1) - P(i + 1, j, k - 1) + P(i - 1, j, k - 1)) / L.dcell[0] / L.dcell[2];
          pyz = 0.25 * (P(i, j + 1, k + 1) - P(i, j + 1, k - 1) - P(i, j - 1, k + 1) + P(i, j - 1, k - 1)) / L.dcell[1] / L.dcell[2];
        }
        double c = (px * px * pyy - 2 * px * py * pxy + py * py * pxx + px * px * pzz - 2 * px * pz * pxz +
                    pz * pz * pxx + py * py * pzz - 2 * py * pz * pyz + pz * pz * pyy) /
                   pow(px * px + py * py + pz * pz, 1.5);
        double cd = 0.0;
        for (int d = 0; d < L.D; d++) cd += L.dcell[d] * L.dcell[d];
        cd = sqrt(cd);
        double lo = -2. / cd, hi = 2. / cd;
        double cl = c >= lo ? c : lo;
        cl = cl <= hi ? cl : hi;
        cv = fabs(cl);
        my_cmax = cv;
        my_cmin = cv;
      }
    }
    tag[a] = t;
    curv[a] = cv;
  }
  // |curvature| range over CUT cells (Get_global_scale, lset_package.cpp:765-785):
  // non-negative values, so the FP64 bit patterns order like the values
  for (int o = 16; o > 0; o >>= 1) {
    my_cmax = fmax(my_cmax, __shfl_xor_sync(0xffffffffu, my_cmax, o));
    my_cmin = fmin(my_cmin, __shfl_xor_sync(0xffffffffu, my_cmin, o));
  }
  if ((threadIdx.x & 31) == 0) {
    if (my_cmax > 0.0) atomicMax(max_phi_bits + 1, (unsigned long long)__double_as_longlong(my_cmax));
    if (my_cmin < 1.e20) atomicMin(max_phi_bits + 2, (unsigned long long)__double_as_longlong(my_cmin));
  }
  // block max of non-negative values -> global bit atomic
  for (int o = 16; o > 0; o >>= 1) my_max = fmax(my_max, __shfl_xor_sync(0xffffffffu, my_max, o));
  __shared__ double sm[32];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sm[wid] = my_max;
  __syncthreads();
  if (wid == 0) {
    int nw = (blockDim.x + 31) >> 5;
    double v = lane < nw ? sm[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (lane == 0 && v > 0.0) atomicMax(max_phi_bits, (unsigned long long)__double_as_longlong(v));
  }
}

__global__ void k_ls_to32(long long ntot, const double4* __restrict__ g, const double* __restrict__ c,
                          float4* __restrict__ g32, float* __restrict__ c32) {
  long long a = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= ntot) return;
  double4 v = g[a];
  g32[a] = make_float4((float)v.x, (float)v.y, (float)v.z, (float)v.w);
  c32[a] = (float)c[a];
}

}  // namespace

// Builds one level in place: g64 (phi, n), c64, tag, and its float copies.
// max_phi_bits[0] accumulates the maximum positive interior phi, [1] and [2]
// the maximum and minimum |curvature| of CUT cells (FP64 bit patterns).
cudaError_t ls_build_level(const LsBuildDesc& L, const double* d_phi, double4* g64, double* c64, float4* g32,
                           float* c32, uint8_t* tag, unsigned long long* max_phi_bits, cudaStream_t s) {
  long long ntot = (long long)L.n[0] * L.n[1] * L.n[2];
  int nb = (int)((ntot + 255) / 256);
  k_ls_normal<<<nb, 256, 0, s>>>(L, d_phi, g64);
  k_ls_tag_curv<<<nb, 256, 0, s>>>(L, d_phi, tag, c64, max_phi_bits);
  k_ls_to32<<<nb, 256, 0, s>>>(ntot, g64, c64, g32, c32);
  return cudaGetLastError();
}

}  // namespace mrsph
