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

// ------------------------------------------------------------------------
// Cut-cell volume, surface area and mass of one level (row F1):
// Levelset_package::Calculate_volume_mass (lset_package.cpp:1283-1397) with
// GeometryCalculator (geometry_calculator.cpp:12-570), FP64 in the
// reference's operation order.
//
// A cut cell's volume fraction comes from adaptive bisection of its eight
// half-cell sub-cubes (get_subvolume: up to six levels, corner values
// averaged pairwise, a sign vote at the last level).  Every partial volume is
// a multiple of 2^-23 of the cell, so the sum is exact in any order.  The
// surface area polygonises each sub-cube by marching cubes; the polygons of a
// sign case follow from the signs alone (a face with two diagonal corners
// below zero cuts those corners off, as the reference's tables do on every
// ambiguous face) and are split as fans from their lowest edge.

// cube vertices of a sub-cube (geometry_calculator.cpp:296-297) and edges
// (polygonise.cpp:37-60; the first endpoint is interpolated from)
__constant__ unsigned char c_mcv[8][3] = {{0, 0, 0}, {0, 1, 0}, {1, 1, 0}, {1, 0, 0},
                                          {0, 0, 1}, {0, 1, 1}, {1, 1, 1}, {1, 0, 1}};
__constant__ unsigned char c_mce[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                                           {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
__constant__ unsigned char c_mcf[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 5, 4},
                                          {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}};

__device__ int mc_edge_of(int a, int b) {
  for (int e = 0; e < 12; e++)
    if ((c_mce[e][0] == a && c_mce[e][1] == b) || (c_mce[e][0] == b && c_mce[e][1] == a)) return e;
  return 0;
}

// One thread per sign case (bit v set: vertex v below zero): the polygons
// of the case as fans of edge triples, -1 padded to 16 entries.
__global__ void k_mc_table(signed char* __restrict__ tab) {
  const int ci = threadIdx.x;
  if (ci >= 256) return;
  int nb[12][2], nn[12];
  for (int e = 0; e < 12; e++) nn[e] = 0;
  for (int f = 0; f < 6; f++) {
    int in[4], es[4], cut[4], nc = 0;
    for (int k = 0; k < 4; k++) in[k] = (ci >> c_mcf[f][k]) & 1;
    for (int k = 0; k < 4; k++) es[k] = mc_edge_of(c_mcf[f][k], c_mcf[f][(k + 1) & 3]);
    for (int k = 0; k < 4; k++)
      if (in[k] != in[(k + 1) & 3]) cut[nc++] = es[k];
    if (nc == 2) {
      nb[cut[0]][nn[cut[0]]++] = cut[1];
      nb[cut[1]][nn[cut[1]]++] = cut[0];
    } else if (nc == 4) {
      for (int k = 0; k < 4; k++)
        if (in[k]) {
          int a = es[(k + 3) & 3], b = es[k];
          nb[a][nn[a]++] = b;
          nb[b][nn[b]++] = a;
        }
    }
  }
  int n = 0;
  bool seen[12];
  for (int e = 0; e < 12; e++) seen[e] = false;
  for (int s = 0; s < 12; s++) {
    if (nn[s] != 2 || seen[s]) continue;
    int cyc[12], m = 0, prev = s, cur = min(nb[s][0], nb[s][1]);
    cyc[m++] = s;
    seen[s] = true;
    for (int guard = 0; cur != s && guard < 12; guard++) {  // a cycle has at most 12 edges
      cyc[m++] = cur;
      seen[cur] = true;
      int nxt = nb[cur][0] == prev ? nb[cur][1] : nb[cur][0];
      prev = cur;
      cur = nxt;
    }
    for (int k = 1; k + 1 < m && n + 3 <= 15; k++) {
      tab[ci * 16 + n++] = (signed char)cyc[0];
      tab[ci * 16 + n++] = (signed char)cyc[k];
      tab[ci * 16 + n++] = (signed char)cyc[k + 1];
    }
  }
  for (; n < 16; n++) tab[ci * 16 + n] = -1;
}

// check_volume / check_face / mark_volume / mark_face: 1 all positive, 0 all negative, -1 cut
__host__ __device__ inline int gc_mark(const double* v, int n) {
  int flag = 0;
  for (int q = 0; q < n; q++) flag += (v[q] > 0.0) - (v[q] < 0.0);
  return flag == n ? 1 : (flag == -n ? 0 : -1);
}

// rf (3x3x3, [x][y][z]) from the 8 corners cor ([x][y][z]) in the order of
// geometry_calculator.cpp:517-538
template <class T>
__host__ __device__ inline void gc_refine3(const T* cor, T* rf) {
  const T h = (T)0.5;
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2; j++)
      for (int k = 0; k < 2; k++) rf[(2 * i * 3 + 2 * j) * 3 + 2 * k] = cor[(i * 2 + j) * 2 + k];
  for (int i = 0; i < 3; i += 2)
    for (int j = 0; j < 3; j += 2) rf[(i * 3 + j) * 3 + 1] = h * (rf[(i * 3 + j) * 3 + 0] + rf[(i * 3 + j) * 3 + 2]);
  for (int k = 0; k < 3; k++)
    for (int i = 0; i < 3; i += 2) rf[(i * 3 + 1) * 3 + k] = h * (rf[(i * 3 + 0) * 3 + k] + rf[(i * 3 + 2) * 3 + k]);
  for (int j = 0; j < 3; j++)
    for (int k = 0; k < 3; k++) rf[(1 * 3 + j) * 3 + k] = h * (rf[(0 * 3 + j) * 3 + k] + rf[(2 * 3 + j) * 3 + k]);
}

// rf (3x3, [x][y]) from 4 corners, geometry_calculator.cpp:462-473
template <class T>
__host__ __device__ inline void gc_refine2(const T* cor, T* rf) {
  const T h = (T)0.5;
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2; j++) rf[2 * i * 3 + 2 * j] = cor[i * 2 + j];
  for (int i = 0; i < 3; i += 2) rf[i * 3 + 1] = h * (rf[i * 3 + 0] + rf[i * 3 + 2]);
  for (int j = 0; j < 3; j++) rf[3 + j] = h * (rf[0 + j] + rf[6 + j]);
}

template <int D, class T>
__host__ __device__ inline void gc_refine(const T* cor, T* rf) {
  if (D == 3) gc_refine3(cor, rf);
  else gc_refine2(cor, rf);
}

// corners of child c of a refined lattice rf
template <int D, class T>
__host__ __device__ inline void gc_child(const T* rf, int c, T* sub) {
  if (D == 3) {
    const int i = c >> 2, j = (c >> 1) & 1, k = c & 1;
    for (int r = 0; r < 2; r++)
      for (int s = 0; s < 2; s++)
        for (int t = 0; t < 2; t++) sub[(r * 2 + s) * 2 + t] = rf[((i + r) * 3 + (j + s)) * 3 + (k + t)];
  } else {
    const int i = c >> 1, j = c & 1;
    for (int r = 0; r < 2; r++)
      for (int s = 0; s < 2; s++) sub[r * 2 + s] = rf[(i + r) * 3 + (j + s)];
  }
}

// FP64 corners of the node reached from the root corners cor by the child
// indices path[0..n): the reference's refinements along that path.
template <int D>
__host__ __device__ __noinline__ void gc_path64(const double* cor, const int* path, int n, double* out) {
  constexpr int NC = D == 3 ? 8 : 4, NR = D == 3 ? 27 : 9;
  double cur[NC], rf[NR];
  for (int q = 0; q < NC; q++) cur[q] = cor[q];
  for (int l = 0; l < n; l++) {
    gc_refine<D>(cur, rf);
    gc_child<D>(rf, path[l], cur);
  }
  for (int q = 0; q < NC; q++) out[q] = cur[q];
}

// FP32 corners of child c of a node with FP32 corners p: the midpoints of
// the refinement taken axis by axis (z, then y, then x) with selects, so that
// no index depends on c; each value takes at most three rounded midpoints
// (two in 2D) from the node's corners.
template <int D>
__host__ __device__ inline void gc_child32(const float* p, int c, float* out) {
  if (D == 3) {
    const bool i = (c >> 2) & 1, j = (c >> 1) & 1, k = c & 1;
    float z[2][2][2], y[2][2][2];
    for (int x = 0; x < 2; x++)
      for (int yy = 0; yy < 2; yy++) {
        const float a = p[(x * 2 + yy) * 2 + 0], b = p[(x * 2 + yy) * 2 + 1], m = 0.5f * (a + b);
        z[x][yy][0] = k ? m : a;
        z[x][yy][1] = k ? b : m;
      }
    for (int x = 0; x < 2; x++)
      for (int t = 0; t < 2; t++) {
        const float a = z[x][0][t], b = z[x][1][t], m = 0.5f * (a + b);
        y[x][0][t] = j ? m : a;
        y[x][1][t] = j ? b : m;
      }
    for (int s = 0; s < 2; s++)
      for (int t = 0; t < 2; t++) {
        const float a = y[0][s][t], b = y[1][s][t], m = 0.5f * (a + b);
        out[(0 * 2 + s) * 2 + t] = i ? m : a;
        out[(1 * 2 + s) * 2 + t] = i ? b : m;
      }
  } else {
    const bool i = (c >> 1) & 1, j = c & 1;
    float y[2][2];
    for (int x = 0; x < 2; x++) {
      const float a = p[x * 2 + 0], b = p[x * 2 + 1], m = 0.5f * (a + b);
      y[x][0] = j ? m : a;
      y[x][1] = j ? b : m;
    }
    for (int s = 0; s < 2; s++) {
      const float a = y[0][s], b = y[1][s], m = 0.5f * (a + b);
      out[0 * 2 + s] = i ? m : a;
      out[1 * 2 + s] = i ? b : m;
    }
  }
}

// Shared state of one warp of k_vm_walk.
template <int D>
struct VmWarp {
  static constexpr int NC = D == 3 ? 8 : 4;
  double s1[NC][NC];        // cut level-1 nodes (FP64 corners)
  double anc[NC * NC][NC];  // cut level-2 nodes, the anchors (FP64 corners)
  float th[NC * NC], thc[NC * NC];
  float q2[NC * NC][NC];    // queue of level-2 nodes (FP32 corners)
  int c2[NC * NC];          // their codes: anchor << 12 | child path (3 bits per level)
  float q[3][32][NC];       // queues of levels 3..5
  int c[3][32];
};

// Pass 2b, one warp per cut sub-cube: get_subvolume(0, 1/8, cor) (3D) or
// get_face(0, 1/4, cor) (2D), geometry_calculator.cpp:450-570, in units of
// 2^-23 of the cell, added to the cell's units.  Every partial volume of the
// bisection is a multiple of 2^-23 (weights 8^-k or 4^-k, times 1/4, 1/2 or
// 3/4 at the last level, k <= 7), so the FP64 sum is exact in any order and
// equals this integer sum.  Children of a level-l node weigh 8^-(l+2)
// (4^-(l+2)); a cut child below level 6 is refined, at level 6 it counts
// 3/4, 1/2 or 1/4 of its weight by the sign of its corner sum.
//
// Levels 1 and 2 are refined in FP64 as the reference does; the cut level-2
// nodes (anchors) are then bisected breadth-first by the whole warp, one
// (node, child) pair per lane, deepest queue first (so no queue below level
// 2 holds more than 32 nodes).  Only signs steer the bisection, and below
// the anchors they are taken from FP32 copies: with M the largest |corner|
// of the anchor, every FP32 value lies within (1 + 3 * 4) * 2^-24 * M of the
// exact refinement of the anchor's FP64 corners (one rounding for the copy,
// at most three rounded midpoints in each of four levels) and every FP64
// value within 12 * 2^-53 * M, so an FP32 value beyond 2^-20 * M has the
// sign of the FP64 value, and an FP32 corner sum beyond 2^-16 * M (eight
// such errors plus seven rounded additions of magnitude <= 8M) the sign of
// the FP64 sum.  A child with a corner (or a corner sum) inside the bound
// takes its corners from the FP64 refinements along its path from the
// anchor, as the reference computes them.
template <int D>
__global__ void __launch_bounds__(128) k_vm_walk(const int* __restrict__ item_cell, const double* __restrict__ item_cor,
                                                 long long nitem, unsigned* __restrict__ units) {
  constexpr int NC = D == 3 ? 8 : 4, NR = D == 3 ? 27 : 9, LB = D == 3 ? 3 : 2, NB = 32 / NC;
  constexpr unsigned FULL = 0xffffffffu;
  __shared__ VmWarp<D> smem[4];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long it = (long long)blockIdx.x * 4 + wid;
  if (it >= nitem) return;  // whole warps
  VmWarp<D>& S = smem[wid];
  const unsigned below = (1u << lane) - 1u;
  double root[NC];
  for (int q = 0; q < NC; q++) root[q] = item_cor[it * NC + q];
  unsigned acc = 0;
  // level 1 (FP64), one child per lane
  bool cut1 = false;
  if (lane < NC) {
    double rf[NR], s1[NC];
    gc_refine<D>(root, rf);
    gc_child<D>(rf, lane, s1);
    const int f = gc_mark(s1, NC);
    if (f == 1) acc += 1u << (23 - 2 * LB);
    if (f == -1) {
      cut1 = true;
      for (int q = 0; q < NC; q++) S.s1[lane][q] = s1[q];
    }
  }
  const unsigned m1 = __ballot_sync(FULL, cut1);
  __syncwarp();
  // level 2 (FP64): the anchors
  int n2 = 0;
  for (int t0 = 0; t0 < NC * NC; t0 += 32) {
    const int t = t0 + lane;
    bool app = false;
    double s2[NC];
    if (t < NC * NC && ((m1 >> (t / NC)) & 1)) {
      double p[NC], rf[NR];
      for (int q = 0; q < NC; q++) p[q] = S.s1[t / NC][q];
      gc_refine<D>(p, rf);
      gc_child<D>(rf, t % NC, s2);
      const int f = gc_mark(s2, NC);
      if (f == 1) acc += 1u << (23 - 3 * LB);
      app = f == -1;
    }
    const unsigned ma = __ballot_sync(FULL, app);
    if (app) {
      const int pos = n2 + __popc(ma & below);
      double M = 0.0;
      for (int q = 0; q < NC; q++) {
        S.anc[pos][q] = s2[q];
        S.q2[pos][q] = (float)s2[q];
        M = fmax(M, fabs(s2[q]));
      }
      S.th[pos] = (float)(M * 0x1p-20) + 1.e-37f;
      S.thc[pos] = (float)(M * 0x1p-16) + 1.e-37f;
      S.c2[pos] = pos << 12;
    }
    n2 += __popc(ma);
  }
  __syncwarp();
  // levels 3..6 (FP32 signs): queue 0 = level 2, queues 1..3 = levels 3..5
  int n0 = n2, n1 = 0, nq2 = 0, n3 = 0;
  for (int guard = 0; guard < (1 << 20); guard++) {
    const int l = n3 ? 3 : (nq2 ? 2 : (n1 ? 1 : (n0 ? 0 : -1)));  // deepest non-empty queue
    if (l < 0) break;
    const int have = l == 0 ? n0 : (l == 1 ? n1 : (l == 2 ? nq2 : n3));
    const int k = have < NB ? have : NB;
    const int base = have - k;
    if (l == 0) n0 -= k;
    else if (l == 1) n1 -= k;
    else if (l == 2) nq2 -= k;
    else n3 -= k;
    const int nd = lane / NC, c = lane % NC;
    const bool live = nd < k;
    float pc[NC], ch[NC];
    int code = 0;
    if (live) {
      const float* src = l == 0 ? S.q2[base + nd] : S.q[l - 1][base + nd];
      for (int q = 0; q < NC; q++) pc[q] = src[q];
      code = l == 0 ? S.c2[base + nd] : S.c[l - 1][base + nd];
    }
    __syncwarp();
    const int lev = l + 3;                  // the child's refinement level
    const int sh = 23 - LB * (lev + 1);     // its weight, 2^sh units
    int f = 2;
    bool push = false;
    if (live) {
      gc_child32<D>(pc, c, ch);
      const int anc = code >> 12;
      const float th = S.th[anc];
      int pos = 0, neg = 0;
      for (int q = 0; q < NC; q++) {
        pos += ch[q] > th;
        neg += ch[q] < -th;
      }
      double s64[NC];
      bool have64 = false;
      int path[4];
      for (int m = 0; m < l; m++) path[m] = (code >> (3 * m)) & 7;
      path[l] = c;
      if (pos + neg == NC) {
        f = pos == NC ? 1 : (neg == NC ? 0 : -1);
      } else {
        gc_path64<D>(S.anc[anc], path, l + 1, s64);
        have64 = true;
        f = gc_mark(s64, NC);
      }
      if (f == 1) acc += 1u << sh;
      if (f == -1) {
        if (lev <= 5) {
          push = true;
        } else {
          float cv = 0.f;
          for (int q = 0; q < NC; q++) cv += ch[q];
          int sg;
          if (fabsf(cv) > S.thc[anc]) {
            sg = cv > 0.f ? 1 : -1;
          } else {
            if (!have64) gc_path64<D>(S.anc[anc], path, l + 1, s64);
            double cv64 = 0.0;
            for (int q = 0; q < NC; q++) cv64 += s64[q];
            sg = cv64 > 0.0 ? 1 : (cv64 == 0.0 ? 0 : -1);
          }
          acc += (unsigned)(sg > 0 ? 3 : (sg == 0 ? 2 : 1)) << (sh - 2);
        }
      }
    }
    const unsigned mp = __ballot_sync(FULL, push);
    if (mp) {  // l < 3 here; queue l + 1 is empty before this batch
      const int cnt = l == 0 ? n1 : (l == 1 ? nq2 : n3);
      if (push) {
        const int pos = cnt + __popc(mp & below);
        for (int q = 0; q < NC; q++) S.q[l][pos][q] = ch[q];
        S.c[l][pos] = code | (c << (3 * l));
      }
      if (l == 0) n1 += __popc(mp);
      else if (l == 1) nq2 += __popc(mp);
      else n3 += __popc(mp);
    }
    __syncwarp();
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(FULL, acc, o);
  if (lane == 0 && acc) atomicAdd(units + item_cell[it], acc);
}

// Polygonise_MQ::VertexInterp at isolevel 0 (polygonise.cpp:74-92), one axis
__device__ inline void mc_interp(const double* p1, const double* p2, double v1, double v2, double* o) {
  if (fabs(0.0 - v1) < 1.0e-15) {
    o[0] = p1[0]; o[1] = p1[1]; o[2] = p1[2];
    return;
  }
  if (fabs(0.0 - v2) < 1.0e-15) {
    o[0] = p2[0]; o[1] = p2[1]; o[2] = p2[2];
    return;
  }
  if (fabs(v1 - v2) < 1.0e-15) {
    o[0] = p1[0]; o[1] = p1[1]; o[2] = p1[2];
    return;
  }
  const double mu = (0.0 - v1) / (v2 - v1);
  for (int a = 0; a < 3; a++) o[a] = p1[a] + mu * (p2[a] - p1[a]);
}

// GeometryCalculator::get_area_tri, geometry_calculator.cpp:325-350
__device__ inline double mc_tri_area(const double* p1, const double* p2, const double* p3) {
  const double v1x = p2[0] - p1[0], v1y = p2[1] - p1[1], v1z = p2[2] - p1[2];
  const double v3x = p3[0] - p1[0], v3y = p3[1] - p1[1], v3z = p3[2] - p1[2];
  const double d1 = sqrt(v1x * v1x + v1y * v1y + v1z * v1z);
  const double d3 = sqrt(v3x * v3x + v3y * v3y + v3z * v3z);
  double a = 0.5 * (d3 * d1) * sin(acos((v1x * v3x + v1y * v3y + v1z * v3z) / (d3 * d1 + 1.e-20)));
  return isnan(a) ? 0.0 : a;
}

// Marching-cubes area of sub-cube (i, j, k) of a 3x3x3 lattice c ([x][y][z]),
// one term of get_area_MQ (geometry_calculator.cpp:283-321)
__device__ double mc_subcube_area(const double* c, int i, int j, int k, double dx, double dy, double dz,
                                  const signed char* tab) {
  double p[8][3], val[8];
  int ci = 0;
  for (int v = 0; v < 8; v++) {
    const int vx = i + c_mcv[v][0], vy = j + c_mcv[v][1], vz = k + c_mcv[v][2];
    p[v][0] = vx * 0.5 * dx;
    p[v][1] = vy * 0.5 * dy;
    p[v][2] = vz * 0.5 * dz;
    val[v] = c[(vx * 3 + vy) * 3 + vz];
    if (val[v] < 0.0) ci |= 1 << v;
  }
  const signed char* t = tab + ci * 16;
  double area = 0.0;
  for (int q = 0; q < 15 && t[q] >= 0; q += 3) {
    double a[3][3];
    for (int u = 0; u < 3; u++) {
      const int e = t[q + u], v0 = c_mce[e][0], v1 = c_mce[e][1];
      mc_interp(p[v0], p[v1], val[v0], val[v1], a[u]);
    }
    area += mc_tri_area(a[0], a[1], a[2]);
  }
  return area;
}

__device__ inline long long vm_index(const LsLevel& L, int D, int gi, int gj, int gk) {
  const long long m4 = 4 * L.margin;
  return (((D == 3) ? gk + m4 : 0) * L.n[1] + (gj + m4)) * L.n[0] + (gi + m4);
}

__device__ inline void vm_cell_of(const LsLevel& L, int D, long long q, int* g) {
  const int n0 = 4 * L.num_pkg[0], n1 = 4 * L.num_pkg[1];
  g[0] = (int)(q % n0);
  g[1] = (int)((q / n0) % n1);
  g[2] = (D == 3) ? (int)(q / ((long long)n0 * n1)) : 0;
}

__device__ inline bool vm_counted(double phi, double dl) { return phi > 0. || fabs(phi) < dl; }

// Pass 1, one thread per interior cell: CUT cells are counted
// (glbl_num_interface_cell) and those the mass sums include are listed.
__global__ void k_vm_list(LsLevel L, int D, long long nin, double dl, int* __restrict__ list,
                          unsigned long long* __restrict__ cnt) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  bool cut = false, listed = false;
  long long a = 0;
  if (q < nin) {
    int g[3];
    vm_cell_of(L, D, q, g);
    a = vm_index(L, D, g[0], g[1], g[2]);
    cut = L.tag[a] != 0;
    listed = cut && vm_counted(L.g64[a].x, dl);
  }
  const unsigned mc = __ballot_sync(0xffffffffu, cut), ml = __ballot_sync(0xffffffffu, listed);
  const int lane = threadIdx.x & 31;
  unsigned long long base = 0;
  if (lane == 0) {
    if (mc) atomicAdd(cnt + 0, (unsigned long long)__popc(mc));
    if (ml) base = atomicAdd(cnt + 1, (unsigned long long)__popc(ml));
  }
  base = __shfl_sync(0xffffffffu, base, 0);
  if (listed) list[base + __popc(ml & ((1u << lane) - 1u))] = (int)(a);
}

// Pass 2, eight threads per listed CUT cell (thread s: half-cell sub-cube
// (s>>2, (s>>1)&1, s&1)): Get_corner and Get_surface_area
// (geometry_calculator.cpp:12-262) and the first level of
// Get_cutcell_volume: full sub-cubes add their units to the cell, cut ones
// become work items (cell, FP64 corners) for pass 2b.  Cells whose corner
// lattice is not cut get their volume here.
template <int D>
__global__ void __launch_bounds__(256) k_vm_cut(LsLevel L, const int* __restrict__ list, long long nlist,
                                                const signed char* __restrict__ gtab, double* __restrict__ cvol,
                                                double* __restrict__ carea, unsigned* __restrict__ units,
                                                signed char* __restrict__ mark, int* __restrict__ item_cell,
                                                double* __restrict__ item_cor, unsigned long long* __restrict__ nitem) {
  __shared__ signed char tab[256 * 16];
  for (int t = threadIdx.x; t < 256 * 16 / 4; t += blockDim.x)
    reinterpret_cast<int*>(tab)[t] = reinterpret_cast<const int*>(gtab)[t];
  __syncthreads();
  constexpr int NC = D == 3 ? 8 : 4;
  const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 3;
  const int s = threadIdx.x & 7;
  const bool live = w < nlist;
  const long long a = live ? list[w] : 0;
  double area_s = 0.0, sub[8];
  unsigned u = 0;
  bool emit = false;
  int marker = 0;
  const double dx = L.dcell[0], dy = L.dcell[1], dz = D == 3 ? L.dcell[2] : 1.0;
  if (live) {
    // phii0: the 3^D neighbourhood (z index 0 in 2D)
    double p[27], c[27];
    const long long sx = 1, sy = L.n[0], sz = (long long)L.n[0] * L.n[1];
    for (int r = 0; r < 3; r++)
      for (int q = 0; q < 3; q++)
        for (int t = 0; t < 3; t++) {
          if (D == 2 && t > 0) {
            p[(r * 3 + q) * 3 + t] = 0.0;
            continue;
          }
          const long long off = (r - 1) * sx + (q - 1) * sy + (D == 3 ? (t - 1) * sz : 0);
          p[(r * 3 + q) * 3 + t] = L.g64[a + off].x;
        }
    // Get_corner, geometry_calculator.cpp:12-77
    constexpr int DZ = D == 3 ? 1 : 0;
    auto P = [&](int r, int q, int t) { return p[(r * 3 + q) * 3 + t]; };
    auto Cc = [&](int r, int q, int t) -> double& { return c[(r * 3 + q) * 3 + t]; };
    for (int v = 0; v < 27; v++) c[v] = 0.0;
    Cc(1, 1, DZ) = P(1, 1, DZ);
    for (int r = 0; r < 2; r++)
      for (int q = 0; q < 2; q++)
        for (int t = 0; t < 1 + DZ; t++)
          Cc(2 * r, 2 * q, 2 * t) = 0.125 * (P(r, q, t) + P(r + 1, q, t) + P(r, q + 1, t) + P(r + 1, q + 1, t) +
                                             P(r, q, t + DZ) + P(r + 1, q, t + DZ) + P(r, q + 1, t + DZ) +
                                             P(r + 1, q + 1, t + DZ));
    if (DZ)
      for (int r = 0; r < 2; r++)
        for (int q = 0; q < 2; q++)
          Cc(2 * r, 2 * q, 1) = 0.25 * (P(r, q, 1) + P(r + 1, q, 1) + P(r, q + 1, 1) + P(r + 1, q + 1, 1));
    for (int q = 0; q < 2; q++)
      for (int t = 0; t < 1 + DZ; t++)
        Cc(1, 2 * q, 2 * t) = 0.25 * (P(1, q, t) + P(1, q, t + DZ) + P(1, q + 1, t) + P(1, q + 1, t + DZ));
    for (int r = 0; r < 2; r++)
      for (int t = 0; t < 1 + DZ; t++)
        Cc(2 * r, 1, 2 * t) = 0.25 * (P(r, 1, t) + P(r + 1, 1, t) + P(r, 1, t + DZ) + P(r + 1, 1, t + DZ));
    if (DZ)
      for (int r = 0; r < 2; r++) {
        Cc(2 * r, 1, 1) = 0.5 * (P(r, 1, 1) + P(r + 1, 1, 1));
        Cc(1, 2 * r, 1) = 0.5 * (P(1, r, 1) + P(1, r + 1, 1));
        Cc(1, 1, 2 * r) = 0.5 * (P(1, 1, r) + P(1, 1, r + 1));
      }
    if (D == 3) {
      marker = gc_mark(c, 27);
      if (marker == -1) {
        const int i = s >> 2, j = (s >> 1) & 1, k = s & 1;
        for (int r = 0; r < 2; r++)
          for (int q = 0; q < 2; q++)
            for (int t = 0; t < 2; t++) sub[(r * 2 + q) * 2 + t] = Cc(i + r, j + q, k + t);
        area_s = mc_subcube_area(c, i, j, k, dx, dy, dz, tab);
      }
    } else {
      double face[9], ext[27];
      for (int r = 0; r < 3; r++)
        for (int q = 0; q < 3; q++) face[r * 3 + q] = Cc(r, q, 0);
      marker = gc_mark(face, 9);
      if (marker == -1) {
        if (s < 4) {
          const int i = s >> 1, j = s & 1;
          for (int r = 0; r < 2; r++)
            for (int q = 0; q < 2; q++) sub[r * 2 + q] = face[(i + r) * 3 + (j + q)];
        }
        // the face extruded over a unit depth (geometry_calculator.cpp:137-148)
        for (int r = 0; r < 3; r++)
          for (int q = 0; q < 3; q++)
            for (int t = 0; t < 3; t++) ext[(r * 3 + q) * 3 + t] = face[r * 3 + q];
        area_s = mc_subcube_area(ext, s >> 2, (s >> 1) & 1, s & 1, dx, dy, 1.0, tab);
      }
    }
    if (marker == -1 && (D == 3 || s < 4)) {
      const int f = gc_mark(sub, NC);
      if (f == 1) u = 1u << (23 - (D == 3 ? 3 : 2));
      else if (f == -1) emit = true;
    }
  }
  // work items, warp-aggregated
  const unsigned me = __ballot_sync(0xffffffffu, emit);
  const int lane = threadIdx.x & 31;
  unsigned long long base = 0;
  if (lane == 0 && me) base = atomicAdd(nitem, (unsigned long long)__popc(me));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (emit) {
    const unsigned long long it = base + __popc(me & ((1u << lane) - 1u));
    item_cell[it] = (int)w;
    for (int q = 0; q < NC; q++) item_cor[it * NC + q] = sub[q];
  }
  // the eight sub-cubes of a cell in order (s = 0..7)
  double asum = 0.0;
  unsigned usum = 0;
  const int g0 = threadIdx.x & 24;
  for (int v = 0; v < 8; v++) {
    asum += __shfl_sync(0xffffffffu, area_s, g0 + v);
    usum += __shfl_sync(0xffffffffu, u, g0 + v);
  }
  if (live && s == 0) {
    mark[w] = (signed char)marker;
    units[w] = usum;
    if (marker != -1) cvol[a] = (marker == 1 ? 1.0 : 0.0) * (dx * dy * dz);
    carea[a] = marker == -1 ? asum : 0.0;
  }
}

// Pass 2c, one thread per listed cell with a cut corner lattice: volume =
// min(fraction, 1) * cell volume (get_volume / get_area, then
// Get_cutcell_volume).
__global__ void k_vm_finish(const int* __restrict__ list, long long nlist, const unsigned* __restrict__ units,
                            const signed char* __restrict__ mark, double dv, double* __restrict__ cvol) {
  const long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nlist || mark[w] != -1) return;
  const double vof = (double)units[w] * 0x1p-23;
  const double H = vof <= 1.0 ? vof : 1.0;
  cvol[list[w]] = H * dv;
}

// Length of segment v0-v1 inside the box [mn, mx]: the segment is clipped
// to the parameter range [0, 1] by the box's three slabs in turn, each slab
// giving the parameters where the segment crosses its two planes (IEEE
// infinities and NaNs for a segment parallel to it, which the comparisons
// then pass or reject), and the clipped piece's length is returned (0 when
// it is empty).  Segment_AABB_Intersection (AABB_calculator.cpp:6-55) and
// GeometryCalculator::Get_segment_length (geometry_calculator.cpp:571-589),
// in their operation order (this file is compiled with -fmad=false).
__device__ inline double seg_box_length(const double* mn, const double* mx, const double* v0, const double* v1) {
  double f0 = 0., f1 = 1.;
  for (int d = 0; d < 3; d++) {
    double a = (mn[d] - v0[d]) / (v1[d] - v0[d]);
    double b = (mx[d] - v0[d]) / (v1[d] - v0[d]);
    if (b < a) {
      const double t = a;
      a = b;
      b = t;
    }
    if (b < f0 || a > f1) return 0.;
    f0 = a >= f0 ? a : f0;
    f1 = b <= f1 ? b : f1;
    if (f0 > f1) return 0.;
  }
  double pp[3];
  for (int d = 0; d < 3; d++) pp[d] = ((v1[d] - v0[d]) * f1 + v0[d]) - ((v1[d] - v0[d]) * f0 + v0[d]);
  return sqrt(pp[0] * pp[0] + pp[1] * pp[1] + pp[2] * pp[2]);
}

// Pass 3, one thread per interior cell: the mass sums of
// Calculate_volume_mass (lset_package.cpp:1340-1395) with
// scale = Get_scale(curv, phi), into per-block partials (fixed order): mass,
// surface mass, volume, area, and in 3D the segment mass and length of the
// SEGMENT cells (:1371-1383).
template <int D>
__global__ void __launch_bounds__(256) k_vm_reduce(LsSet ls, int level, long long nin, double dl,
                                                   double* __restrict__ cvol, double* __restrict__ carea,
                                                   double* __restrict__ part) {
  const LsLevel& L = ls.lv[level];
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double m = 0., ms = 0., v = 0., ar = 0., mg = 0., lg = 0.;
  if (q < nin) {
    int g[3];
    vm_cell_of(L, D, q, g);
    const long long a = vm_index(L, D, g[0], g[1], g[2]);
    const double phi = L.g64[a].x;
    if (vm_counted(phi, dl)) {
      const double scale = get_scale<double>(ls, phi, L.c64[a]);
      double vol, area = 0.;
      if (L.tag[a] != 0) {
        vol = cvol[a];
        area = carea[a];
        double sp = 1.0;
        for (int d = 0; d < D - 1; d++) sp *= scale;
        ar = area;
        ms = area / sp;
      } else {
        vol = (L.dcell[0] * L.dcell[1]) * (D == 3 ? L.dcell[2] : 1.0);
        cvol[a] = vol;
      }
      if (D == 3 && L.chr && L.chr[a] > 0) {  // a SEGMENT cell of segment chr - 1
        double mn[3], mx[3];
        for (int d = 0; d < 3; d++) {
          const int pk = g[d] >> 2, ce = g[d] & 3;
          mn[d] = (pk * L.dpkg[d] + ce * L.dcell[d]) + L.box_l[d];
          mx[d] = mn[d] + L.dcell[d];
        }
        const double* sg = ls.seg + 6 * (L.chr[a] - 1);
        lg = seg_box_length(mn, mx, sg, sg + 3);
        mg = lg / scale;
      }
      double sp = 1.0;
      for (int d = 0; d < D; d++) sp *= scale;
      m = vol / sp;
      v = vol;
    }
  }
  __shared__ double sm[6][256];
  sm[0][threadIdx.x] = m;
  sm[1][threadIdx.x] = ms;
  sm[2][threadIdx.x] = v;
  sm[3][threadIdx.x] = ar;
  sm[4][threadIdx.x] = mg;
  sm[5][threadIdx.x] = lg;
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if (threadIdx.x < st)
      for (int u = 0; u < 6; u++) sm[u][threadIdx.x] += sm[u][threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x < 6) part[(long long)blockIdx.x * 6 + threadIdx.x] = sm[threadIdx.x][0];
}

// Pass 4, one block: the partials summed in a fixed order.
__global__ void __launch_bounds__(256) k_vm_final(const double* __restrict__ part, long long nb,
                                                  double* __restrict__ tot) {
  __shared__ double sm[6][256];
  double acc[6] = {0., 0., 0., 0., 0., 0.};
  for (long long b = threadIdx.x; b < nb; b += blockDim.x)
    for (int u = 0; u < 6; u++) acc[u] += part[b * 6 + u];
  for (int u = 0; u < 6; u++) sm[u][threadIdx.x] = acc[u];
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if (threadIdx.x < st)
      for (int u = 0; u < 6; u++) sm[u][threadIdx.x] += sm[u][threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x < 6) tot[threadIdx.x] = sm[threadIdx.x][0];
}

}  // namespace

// Cut-cell volume / area / mass pass of one level (see above).  Device
// buffers: cvol, carea (full grid incl. margins, zeroed here), list (one int
// per interior cell), part (6 doubles per 256 interior cells), tab (4 KB),
// cnt (3 counters), tot (6 doubles); the work items of the cut sub-cubes
// are allocated here once their number is known.  Enqueued on s, which is
// synchronised twice.
cudaError_t ls_volume_mass(const LsSet& ls, int level, int D, double* cvol, double* carea, int* list,
                           double* part, signed char* tab, unsigned long long* cnt, double* tot,
                           long long* ncut_listed_host, cudaStream_t s) {
  const LsLevel& L = ls.lv[level];
  long long ntot = 1, nin = 1;
  for (int d = 0; d < D; d++) {
    ntot *= L.n[d];
    nin *= 4LL * L.num_pkg[d];
  }
  double dl = 1.e20;  // lset_level_infor.cpp:48-52
  for (int d = 0; d < D; d++) dl = dl <= L.dcell[d] ? dl : L.dcell[d];
  const double dv = (L.dcell[0] * L.dcell[1]) * (D == 3 ? L.dcell[2] : 1.0);
  cudaError_t e;
  if ((e = cudaMemsetAsync(cvol, 0, sizeof(double) * ntot, s)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(carea, 0, sizeof(double) * ntot, s)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(cnt, 0, 3 * sizeof(unsigned long long), s)) != cudaSuccess) return e;
  k_mc_table<<<1, 256, 0, s>>>(tab);
  const long long nb = (nin + 255) / 256;
  k_vm_list<<<(unsigned)nb, 256, 0, s>>>(L, D, nin, dl, list, cnt);
  unsigned long long hc[2] = {0, 0};
  if ((e = cudaMemcpyAsync(hc, cnt, sizeof(hc), cudaMemcpyDeviceToHost, s)) != cudaSuccess) return e;
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
  ncut_listed_host[0] = (long long)hc[0];
  ncut_listed_host[1] = (long long)hc[1];
  const long long nl = (long long)hc[1];
  if (nl > 0) {
    // per listed cell: units, corner-lattice marker; at most 8 (4) work items each
    const int NC = D == 3 ? 8 : 4;
    const long long cap = nl * NC;
    char* buf = nullptr;
    const size_t o_units = 0, o_mark = (size_t)((sizeof(unsigned) * nl + 255) & ~255LL);
    const size_t o_cell = o_mark + (size_t)((nl + 255) & ~255LL);
    const size_t o_cor = o_cell + (size_t)((sizeof(int) * cap + 255) & ~255LL);
    const size_t bytes = o_cor + sizeof(double) * NC * cap;
    if ((e = cudaMalloc(&buf, bytes)) != cudaSuccess) return e;
    unsigned* units = reinterpret_cast<unsigned*>(buf + o_units);
    signed char* mark = reinterpret_cast<signed char*>(buf + o_mark);
    int* item_cell = reinterpret_cast<int*>(buf + o_cell);
    double* item_cor = reinterpret_cast<double*>(buf + o_cor);
    const long long nbc = (nl * 8 + 255) / 256;
    if (D == 3)
      k_vm_cut<3><<<(unsigned)nbc, 256, 0, s>>>(L, list, nl, tab, cvol, carea, units, mark, item_cell, item_cor,
                                                cnt + 2);
    else
      k_vm_cut<2><<<(unsigned)nbc, 256, 0, s>>>(L, list, nl, tab, cvol, carea, units, mark, item_cell, item_cor,
                                                cnt + 2);
    unsigned long long ni = 0;
    if ((e = cudaMemcpyAsync(&ni, cnt + 2, sizeof(ni), cudaMemcpyDeviceToHost, s)) == cudaSuccess &&
        (e = cudaStreamSynchronize(s)) == cudaSuccess) {
      if (ni > 0) {
        const long long nbi = ((long long)ni + 3) / 4;  // one warp per cut sub-cube
        if (D == 3) k_vm_walk<3><<<(unsigned)nbi, 128, 0, s>>>(item_cell, item_cor, (long long)ni, units);
        else k_vm_walk<2><<<(unsigned)nbi, 128, 0, s>>>(item_cell, item_cor, (long long)ni, units);
      }
      k_vm_finish<<<(unsigned)((nl + 255) / 256), 256, 0, s>>>(list, nl, units, mark, dv, cvol);
      e = cudaStreamSynchronize(s);
    }
    cudaError_t e2 = cudaFree(buf);
    if (e != cudaSuccess) return e;
    if (e2 != cudaSuccess) return e2;
  }
  if (D == 3) k_vm_reduce<3><<<(unsigned)nb, 256, 0, s>>>(ls, level, nin, dl, cvol, carea, part);
  else k_vm_reduce<2><<<(unsigned)nb, 256, 0, s>>>(ls, level, nin, dl, cvol, carea, part);
  k_vm_final<<<1, 256, 0, s>>>(part, nb, tot);
  return cudaGetLastError();
}

// Builds one level in place: g64 (phi, n), c64, tag, and its float copies.
// max_phi_bits[0] accumulates the maximum positive interior phi, [1] and [2]
// the maximum and minimum |curvature| of CUT cells (FP64 bit patterns).
// ---------------------------------------------------------------- characteristic cells
// Levelset_package::Get_singularity_tag (lset_package.cpp:515-556) and
// Get_segment_tag (:560-590) with is_Segment_intersec_AABB (:594-619), after
// the interface tags, in FP64 without contraction (this file is compiled with
// -fmad=false), in the reference's operation order.  A singularity tags, in
// every interior package whose half-open box holds it (0 < x - corner <
// dpkg + 1e-10 per axis), the interface cell (tag != NORMAL) nearest to it by
// cell centre, equal distances going to the first cell in (x, y, z) loop
// order; the singularities run in order on one thread, so a later one
// overwrites an earlier one's cell.  A segment tags every other interface
// cell whose box it meets, the first segment in order winning.
__device__ inline bool segment_meets_box(const double* p1, const double* p2, const double* mn, const double* mx) {
  const double EPSILON = 1.e-20;
  double d[3], e[3], cc[3], ad[3];
  for (int k = 0; k < 3; k++) {
    d[k] = (p2[k] - p1[k]) * 0.5;
    e[k] = (mx[k] - mn[k]) * 0.5;
    cc[k] = (p1[k] + d[k]) - (mx[k] + mn[k]) * 0.5;
    ad[k] = fabs(d[k]);
  }
  for (int k = 0; k < 3; k++)
    if (fabs(cc[k]) > e[k] + ad[k]) return false;
  if (fabs(d[1] * cc[2] - d[2] * cc[1]) > e[1] * ad[2] + e[2] * ad[1] + EPSILON) return false;
  if (fabs(d[2] * cc[0] - d[0] * cc[2]) > e[2] * ad[0] + e[0] * ad[2] + EPSILON) return false;
  if (fabs(d[0] * cc[1] - d[1] * cc[0]) > e[0] * ad[1] + e[1] * ad[0] + EPSILON) return false;
  return true;
}

__global__ void k_ls_singularities(LsLevel L, int D, const uint8_t* __restrict__ tag, int* __restrict__ chr,
                                   const double* __restrict__ sing, int nsing) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  for (int ic = 0; ic < nsing; ic++) {
    const double* p = sing + 3 * ic;
    int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    for (int d = 0; d < D; d++) {
      const int q = (int)floor((p[d] - L.box_l[d]) / L.dpkg[d]);
      lo[d] = max(0, q - 1);
      hi[d] = min(L.num_pkg[d] - 1, q + 1);
    }
    for (int pi = lo[0]; pi <= hi[0]; pi++)
      for (int pj = lo[1]; pj <= hi[1]; pj++)
        for (int pk_ = lo[2]; pk_ <= hi[2]; pk_++) {
          const int pk[3] = {pi, pj, pk_};
          bool inside = true;
          for (int d = 0; d < D; d++) {
            const double corner = pk[d] * L.dpkg[d] + L.box_l[d];
            const double dr = p[d] - corner;
            inside = inside && dr < L.dpkg[d] + 1.e-10 && dr > 0.;
          }
          if (!inside) continue;
          double best = 0.0;
          long long besta = -1;
          for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++)
              for (int k = 0; k < (D == 3 ? 4 : 1); k++) {
                const int ce[3] = {i, j, k};
                const long long a = ls_index(L, D, 4 * pk[0] + i, 4 * pk[1] + j, D == 3 ? 4 * pk[2] + k : 0);
                if (tag[a] == 0) continue;
                double dist = 0.0;
                for (int d = 0; d < D; d++) {
                  const double cp = (pk[d] * L.dpkg[d] + (ce[d] + 0.5) * L.dcell[d]) + L.box_l[d];
                  dist += (cp - p[d]) * (cp - p[d]);
                }
                dist = sqrt(dist);
                if (besta < 0 || dist < best) { best = dist; besta = a; }
              }
          if (besta >= 0) chr[besta] = -(ic + 1);
        }
  }
}

__global__ void k_ls_segments(LsLevel L, int D, const uint8_t* __restrict__ tag, int* __restrict__ chr,
                              const double* __restrict__ seg, int nseg) {
  const long long ni[3] = {4ll * L.num_pkg[0], 4ll * L.num_pkg[1], D == 3 ? 4ll * L.num_pkg[2] : 1};
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ni[0] * ni[1] * ni[2]) return;
  const int g[3] = {(int)(t % ni[0]), (int)((t / ni[0]) % ni[1]), (int)(t / (ni[0] * ni[1]))};
  const long long a = ls_index(L, D, g[0], g[1], g[2]);
  if (tag[a] == 0 || chr[a] < 0) return;
  double mn[3] = {0, 0, 0}, mx[3] = {0, 0, 0};
  for (int d = 0; d < D; d++) {
    const int pk = g[d] >> 2, ce = g[d] & 3;
    mn[d] = (pk * L.dpkg[d] + ce * L.dcell[d]) + L.box_l[d];
    mx[d] = mn[d] + L.dcell[d];
  }
  for (int is = 0; is < nseg; is++)
    if (segment_meets_box(seg + 6 * is, seg + 6 * is + 3, mn, mx)) {
      chr[a] = is + 1;
      return;
    }
}

cudaError_t ls_build_characteristics(const LsLevel& L, int D, long long ntot, int* chr, const double* d_sing,
                                     int nsing, const double* d_seg, int nseg, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(chr, 0, sizeof(int) * ntot, s);
  if (e != cudaSuccess) return e;
  if (nsing > 0) k_ls_singularities<<<1, 1, 0, s>>>(L, D, L.tag, chr, d_sing, nsing);
  const long long ncell = 4ll * L.num_pkg[0] * 4ll * L.num_pkg[1] * (D == 3 ? 4ll * L.num_pkg[2] : 1);
  if (nseg > 0) k_ls_segments<<<(unsigned)((ncell + 255) / 256), 256, 0, s>>>(L, D, L.tag, chr, d_seg, nseg);
  return cudaGetLastError();
}

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
