// mrsph_tri.cu — 2D neighbour-graph triangulation and mesh quality (row A14).
//
//   Voronoi_construction::Local_VD_generation (voronoi_construction.cpp:6-127)
//     -> k_tri_mark / k_tri_mark_exact: j is an edge of i when j is a Voronoi
//        neighbour of i among i's neighbour set (voro++ replaced by exact
//        orient2d / incircle signs: FP64 filter, then expansion arithmetic)
//   Graphmeshcls::Reconstruct_tris (graph_mesh.cpp:37-409)
//     -> k_tri_pass1 (3-cycles i > j > k, longest-edge deletion for all-boundary
//        triangles whose centroid phi <= 1e-4 of the vertex mean), k_tri_alive
//        (rebuild from the kept triangles), k_tri_count / k_tri_fill (final
//        3-cycles, non-manifold and crossing checks)
//   Tri_quality_statistics (graph_mesh.cpp:411-670) -> k_tri_quality
// Exact predicate signs make the edge set independent of evaluation order, so
// it matches the oracle exactly.  Compiled with -fmad=false.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "handle.h"

namespace mrsph {
namespace {

// ------------------------------------------------------------ expansions
__device__ inline void two_sum(double a, double b, double& x, double& y) {
  x = a + b;
  double bv = x - a, av = x - bv, br = b - bv, ar = a - av;
  y = ar + br;
}
__device__ inline void two_diff(double a, double b, double& x, double& y) {
  x = a - b;
  double bv = a - x, av = x + bv, br = bv - b, ar = a - av;
  y = ar + br;
}
__device__ inline void two_prod(double a, double b, double& x, double& y) {
  x = a * b;
  y = fma(a, b, -x);
}
__device__ int xgrow(const double* e, int m, double b, double* h) {
  double Q = b;
  int k = 0;
  for (int i = 0; i < m; i++) {
    double Qn, hh;
    two_sum(Q, e[i], Qn, hh);
    Q = Qn;
    if (hh != 0.0) h[k++] = hh;
  }
  if (Q != 0.0 || k == 0) h[k++] = Q;
  return k;
}
__device__ int xscale(const double* e, int m, double b, double* h) {
  double Q, hh;
  int k = 0;
  two_prod(e[0], b, Q, hh);
  if (hh != 0.0) h[k++] = hh;
  for (int i = 1; i < m; i++) {
    double T, t, Q2, s;
    two_prod(e[i], b, T, t);
    two_sum(Q, t, Q2, s);
    if (s != 0.0) h[k++] = s;
    double x = T + Q2, bv = x - T;
    s = Q2 - bv;
    Q = x;
    if (s != 0.0) h[k++] = s;
  }
  if (Q != 0.0 || k == 0) h[k++] = Q;
  return k;
}
constexpr int XCAP = 256;
// acc += sign * p*q*r*s exactly; returns false when the accumulator would overflow
__device__ bool xacc4(double* acc, int* n, double* tmp, double p, double q, double r, double s, double sign) {
  double e[8], f[8];
  two_prod(p, q, e[1], e[0]);
  int m = xscale(e, 2, r, f);
  m = xscale(f, m, s * sign, e);
  for (int i = 0; i < m; i++) {
    if (*n + 1 > XCAP) return false;
    int l = xgrow(acc, *n, e[i], tmp);
    for (int t = 0; t < l; t++) acc[t] = tmp[t];
    *n = l;
  }
  return true;
}
__device__ int xsign(const double* e, int n) {
  for (int i = n - 1; i >= 0; i--)
    if (e[i] != 0.0) return e[i] > 0 ? 1 : -1;
  return 0;
}

// ------------------------------------------------------------ predicates
// Filtered: returns 2 when the FP64 sign is not certain.
__device__ int orient_f(const double* a, const double* b, const double* c) {
  double acx = a[0] - c[0], bcx = b[0] - c[0], acy = a[1] - c[1], bcy = b[1] - c[1];
  double l = acx * bcy, r = acy * bcx;
  double det = l - r;
  double bound = 1.0e-15 * (fabs(l) + fabs(r));
  if (det > bound) return 1;
  if (-det > bound) return -1;
  return 2;
}
__device__ int incircle_f(const double* a, const double* b, const double* c, const double* d) {
  double adx = a[0] - d[0], ady = a[1] - d[1], bdx = b[0] - d[0], bdy = b[1] - d[1];
  double cdx = c[0] - d[0], cdy = c[1] - d[1];
  double al = adx * adx + ady * ady, bl = bdx * bdx + bdy * bdy, cl = cdx * cdx + cdy * cdy;
  double t1 = bdx * cdy, t2 = cdx * bdy, t3 = cdx * ady, t4 = adx * cdy, t5 = adx * bdy, t6 = bdx * ady;
  double det = al * (t1 - t2) + bl * (t3 - t4) + cl * (t5 - t6);
  double perm = (fabs(t1) + fabs(t2)) * al + (fabs(t3) + fabs(t4)) * bl + (fabs(t5) + fabs(t6)) * cl;
  double bound = 2.0e-14 * perm;
  if (det > bound) return 1;
  if (-det > bound) return -1;
  return 2;
}
// Exact signs (expansion arithmetic); *ok = false on accumulator overflow.
__device__ int orient_x(const double* a, const double* b, const double* c, double* acc, double* tmp, bool* ok) {
  int f = orient_f(a, b, c);
  if (f != 2) return f;
  double ax[2], ay[2], bx[2], by[2];
  two_diff(a[0], c[0], ax[1], ax[0]);
  two_diff(a[1], c[1], ay[1], ay[0]);
  two_diff(b[0], c[0], bx[1], bx[0]);
  two_diff(b[1], c[1], by[1], by[0]);
  int n = 0;
  for (int u = 0; u < 2; u++)
    for (int v = 0; v < 2; v++) {
      *ok = *ok && xacc4(acc, &n, tmp, ax[u], by[v], 1.0, 1.0, 1.0);
      *ok = *ok && xacc4(acc, &n, tmp, ay[u], bx[v], 1.0, 1.0, -1.0);
    }
  return xsign(acc, n);
}
__device__ int incircle_x(const double* a, const double* b, const double* c, const double* d, double* acc,
                          double* tmp, bool* ok) {
  int f = incircle_f(a, b, c, d);
  if (f != 2) return f;
  double X[3][2], Y[3][2];
  const double* P[3] = {a, b, c};
  for (int q = 0; q < 3; q++) {
    two_diff(P[q][0], d[0], X[q][1], X[q][0]);
    two_diff(P[q][1], d[1], Y[q][1], Y[q][0]);
  }
  int n = 0;
  for (int q = 0; q < 3; q++) {
    int r = (q + 1) % 3, s = (q + 2) % 3;
    for (int u = 0; u < 2; u++)
      for (int v = 0; v < 2; v++)
        for (int w = 0; w < 2; w++)
          for (int z = 0; z < 2; z++) {
            *ok = *ok && xacc4(acc, &n, tmp, X[q][u], X[q][v], X[r][w], Y[s][z], 1.0);
            *ok = *ok && xacc4(acc, &n, tmp, Y[q][u], Y[q][v], X[r][w], Y[s][z], 1.0);
            *ok = *ok && xacc4(acc, &n, tmp, X[q][u], X[q][v], X[s][w], Y[r][z], -1.0);
            *ok = *ok && xacc4(acc, &n, tmp, Y[q][u], Y[q][v], X[s][w], Y[r][z], -1.0);
          }
  }
  return xsign(acc, n);
}

// Local Delaunay test of edge (i, j) among row S.  EXACT = false returns 2
// as soon as a filtered sign is uncertain.
template <bool EXACT>
__device__ int local_delaunay(const double* xyz, int i, int j, const int* S, int ns, double* acc, double* tmp,
                              bool* ok) {
  const double pi[2] = {xyz[3 * (long long)i], xyz[3 * (long long)i + 1]};
  const double pj[2] = {xyz[3 * (long long)j], xyz[3 * (long long)j + 1]};
  int lstar = -1, rstar = -1;
  double pl[2] = {0, 0}, pr[2] = {0, 0};
  for (int q = 0; q < ns; q++) {
    int k = S[q];
    if (k == i || k == j) continue;
    const double pk[2] = {xyz[3 * (long long)k], xyz[3 * (long long)k + 1]};
    int o = EXACT ? orient_x(pi, pj, pk, acc, tmp, ok) : orient_f(pi, pj, pk);
    if (o == 2) return 2;
    if (o == 0) {
      double t = (pk[0] - pi[0]) * (pj[0] - pi[0]) + (pk[1] - pi[1]) * (pj[1] - pi[1]);
      double L = (pj[0] - pi[0]) * (pj[0] - pi[0]) + (pj[1] - pi[1]) * (pj[1] - pi[1]);
      if (t > 0 && t < L) return 0;
      continue;
    }
    if (o > 0) {
      int c = 1;
      if (lstar >= 0) {
        c = EXACT ? incircle_x(pi, pj, pl, pk, acc, tmp, ok) : incircle_f(pi, pj, pl, pk);
        if (c == 2) return 2;
      }
      if (lstar < 0 || c > 0) { lstar = k; pl[0] = pk[0]; pl[1] = pk[1]; }
    } else {
      int c = 1;
      if (rstar >= 0) {
        c = EXACT ? incircle_x(pj, pi, pr, pk, acc, tmp, ok) : incircle_f(pj, pi, pr, pk);
        if (c == 2) return 2;
      }
      if (rstar < 0 || c > 0) { rstar = k; pr[0] = pk[0]; pr[1] = pk[1]; }
    }
  }
  if (lstar < 0 || rstar < 0) return 1;
  int c = EXACT ? incircle_x(pi, pj, pl, pr, acc, tmp, ok) : incircle_f(pi, pj, pl, pr);
  if (c == 2) return 2;
  return c < 0 ? 1 : 0;
}

struct TriIn {
  long long n;
  int cap;
  const double* xyz;
  const int* type;
  const double* phi;
  const int* rows;  // n x cap, sorted ids incl. self
  const int* cnt;
};

__device__ inline int row_find(const TriIn& T, int a, int b) {
  const int* S = T.rows + (long long)a * T.cap;
  int lo = 0, hi = T.cnt[a] - 1;
  while (lo <= hi) {
    int m = (lo + hi) >> 1;
    int v = S[m];
    if (v == b) return m;
    if (v < b) lo = m + 1; else hi = m - 1;
  }
  return -1;
}

// mark[i*cap+q]: 1 edge, 0 none, 2 undecided by the FP64 filter
__global__ void k_tri_mark(TriIn T, unsigned char* mark) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T.n * T.cap) return;
  int i = (int)(t / T.cap), q = (int)(t % T.cap);
  if (q >= T.cnt[i]) return;
  const int* S = T.rows + (long long)i * T.cap;
  int j = S[q];
  if (j == i) { mark[t] = 0; return; }
  bool ok = true;
  mark[t] = (unsigned char)local_delaunay<false>(T.xyz, i, j, S, T.cnt[i], nullptr, nullptr, &ok);
}

// Exact test of every undecided slot (grid-stride over all slots).
// scratch: 2 * XCAP doubles per thread of the launch.
__global__ void __launch_bounds__(64) k_tri_mark_exact(TriIn T, unsigned char* mark, unsigned* flags,
                                                         double* scratch) {
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double* acc = scratch + tid * (2 * XCAP);
  double* tmp = acc + XCAP;
  const long long NC = T.n * T.cap;
  for (long long t = tid; t < NC; t += (long long)gridDim.x * blockDim.x) {
    if (mark[t] != 2) continue;
    int i = (int)(t / T.cap), q = (int)(t % T.cap);
    const int* S = T.rows + (long long)i * T.cap;
    bool ok = true;
    int r = local_delaunay<true>(T.xyz, i, S[q], S, T.cnt[i], acc, tmp, &ok);
    if (!ok) atomicOr(flags, 2u);
    mark[t] = (unsigned char)(r == 1 ? 1 : 0);
  }
}

// adj[i*cap+q] = edge(i, S[q]) in either direction
__global__ void k_tri_adj(TriIn T, const unsigned char* mark, unsigned char* adj) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T.n * T.cap) return;
  int i = (int)(t / T.cap), q = (int)(t % T.cap);
  if (q >= T.cnt[i]) return;
  int j = T.rows[t];
  unsigned char e = 0;
  if (j != i) {
    e = mark[t];
    if (!e) {
      int p = row_find(T, j, i);
      if (p >= 0) e = mark[(long long)j * T.cap + p];
    }
  }
  adj[t] = e;
}

__device__ inline bool is_adj(const TriIn& T, const unsigned char* adj, int a, int b) {
  int p = row_find(T, a, b);
  return p >= 0 && adj[(long long)a * T.cap + p];
}

// deletion rule of Reconstruct_tris (graph_mesh.cpp:144-205); returns true when kept,
// else *ea/*eb = longest edge
__device__ bool tri_rule(const TriIn& T, const LsSet& ls, int I, int j, int k, int* ea, int* eb) {
  if (T.type[I] == REAL_P || T.type[j] == REAL_P || T.type[k] == REAL_P) return true;
  const double* p1 = T.xyz + 3 * (long long)I;
  const double* p2 = T.xyz + 3 * (long long)j;
  const double* p3 = T.xyz + 3 * (long long)k;
  double cen[3] = {1. / 3. * (p1[0] + p2[0] + p3[0]), 1. / 3. * (p1[1] + p2[1] + p3[1]),
                   1. / 3. * (p1[2] + p2[2] + p3[2])};
  double pc, nn[3], cv;
  ls_sample<2, double>(ls, cen, pc, nn, cv);
  double phi_size = 1. / 3. * (T.phi[I] + T.phi[j] + T.phi[k]);
  if (pc > 0.0001 * phi_size) return true;
  double v1[2] = {p2[0] - p1[0], p2[1] - p1[1]};
  double v2[2] = {p3[0] - p2[0], p3[1] - p2[1]};
  double v3[2] = {p1[0] - p3[0], p1[1] - p3[1]};
  double d = sqrt(v1[0] * v1[0] + v1[1] * v1[1]);
  *ea = I; *eb = j;
  double d2 = sqrt(v2[0] * v2[0] + v2[1] * v2[1]);
  if (d2 > d) { d = d2; *ea = j; *eb = k; }
  double d3 = sqrt(v3[0] * v3[0] + v3[1] * v3[1]);
  if (d3 > d) { d = d3; *ea = I; *eb = k; }
  return false;
}

__device__ inline void set_flag(const TriIn& T, unsigned* fl, int a, int b) {
  int p = row_find(T, a, b);
  if (p >= 0) atomicOr(&fl[(long long)a * T.cap + p], 1u);
  p = row_find(T, b, a);
  if (p >= 0) atomicOr(&fl[(long long)b * T.cap + p], 1u);
}

// pass 1a: deleted edges
__global__ void k_tri_pass1(TriIn T, LsSet ls, const unsigned char* adj, unsigned* del) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= T.n) return;
  const int* S = T.rows + i * T.cap;
  const unsigned char* A = adj + i * T.cap;
  const int c = T.cnt[i];
  for (int a = 0; a < c; a++) {
    int j = S[a];
    if (j >= i) break;
    if (!A[a]) continue;
    for (int b = 0; b < a; b++) {
      int k = S[b];
      if (!A[b] || !is_adj(T, adj, j, k)) continue;
      int ea, eb;
      if (!tri_rule(T, ls, (int)i, j, k, &ea, &eb)) set_flag(T, del, ea, eb);
    }
  }
}

// pass 1b: edges of kept triangles without a deleted edge are alive
__global__ void k_tri_alive(TriIn T, LsSet ls, const unsigned char* adj, const unsigned* del, unsigned* alive) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= T.n) return;
  const int* S = T.rows + i * T.cap;
  const unsigned char* A = adj + i * T.cap;
  const int c = T.cnt[i];
  for (int a = 0; a < c; a++) {
    int j = S[a];
    if (j >= i) break;
    if (!A[a]) continue;
    for (int b = 0; b < a; b++) {
      int k = S[b];
      if (!A[b]) continue;
      int pjk = row_find(T, j, k);
      if (pjk < 0 || !adj[(long long)j * T.cap + pjk]) continue;
      int ea, eb;
      if (!tri_rule(T, ls, (int)i, j, k, &ea, &eb)) continue;
      if (del[i * T.cap + a] || del[i * T.cap + b] || del[(long long)j * T.cap + pjk]) continue;
      set_flag(T, alive, (int)i, j);
      set_flag(T, alive, (int)i, k);
      set_flag(T, alive, j, k);
    }
  }
}

__device__ inline bool is_alive(const TriIn& T, const unsigned* alive, int a, int b) {
  int p = row_find(T, a, b);
  return p >= 0 && alive[(long long)a * T.cap + p];
}

// pass 2: final triangles (count or fill) and edge checks (graph_mesh.cpp:300-365)
template <bool FILL>
__global__ void k_tri_pass2(TriIn T, const unsigned* alive, int* count, const int* offset, int* tris,
                            unsigned long long* stats) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long nerr = 0, nedge = 0, nedge_first = 0;
  if (i < T.n) {
    const int* S = T.rows + i * T.cap;
    const unsigned* A = alive + i * T.cap;
    const int c = T.cnt[i];
    int ntri = 0;
    int base = FILL ? offset[i] : 0;
    for (int a = 0; a < c; a++) {
      int j = S[a];
      if (j >= i) break;
      if (!A[a]) continue;
      nedge++;
      int common = 0, c0 = -1, c1 = -1;
      for (int b = 0; b < c; b++) {
        int k = S[b];
        if (k == j || k == (int)i || !A[b]) continue;
        if (!is_alive(T, alive, j, k)) continue;
        if (common == 0) c0 = k; else if (common == 1) c1 = k;
        common++;
        if (k < j) {
          if (FILL) {
            int* o = tris + 3 * (long long)(base + ntri);
            o[0] = (int)i; o[1] = j; o[2] = k;
          }
          ntri++;
        }
      }
      if (common > 2 || (common == 2 && is_alive(T, alive, c0, c1))) nerr++;
    }
    if (!FILL) count[i] = ntri;
  }
  if (!FILL && stats) {
    for (int o = 16; o > 0; o >>= 1) {
      nerr += __shfl_xor_sync(0xffffffffu, nerr, o);
      nedge += __shfl_xor_sync(0xffffffffu, nedge, o);
    }
    if ((threadIdx.x & 31) == 0) {
      if (nerr) atomicAdd(&stats[0], nerr);
      if (nedge) atomicAdd(&stats[1], nedge);
    }
  }
  (void)nedge_first;
}

__global__ void k_tri_count_first(TriIn T, const unsigned char* adj, const unsigned* del,
                                  unsigned long long* stats) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long e1 = 0, nd = 0;
  if (i < T.n) {
    const int* S = T.rows + i * T.cap;
    for (int a = 0; a < T.cnt[i]; a++) {
      int j = S[a];
      if (j <= i) continue;
      if (adj[i * T.cap + a]) e1++;
      if (del[i * T.cap + a]) nd++;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    e1 += __shfl_xor_sync(0xffffffffu, e1, o);
    nd += __shfl_xor_sync(0xffffffffu, nd, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (e1) atomicAdd(&stats[2], e1);
    if (nd) atomicAdd(&stats[3], nd);
  }
}

// per-triangle quality terms (graph_mesh.cpp:445-520)
struct TriStat {
  double max_angle, min_angle, max_aspect, max_edge, min_edge, max_area, min_area, G_min;
  double sum_G, sum_minangle, sum_area;
  unsigned long long theta30;
};

__global__ void k_tri_quality(const double* __restrict__ xyz, long long ntri, const int* __restrict__ tris,
                              TriStat* part, unsigned long long* hist) {
  __shared__ TriStat sh[256];
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  TriStat s;
  s.max_angle = 0.; s.min_angle = 1.e15; s.max_aspect = 0.; s.max_edge = 0.; s.min_edge = 1.e15;
  s.max_area = 0.; s.min_area = 1.e15; s.G_min = 1.e20; s.sum_G = 0.; s.sum_minangle = 0.; s.sum_area = 0.;
  s.theta30 = 0;
  if (t < ntri) {
    const double rad = 180. / acos(-1.);
    const double* v0 = xyz + 3 * (long long)tris[3 * t];
    const double* v1 = xyz + 3 * (long long)tris[3 * t + 1];
    const double* v2 = xyz + 3 * (long long)tris[3 * t + 2];
    double a1[2] = {v1[0] - v0[0], v1[1] - v0[1]}, a2[2] = {v2[0] - v1[0], v2[1] - v1[1]},
           a3[2] = {v0[0] - v2[0], v0[1] - v2[1]};
    double d1 = sqrt(a1[0] * a1[0] + a1[1] * a1[1]);
    double d2 = sqrt(a2[0] * a2[0] + a2[1] * a2[1]);
    double d3 = sqrt(a3[0] * a3[0] + a3[1] * a3[1]);
    double dmax = fmax(d1, fmax(d2, d3)), dmin = fmin(d1, fmin(d2, d3));
    s.max_edge = dmax;
    s.min_edge = dmin;
    s.max_aspect = dmax / (dmin + 1.e-20);
    double c13 = -(a1[0] * a3[0] + a1[1] * a3[1]) / (d3 * d1 + 1.e-20);
    double al1 = rad * acos(c13);
    double al2 = rad * acos(-(a1[0] * a2[0] + a1[1] * a2[1]) / (d2 * d1 + 1.e-20));
    double al3 = rad * acos(-(a2[0] * a3[0] + a2[1] * a3[1]) / (d3 * d2 + 1.e-20));
    al1 = fmax(0., fmin(al1, 180.));
    al2 = fmax(0., fmin(al2, 180.));
    al3 = fmax(0., fmin(al3, 180.));
    s.max_angle = fmax(al1, fmax(al2, al3));
    double mm = fmin(al1, fmin(al2, al3));
    s.min_angle = mm;
    atomicAdd(&hist[min(44, (int)(al1 / 4.0))], 1ull);
    atomicAdd(&hist[min(44, (int)(al2 / 4.0))], 1ull);
    atomicAdd(&hist[min(44, (int)(al3 / 4.0))], 1ull);
    s.theta30 = mm < 30. ? 1 : 0;
    s.sum_minangle = mm;
    double area = 0.5 * (d3 * d1) * sin(acos(c13));
    s.sum_area = area;
    s.max_area = area;
    s.min_area = area;
    double G = 2. * sqrt(3.) * area / (dmax * (d1 + d2 + d3) / 2.);
    s.G_min = G;
    s.sum_G = G;
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {  // fixed-order block fold
    TriStat r = sh[0];
    for (int k = 1; k < blockDim.x; k++) {
      const TriStat& q = sh[k];
      r.max_angle = fmax(r.max_angle, q.max_angle);
      r.min_angle = fmin(r.min_angle, q.min_angle);
      r.max_aspect = fmax(r.max_aspect, q.max_aspect);
      r.max_edge = fmax(r.max_edge, q.max_edge);
      r.min_edge = fmin(r.min_edge, q.min_edge);
      r.max_area = fmax(r.max_area, q.max_area);
      r.min_area = fmin(r.min_area, q.min_area);
      r.G_min = fmin(r.G_min, q.G_min);
      r.sum_G += q.sum_G;
      r.sum_minangle += q.sum_minangle;
      r.sum_area += q.sum_area;
      r.theta30 += q.theta30;
    }
    part[blockIdx.x] = r;
  }
}

__global__ void k_tri_quality_fold(const TriStat* part, int nblk, TriStat* out) {
  TriStat r = part[0];
  for (int k = 1; k < nblk; k++) {
    const TriStat& q = part[k];
    r.max_angle = fmax(r.max_angle, q.max_angle);
    r.min_angle = fmin(r.min_angle, q.min_angle);
    r.max_aspect = fmax(r.max_aspect, q.max_aspect);
    r.max_edge = fmax(r.max_edge, q.max_edge);
    r.min_edge = fmin(r.min_edge, q.min_edge);
    r.max_area = fmax(r.max_area, q.max_area);
    r.min_area = fmin(r.min_area, q.min_area);
    r.G_min = fmin(r.G_min, q.G_min);
    r.sum_G += q.sum_G;
    r.sum_minangle += q.sum_minangle;
    r.sum_area += q.sum_area;
    r.theta30 += q.theta30;
  }
  *out = r;
}

int tfail(mrsph_handle* h, int code, const std::string& msg) {
  h->err = msg;
  return code;
}

}  // namespace
}  // namespace mrsph

using namespace mrsph;

extern "C" int mrsph_triangulate(mrsph_handle* h, int* tris, long long cap, long long* ntri_out,
                                 mrsph_tri_quality* q) {
  if (!h) return MRSPH_ERR_ARG;
  if (!h->eng) return tfail(h, MRSPH_ERR_STATE, "mrsph_set_levelset must come first");
  if (h->prm.dim != 2) return tfail(h, MRSPH_ERR_ARG, "triangulation is 2D only");
  if (cudaSetDevice(h->prm.device) != cudaSuccess) return tfail(h, MRSPH_ERR_CUDA, "cudaSetDevice failed");
  const long long n = h->eng->num_particles();
  if (n <= 0) return tfail(h, MRSPH_ERR_STATE, "no particles");
  const int rowcap = h->eng->neighbor_capacity();
  cudaStream_t s = h->stream;
  std::vector<void*> mem;
  int rc = 0;
  auto A = [&](void** p, size_t bytes) -> bool {
    if (cudaMalloc(p, bytes) != cudaSuccess) return false;
    mem.push_back(*p);
    return true;
  };
  double *d_xyz = nullptr, *d_phi = nullptr;
  int *d_type = nullptr, *d_rows = nullptr, *d_cnt = nullptr, *d_count = nullptr, *d_off = nullptr;
  int *d_blk = nullptr, *d_tris = nullptr;
  unsigned char *d_mark = nullptr, *d_adj = nullptr;
  unsigned *d_del = nullptr, *d_alive = nullptr, *d_flags = nullptr;
  unsigned long long *d_stats = nullptr, *d_hist = nullptr;
  TriStat *d_part = nullptr, *d_tq = nullptr;
  double* d_scratch = nullptr;
  const int XB = 152 * 4, XT = 64;  // exact-predicate launch: four blocks per SM
  const size_t NC = (size_t)n * rowcap;
  long long ntri = 0;
  unsigned flags = 0;
  unsigned long long st[4] = {0, 0, 0, 0}, hist[45];
  TriStat tq;
  std::memset(&tq, 0, sizeof(tq));
  if (!A((void**)&d_xyz, sizeof(double) * 3 * n) || !A((void**)&d_phi, sizeof(double) * n) ||
      !A((void**)&d_type, sizeof(int) * n) || !A((void**)&d_rows, sizeof(int) * NC) ||
      !A((void**)&d_cnt, sizeof(int) * n) || !A((void**)&d_count, sizeof(int) * (n + 1)) ||
      !A((void**)&d_off, sizeof(int) * (n + 1)) || !A((void**)&d_blk, sizeof(int) * scan_blocksums_size(n)) ||
      !A((void**)&d_mark, NC) || !A((void**)&d_adj, NC) || !A((void**)&d_del, sizeof(unsigned) * NC) ||
      !A((void**)&d_alive, sizeof(unsigned) * NC) || !A((void**)&d_flags, sizeof(unsigned)) ||
      !A((void**)&d_stats, sizeof(unsigned long long) * 4) ||
      !A((void**)&d_hist, sizeof(unsigned long long) * 45) ||
      !A((void**)&d_scratch, sizeof(double) * 2 * XCAP * XB * XT)) {
    rc = tfail(h, MRSPH_ERR_OOM, "cudaMalloc failed");
    goto done;
  }
  cudaMemsetAsync(d_flags, 0, sizeof(unsigned), s);
  rc = h->eng->export_tri(d_xyz, d_type, d_phi, d_rows, d_cnt, rowcap, d_flags);
  if (rc) { h->err = h->eng->err; goto done; }
  cudaMemsetAsync(d_mark, 0, NC, s);
  cudaMemsetAsync(d_adj, 0, NC, s);
  cudaMemsetAsync(d_del, 0, sizeof(unsigned) * NC, s);
  cudaMemsetAsync(d_alive, 0, sizeof(unsigned) * NC, s);
  cudaMemsetAsync(d_stats, 0, sizeof(unsigned long long) * 4, s);
  cudaMemsetAsync(d_hist, 0, sizeof(unsigned long long) * 45, s);
  {
    TriIn T;
    T.n = n; T.cap = rowcap; T.xyz = d_xyz; T.type = d_type; T.phi = d_phi; T.rows = d_rows; T.cnt = d_cnt;
    const int nbE = (int)((NC + 255) / 256), nbN = (int)((n + 255) / 256);
    k_tri_mark<<<nbE, 256, 0, s>>>(T, d_mark);
    k_tri_mark_exact<<<XB, XT, 0, s>>>(T, d_mark, d_flags, d_scratch);
    k_tri_adj<<<nbE, 256, 0, s>>>(T, d_mark, d_adj);
    k_tri_pass1<<<nbN, 256, 0, s>>>(T, h->ls, d_adj, d_del);
    k_tri_alive<<<nbN, 256, 0, s>>>(T, h->ls, d_adj, d_del, d_alive);
    k_tri_count_first<<<nbN, 256, 0, s>>>(T, d_adj, d_del, d_stats);
    k_tri_pass2<false><<<nbN, 256, 0, s>>>(T, d_alive, d_count, nullptr, nullptr, d_stats);
    cell_scan(d_count, d_off, d_blk, n, 0, s);
    int tot = 0;
    if (cudaMemcpyAsync(&tot, d_off + n - 1, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess) {
      rc = tfail(h, MRSPH_ERR_CUDA, "copy failed");
      goto done;
    }
    int last = 0;
    cudaMemcpyAsync(&last, d_count + n - 1, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&flags, d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) { rc = tfail(h, MRSPH_ERR_CUDA, "triangulation failed"); goto done; }
    ntri = (long long)tot + last;
    if (flags & 4u) { rc = tfail(h, MRSPH_ERR_RANGE, "neighbour list spilled; raise neighbor_cap"); goto done; }
    if (flags) { rc = tfail(h, MRSPH_ERR_DEVICE, "exact predicate accumulator overflow"); goto done; }
    if (ntri > 0) {
      if (!A((void**)&d_tris, sizeof(int) * 3 * ntri)) { rc = tfail(h, MRSPH_ERR_OOM, "cudaMalloc failed"); goto done; }
      k_tri_pass2<true><<<nbN, 256, 0, s>>>(T, d_alive, nullptr, d_off, d_tris, nullptr);
      const int nbT = (int)((ntri + 255) / 256);
      if (!A((void**)&d_part, sizeof(TriStat) * nbT) || !A((void**)&d_tq, sizeof(TriStat))) {
        rc = tfail(h, MRSPH_ERR_OOM, "cudaMalloc failed");
        goto done;
      }
      k_tri_quality<<<nbT, 256, 0, s>>>(d_xyz, ntri, d_tris, d_part, d_hist);
      k_tri_quality_fold<<<1, 1, 0, s>>>(d_part, nbT, d_tq);
      cudaMemcpyAsync(&tq, d_tq, sizeof(TriStat), cudaMemcpyDeviceToHost, s);
      if (tris && cap >= ntri)
        cudaMemcpyAsync(tris, d_tris, sizeof(int) * 3 * ntri, cudaMemcpyDeviceToHost, s);
    }
    cudaMemcpyAsync(st, d_stats, sizeof(st), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(hist, d_hist, sizeof(hist), cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) { rc = tfail(h, MRSPH_ERR_CUDA, std::string("triangulation: ") + cudaGetErrorString(e)); goto done; }
  }
  if (ntri_out) *ntri_out = ntri;
  if (q) {
    std::memset(q, 0, sizeof(*q));
    q->ntri = ntri;
    q->nedge = (long long)st[1];
    q->nedge_first = (long long)st[2];
    q->ndeleted = (long long)st[3];
    q->nerror = (long long)st[0];
    if (ntri > 0) {
      q->max_angle = tq.max_angle; q->min_angle = tq.min_angle; q->max_aspect = tq.max_aspect;
      q->max_edge = tq.max_edge; q->min_edge = tq.min_edge; q->max_area = tq.max_area; q->min_area = tq.min_area;
      q->G_min = tq.G_min;
      q->G_avg = tq.sum_G / ntri;
      q->min_angle_avg = tq.sum_minangle / ntri;
      q->theta_30 = (double)tq.theta30 / (double)ntri;
      q->total_area = tq.sum_area;
    } else {  // the statistics' initial values (graph_mesh.cpp:433-443)
      q->min_angle = 1.e15;
      q->min_edge = 1.e15;
      q->min_area = 1.e15;
      q->G_min = 1.e20;
    }
    for (int b = 0; b < 45; b++) q->hist[b] = (long long)hist[b];
  }
done:
  for (void* p : mem) cudaFree(p);
  return rc;
}
