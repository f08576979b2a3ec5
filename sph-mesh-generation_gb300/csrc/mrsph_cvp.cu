// mrsph_cvp.cu — centroidal Voronoi partitioning of the particles (row A13),
// Voronoi::Partitioning (CVP/voronoi.cpp:1376-1446) on the GPU.
//
// One iteration = six kernels:
//   k_cvp_assign    nearest VP per point, strict '<' (Get_CPU_id, voronoi.cpp:480-493)
//   k_cvp_partials  per (VP, 2048-point chunk) mass, mass centre and energy,
//                   points in order (voronoi.cpp:617-631); one block per chunk
//                   groups its points by VP first
//   k_cvp_reduce    per VP: chunk partials in order, centroid, pressure, error
//   k_cvp_planes    bisector plane of every VP pair
//   k_cvp_faces     per (VP, plane) the exact Voronoi face inside the box: the
//                   plane's polygon clipped by every other bisector half-space
//                   (replaces voro++, voronoi.cpp:724-790)
//   k_cvp_update    face pressure force, h, Update_position (voronoi.cpp:830-897),
//                   Update_position_CVT (:901-992), Check_partition_error (:1228-1262)
// The level-set partition (Voronoi_lset::Partitioning_for_initial_VP_distribution,
// voronoi_lset.cpp:824-889) adds, before the assignment, k_cvp_flags and
// k_cvp_ghosts: the ghost VPs (Ghost_VP_generation, :250-308), which take
// part in the assignment (a point nearest a ghost belongs to no VP, label -1)
// and bound the VPs' cells like walls.
// Compiled with -fmad=false: every operation rounds as written, in the same
// order as the oracle, so labels and VP positions match it bit for bit.
#include <cuda_runtime.h>

#include <cstring>
#include <vector>

#include "handle.h"

namespace mrsph {
namespace {

constexpr int CVP_CHUNK = 2048;
constexpr int CVP_MAXV = 64;
constexpr int CVP_MAX_K = 1024;

// K VPs; the points that bound their cells are the K VPs, then GM ghost
// slots (0 without a level set, else K), then the 2 D box walls: NP planes
// per VP.  Bisector planes are stored per VP for the K + GM points.
struct CvpGeo {
  int dim, K, GM, NP;
  double box_l[3], box_r[3];
};

struct CvpState {  // device-resident iteration state
  double relax, error_record, error_max, total_energy, target;
  int converged, iter;
  int nghost;  // ghosts of the current iteration (in slots K .. K + nghost - 1)
};

__device__ inline double cdot(const double* a, const double* b) {
  double s = 0.0;
  s += a[0] * b[0];
  s += a[1] * b[1];
  s += a[2] * b[2];
  return s;
}

__device__ inline double cdist(int D, const double* a, const double* b) {
  double s = 0.0;
  s += (a[0] - b[0]) * (a[0] - b[0]);
  s += (a[1] - b[1]) * (a[1] - b[1]);
  if (D == 3) s += (a[2] - b[2]) * (a[2] - b[2]);
  return sqrt(s);
}

__device__ inline double cmin(double a, double b) { return a <= b ? a : b; }
__device__ inline double cmax(double a, double b) { return a >= b ? a : b; }

__device__ int cclip(double (*v)[3], int nv, const double* n, double d, double (*o)[3]) {
  int no = 0;
  for (int a = 0; a < nv; a++) {
    int b = (a + 1) % nv;
    double sa = cdot(n, v[a]) - d, sb = cdot(n, v[b]) - d;
    if (sa <= 0.0) {
      if (no < CVP_MAXV) { o[no][0] = v[a][0]; o[no][1] = v[a][1]; o[no][2] = v[a][2]; }
      no++;
    }
    if ((sa <= 0.0) != (sb <= 0.0)) {
      double t = sa / (sa - sb);
      if (no < CVP_MAXV)
        for (int q = 0; q < 3; q++) o[no][q] = v[a][q] + (v[b][q] - v[a][q]) * t;
      no++;
    }
  }
  return no < CVP_MAXV ? no : CVP_MAXV;
}

// plane p of VP k: a bisector with point p (p < K + GM; vp holds the VPs and
// the ghost slots) or wall p - K - GM
__device__ void cplane(const CvpGeo& G, const double* vp, int k, int p, double* n, double* d) {
  if (p < G.K + G.GM) {
    const double* ck = vp + 3 * k;
    const double* cm = vp + 3 * p;
    double e[3] = {cm[0] - ck[0], cm[1] - ck[1], cm[2] - ck[2]};
    double len = sqrt(cdot(e, e));
    double mid[3] = {0.5 * (ck[0] + cm[0]), 0.5 * (ck[1] + cm[1]), 0.5 * (ck[2] + cm[2])};
    for (int q = 0; q < 3; q++) n[q] = e[q] / len;
    *d = cdot(n, mid);
  } else {
    int w = p - G.K - G.GM, ax = w / 2, hi = w % 2;
    n[0] = n[1] = n[2] = 0.0;
    n[ax] = hi ? 1.0 : -1.0;
    *d = hi ? G.box_r[ax] : -G.box_l[ax];
  }
}

// Nearest VP, strict '<' on the FP64 distance (lowest index wins a tie).  An
// FP32 pass finds the smallest FP32 distance first; only VPs within twice the
// FP32 error bound of it (1e-6 x (coordinate magnitude + distance), several
// times the bound) are then compared in FP64, in index order.  Every VP whose
// FP64 distance ties the minimum is among them, so the label is the one the
// full FP64 scan gives.  vp holds the K VPs and then st->nghost ghost VPs
// (st NULL: none); a point nearest a ghost gets label -1.
__global__ void k_cvp_assign(long long n, const double* __restrict__ xyz, int KV, const double* __restrict__ vp,
                             int D, int* __restrict__ label, const CvpState* st) {
  __shared__ double s_vp[3 * CVP_MAX_K];
  __shared__ float4 s_vf[CVP_MAX_K];
  __shared__ float s_lvp;
  const int K = KV + (st ? st->nghost : 0);
  for (int t = threadIdx.x; t < 3 * K; t += blockDim.x) s_vp[t] = vp[t];
  __syncthreads();
  for (int t = threadIdx.x; t < K; t += blockDim.x)
    s_vf[t] = make_float4((float)s_vp[3 * t], (float)s_vp[3 * t + 1], (float)s_vp[3 * t + 2], 0.f);
  if (threadIdx.x == 0) {
    double m = 0.0;
    for (int t = 0; t < 3 * K; t++) m = fmax(m, fabs(s_vp[t]));
    s_lvp = (float)m;
  }
  __syncthreads();
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double x[3] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
  const float xf[3] = {(float)x[0], (float)x[1], D == 3 ? (float)x[2] : 0.f};
  float bf = 3.4e38f, b2 = 3.4e38f;  // smallest and second smallest FP32 distance
  int bk = 0;
  for (int k = 0; k < K; k++) {
    const float4 v = s_vf[k];
    const float dx = xf[0] - v.x, dy = xf[1] - v.y, dz = D == 3 ? xf[2] - v.z : 0.f;
    const float dd = dx * dx + dy * dy + dz * dz;
    if (dd < bf) { b2 = bf; bf = dd; bk = k; }
    else if (dd < b2) b2 = dd;
  }
  const float L = fmaxf(s_lvp, fmaxf(fabsf(xf[0]), fmaxf(fabsf(xf[1]), fabsf(xf[2]))));
  const float df = sqrtf(bf);
  const float thr = df + 2.e-6f * (L + df) + 1.e-30f;
  const float T = thr * thr * 1.0001f;
  if (b2 > T) {  // no other VP within the bound: the FP64 scan would pick bk
    label[i] = bk < KV ? bk : -1;
    return;
  }
  double best = 1.e20;
  int idx = 0;
  for (int k = 0; k < K; k++) {
    const float4 v = s_vf[k];
    const float dx = xf[0] - v.x, dy = xf[1] - v.y, dz = D == 3 ? xf[2] - v.z : 0.f;
    if (dx * dx + dy * dy + dz * dz > T) continue;
    double dd = cdist(D, x, s_vp + 3 * k);
    if (dd < best) { best = dd; idx = k; }
  }
  label[i] = idx < KV ? idx : -1;
}

// VPs k > 0 that hold a point with surface mass (the reference's
// contains_cutcell, colour > 0, voronoi_lset.cpp:256-266)
__global__ void k_cvp_flags(long long n, const double* __restrict__ psurf, const int* __restrict__ label,
                            unsigned char* flag) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int l = label[i];
  if (l > 0 && psurf[i] > 0.) flag[l] = 1;
}

// One block: the VPs copied to the point array, then thread 0 makes the ghost
// VPs in VP order (Ghost_VP_generation, voronoi_lset.cpp:276-301): x - 2 phi n
// with phi and the interpolated normal at the VP, when phi >= 1e-6 there;
// the flags are cleared for the next iteration.
template <int D>
__global__ void k_cvp_ghosts(LsSet ls, int K, const double* __restrict__ vp, unsigned char* flag, double* src,
                             CvpState* st) {
  for (int t = threadIdx.x; t < 3 * K; t += blockDim.x) src[t] = vp[t];
  __syncthreads();
  if (threadIdx.x != 0) return;
  int G = 0;
  for (int k = 0; k < K; k++) {
    if (!flag[k]) continue;
    flag[k] = 0;
    double phi, nn[3], cv;
    ls_sample<D, double>(ls, vp + 3 * k, phi, nn, cv);
    if (phi >= 1.e-6) {
      double* g = src + 3 * (K + G);
      for (int q = 0; q < 3; q++) g[q] = q < D ? vp[3 * k + q] - 2. * phi * nn[q] : vp[3 * k + q];
      G++;
    }
  }
  st->nghost = G;
}

// total point mass in chunked order (Set_target_mass, voronoi.cpp:495-510)
__global__ void k_cvp_chunk_mass(long long n, const double* __restrict__ pm, long long nchunk, double* out) {
  long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nchunk) return;
  double s = 0.0;
  long long e = min(n, (c + 1) * (long long)CVP_CHUNK);
  for (long long i = c * CVP_CHUNK; i < e; i++) s += pm[i];
  out[c] = s;
}

__global__ void k_cvp_target(long long nchunk, const double* tm, int K, CvpState* st) {
  double t = 0.0;
  for (long long c = 0; c < nchunk; c++) t += tm[c];
  st->target = t / K;
}

// Per 2048-point chunk (one block): the chunk's points grouped by VP in point
// order (a stable counting sort in shared memory), then each VP's mass, mass
// centre and energy summed over its points in order, so every (VP, chunk)
// partial adds the same points in the same order as a scan of the chunk per
// VP would, in O(chunk) work instead of O(K x chunk).
__global__ void __launch_bounds__(256) k_cvp_partials(long long n, const double* __restrict__ xyz,
                                                      const double* __restrict__ pm,
                                                      const int* __restrict__ label, int K,
                                                      const double* __restrict__ vp, int D,
                                                      double* __restrict__ part) {
  __shared__ int s_lab[CVP_CHUNK];
  __shared__ short s_list[CVP_CHUNK];
  __shared__ int s_start[CVP_MAX_K + 1];
  __shared__ int s_cur[CVP_MAX_K];
  const long long c = blockIdx.x;
  const long long b = c * (long long)CVP_CHUNK;
  const int m = (int)min((long long)CVP_CHUNK, n - b);
  const int tid = threadIdx.x, lane = tid & 31;
  for (int k = tid; k < K; k += blockDim.x) s_cur[k] = 0;
  __syncthreads();
  for (int t = tid; t < m; t += blockDim.x) {
    const int l = __ldg(&label[b + t]);
    s_lab[t] = l;
    if (l >= 0) atomicAdd(&s_cur[l], 1);  // -1: nearest a ghost, no VP
  }
  __syncthreads();
  if (tid < 32) {  // exclusive scan of the counts; s_cur becomes each VP's fill cursor
    int run = 0;
    for (int k0 = 0; k0 < K; k0 += 32) {
      const int k = k0 + lane;
      const int v = k < K ? s_cur[k] : 0;
      int inc = v;
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
      }
      if (k < K) {
        s_start[k] = run + inc - v;
        s_cur[k] = run + inc - v;
      }
      run += __shfl_sync(0xffffffffu, inc, 31);
    }
    if (lane == 0) s_start[K] = run;
    __syncwarp();
    // stable fill: 32 points at a time in point order; lanes with the same VP
    // take consecutive slots in lane order
    for (int t0 = 0; t0 < m; t0 += 32) {
      const int t = t0 + lane;
      const bool ok = t < m && s_lab[t] >= 0;
      const unsigned act = __ballot_sync(0xffffffffu, ok);
      if (ok) {
        const int l = s_lab[t];
        const unsigned peers = __match_any_sync(act, l);
        const int rank = __popc(peers & ((1u << lane) - 1u));
        s_list[s_cur[l] + rank] = (short)t;
        __syncwarp(act);
        if (rank == 0) s_cur[l] += __popc(peers);
      }
      __syncwarp();
    }
  }
  __syncthreads();
  for (int k = tid; k < K; k += blockDim.x) {
    const double ck[3] = {vp[3 * k], vp[3 * k + 1], vp[3 * k + 2]};
    double ms = 0.0, x = 0.0, y = 0.0, z = 0.0, en = 0.0;
    for (int q = s_start[k]; q < s_start[k + 1]; q++) {
      const long long i = b + s_list[q];
      const double w = pm[i];
      const double p[3] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
      ms += w;
      x = x + p[0] * w;
      y = y + p[1] * w;
      z = z + p[2] * w;
      en += w * cdist(D, ck, p);
    }
    double* o = part + ((size_t)c * K + k) * 5;
    o[0] = ms; o[1] = x; o[2] = y; o[3] = z; o[4] = en;
  }
}

__global__ void k_cvp_reduce(long long nchunk, int K, int D, const double* __restrict__ part,
                             const CvpState* st, const double* __restrict__ vp, double* mass, double* mc,
                             double* energy, double* P, double* err) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K) return;
  double m = 0.0, x = 0.0, y = 0.0, z = 0.0, e = 0.0;
  for (long long c = 0; c < nchunk; c++) {
    const double* q = part + ((size_t)c * K + k) * 5;
    m += q[0]; x = x + q[1]; y = y + q[2]; z = z + q[3]; e += q[4];
  }
  mass[k] = m;
  energy[k] = e;
  double target = st->target;
  if (m > 0.) {
    double inv = 1. / m;
    mc[3 * k] = x * inv;
    mc[3 * k + 1] = y * inv;
    mc[3 * k + 2] = (D == 3) ? z * inv : 0.0;
    P[k] = target / m;
  } else {
    // a cell without points (the reference divides by its zero mass):
    // centroid = its position, no pressure; it does not move (k_cvp_update)
    for (int q = 0; q < 3; q++) mc[3 * k + q] = vp[3 * k + q];
    P[k] = 0.;
  }
  err[k] = fabs(m - target) / target;
}

// bisector planes of every (VP, point) pair, computed once per iteration
// (row stride K + GM; slots of absent ghosts are left alone)
__global__ void k_cvp_planes(CvpGeo G, const double* __restrict__ vp, double* __restrict__ planes,
                             float4* __restrict__ planes_f, const CvpState* st) {
  const int PS = G.K + G.GM;
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)G.K * PS) return;
  int k = (int)(t / PS), m = (int)(t % PS);
  if (k == m || m >= G.K + st->nghost) return;
  double n[3], d;
  cplane(G, vp, k, m, n, &d);
  double* o = planes + 4 * t;
  o[0] = n[0]; o[1] = n[1]; o[2] = n[2]; o[3] = d;
  planes_f[t] = make_float4((float)n[0], (float)n[1], (float)n[2], (float)d);
}

// bounding sphere of a polygon (centre = vertex mean)
__device__ inline void cbound(double (*v)[3], int nv, double* C, double* r) {
  C[0] = C[1] = C[2] = 0.0;
  for (int a = 0; a < nv; a++)
    for (int q = 0; q < 3; q++) C[q] += v[a][q];
  for (int q = 0; q < 3; q++) C[q] /= (double)(nv > 0 ? nv : 1);
  double r2 = 0.0;
  for (int a = 0; a < nv; a++) {
    double e[3] = {v[a][0] - C[0], v[a][1] - C[1], v[a][2] - C[2]};
    r2 = fmax(r2, cdot(e, e));
  }
  *r = sqrt(r2);
}

// face of VP k on plane p; out: exists, area, n (3), dist.  A clip whose
// plane lies beyond the polygon's bounding sphere (with a 1e-9 relative
// margin) would keep every vertex in order, so it is skipped: the result is
// the one of clipping by every plane in turn.  A bisector is first tested in
// FP32 with a margin (4e-6 of the magnitudes) far above the FP32 rounding, so
// an FP32 skip is always an FP64 skip; the others take the FP64 test.
__global__ void __launch_bounds__(128) k_cvp_faces(CvpGeo G, const double* __restrict__ vp,
                                                   const double* __restrict__ planes,
                                                   const float4* __restrict__ planes_f, double* __restrict__ face,
                                                   const CvpState* st) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)G.K * G.NP) return;
  int k = (int)(t / G.NP), p = (int)(t % G.NP);
  double* out = face + 6 * t;
  out[0] = 0.0;
  if (p < G.K && p == k) return;
  const int PS = G.K + G.GM, NPT = G.K + st->nghost;  // plane row stride, points present
  if (p >= NPT && p < PS) return;  // an unused ghost slot
  double n[3], d;
  if (p < PS) {
    const double* pl = planes + 4 * ((long long)k * PS + p);
    n[0] = pl[0]; n[1] = pl[1]; n[2] = pl[2]; d = pl[3];
  } else {
    cplane(G, vp, k, p, n, &d);
  }
  double lo[3], hi[3];
  for (int q = 0; q < 3; q++) {
    lo[q] = q < G.dim ? G.box_l[q] : -0.5;
    hi[q] = q < G.dim ? G.box_r[q] : 0.5;
  }
  double c[3] = {0.5 * (lo[0] + hi[0]), 0.5 * (lo[1] + hi[1]), 0.5 * (lo[2] + hi[2])};
  double S = 0.0;
  for (int q = 0; q < 3; q++) S += (hi[q] - lo[q]) * (hi[q] - lo[q]);
  S = 2.0 * sqrt(S);
  int ax = 0;
  if (fabs(n[1]) < fabs(n[ax])) ax = 1;
  if (fabs(n[2]) < fabs(n[ax])) ax = 2;
  double e[3] = {0, 0, 0};
  e[ax] = 1.0;
  double u[3] = {n[1] * e[2] - n[2] * e[1], n[2] * e[0] - n[0] * e[2], n[0] * e[1] - n[1] * e[0]};
  double ul = sqrt(cdot(u, u));
  for (int q = 0; q < 3; q++) u[q] = u[q] / ul;
  double w[3] = {n[1] * u[2] - n[2] * u[1], n[2] * u[0] - n[0] * u[2], n[0] * u[1] - n[1] * u[0]};
  double off = d - cdot(n, c);
  double p0[3] = {c[0] + n[0] * off, c[1] + n[1] * off, c[2] + n[2] * off};
  double BA[CVP_MAXV][3], BB[CVP_MAXV][3];
  double (*A)[3] = BA, (*B)[3] = BB;
  const double sg[4][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
  for (int a = 0; a < 4; a++)
    for (int q = 0; q < 3; q++) A[a][q] = p0[q] + u[q] * (sg[a][0] * S) + w[q] * (sg[a][1] * S);
  int nv = 4;
  double C[3], r;
  cbound(A, nv, C, &r);
  float Cf[3] = {(float)C[0], (float)C[1], (float)C[2]}, rf = (float)r;
  const float Sf = (float)S;
  auto clip = [&](const double* cn, double cd) {
    const double sc = cdot(cn, C) - cd;
    if (sc + r < -1.e-9 * (fabs(cd) + fabs(cdot(cn, C)) + r + S)) return;  // all vertices inside
    nv = cclip(A, nv, cn, cd, B);
    double (*tmp)[3] = A;
    A = B;
    B = tmp;
    cbound(A, nv, C, &r);
    Cf[0] = (float)C[0]; Cf[1] = (float)C[1]; Cf[2] = (float)C[2];
    rf = (float)r;
  };
  for (int wq = 0; wq < 6 && nv > 0; wq++) {
    if (p >= PS && wq == p - PS) continue;
    int axw = wq / 2, hw = wq % 2;
    double wn[3] = {0, 0, 0};
    wn[axw] = hw ? 1.0 : -1.0;
    double wd = hw ? hi[axw] : -lo[axw];
    clip(wn, wd);
  }
  const double* pk = planes + 4 * (long long)k * PS;
  const float4* pkf = planes_f + (long long)k * PS;
  for (int m = 0; m < NPT && nv > 0; m++) {
    if (m == k || m == p) continue;
    const float4 pf = __ldg(&pkf[m]);
    const float scf = (pf.x * Cf[0] + pf.y * Cf[1] + pf.z * Cf[2]) - pf.w;
    const float magf = fabsf(pf.w) + (fabsf(Cf[0]) + fabsf(Cf[1]) + fabsf(Cf[2])) + rf + Sf;
    if (scf + rf < -4.001e-6f * magf) continue;  // the FP64 test skips it as well
    const double bn[3] = {pk[4 * m], pk[4 * m + 1], pk[4 * m + 2]};
    clip(bn, pk[4 * m + 3]);
  }
  if (nv < 3) return;
  double ar = 0.0;
  for (int a = 1; a + 1 < nv; a++) {
    double x[3] = {A[a][0] - A[0][0], A[a][1] - A[0][1], A[a][2] - A[0][2]};
    double y[3] = {A[a + 1][0] - A[0][0], A[a + 1][1] - A[0][1], A[a + 1][2] - A[0][2]};
    double cr[3] = {x[1] * y[2] - x[2] * y[1], x[2] * y[0] - x[0] * y[2], x[0] * y[1] - x[1] * y[0]};
    ar += cdot(cr, n);
  }
  ar = 0.5 * fabs(ar);
  double ext = S * S;
  if (!(ar > 1.e-13 * ext)) return;
  const double* ck = vp + 3 * k;
  double dx[3] = {A[0][0] - ck[0], A[0][1] - ck[1], A[0][2] - ck[2]};
  out[0] = 1.0;
  out[1] = ar;
  out[2] = n[0];
  out[3] = n[1];
  out[4] = n[2];
  out[5] = fabs(cdot(dx, n)) * 2.;
}

// VP update, one block: per-VP work in parallel (thread k handles VPs
// k, k + blockDim, ...), the order-sensitive scalars (error and energy sums,
// the two global minima) on thread 0 in VP order, as the reference loops do.
__global__ void __launch_bounds__(1024) k_cvp_update(CvpGeo G, double* vp, const double* __restrict__ face,
                                                     const double* mass, const double* mc, const double* energy,
                                                     const double* P, const double* err, double* f, double* hk,
                                                     double* shift, CvpState* st, double error_tolerance,
                                                     int pressure_step) {
  __shared__ double s_ts[CVP_MAX_K];
  __shared__ double s_g;
  __shared__ int s_conv;
  const int K = G.K, D = G.dim, NP = G.NP;
  const int iter = st->iter;
  const double relax = st->relax;  // read by every thread before thread 0 updates it
  const double scale_coeff = 0.25 + 1.75 * (1. - cmin((iter - 1) / 500., 1.));
  for (int k = threadIdx.x; k < K; k += blockDim.x) {
    double fx = 0.0, fy = 0.0, fz = 0.0, sr = 0.0;
    int nnb = 0;
    for (int p = 0; p < NP; p++) {
      const double* fc = face + 6 * ((size_t)k * NP + p);
      if (fc[0] == 0.0) continue;
      nnb++;
      double nP = (p < K) ? P[p] : P[k];
      sr += fc[5];
      double pmid = 0.5 * (P[k] + nP);
      double coef = -1 * pmid * fc[1];
      fx = fx + fc[2] * coef;
      fy = fy + fc[3] * coef;
      fz = fz + fc[4] * coef;
    }
    f[3 * k] = fx; f[3 * k + 1] = fy; f[3 * k + 2] = fz;
    hk[k] = scale_coeff * sr / (double)nnb;
  }
  if (threadIdx.x == 0) {
    double error_max = 0.0, total_energy = 0.0;
    for (int k = 0; k < K; k++) {
      error_max = cmax(error_max, err[k]);
      total_energy += energy[k];
    }
    st->error_record = st->error_record + error_max;
    if (iter % 40 == 0) {
      st->error_record /= 40.;
      if (error_max <= error_tolerance && st->error_record <= error_tolerance) st->converged = 1;
      st->error_record = 0.;
    }
    st->error_max = error_max;
    st->total_energy = total_energy;
    s_conv = st->converged;
  }
  __syncthreads();
  if (s_conv == 0) {
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
      if (!(mass[k] > 0.)) {  // an empty cell neither moves nor limits the step
        s_ts[k] = 1.e20;
        continue;
      }
      double inv = 1. / mass[k];
      double acc = 0.0;
      for (int q = 0; q < D; q++) {
        double a = f[3 * k + q] * inv;
        acc += a * a;
      }
      acc = sqrt(acc);
      s_ts[k] = 0.25 * sqrt(hk[k] / (acc + 1.e-20));
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double gdt = 1.e20;
      for (int k = 0; k < K; k++) gdt = cmin(s_ts[k], gdt);
      s_g = gdt;
    }
    __syncthreads();
    const double gdt = s_g;
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
      const bool full = mass[k] > 0.;
      double inv = full ? 1. / mass[k] : 0.;
      double fac = gdt * gdt * 0.5 * relax;
      for (int q = 0; q < D; q++) {
        double a = full ? f[3 * k + q] * inv : 0.0;
        double v = pressure_step ? vp[3 * k + q] + a * fac : vp[3 * k + q];
        vp[3 * k + q] = cmax(G.box_l[q] + 1.e-20, cmin(v, G.box_r[q] - 1.e-20));
      }
      double sh = 0.0;
      for (int q = 0; q < D; q++) {
        shift[3 * k + q] = mc[3 * k + q] - vp[3 * k + q];
        sh += shift[3 * k + q] * shift[3 * k + q];
      }
      sh = sqrt(sh);
      double sc = cmin(sh, 1. / 32. * hk[k]);
      s_ts[k] = full ? sc / (sh + 1.e-20) : 1.e20;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double gcvt = 1.e20;
      for (int k = 0; k < K; k++) gcvt = cmin(s_ts[k], gcvt);
      s_g = gcvt;
    }
    __syncthreads();
    const double gcvt = s_g;
    for (int k = threadIdx.x; k < K; k += blockDim.x)
      for (int q = 0; q < D; q++) {
        double v = vp[3 * k + q] + shift[3 * k + q] * (gcvt * (1 - relax));
        vp[3 * k + q] = cmax(G.box_l[q] + 1.e-20, cmin(v, G.box_r[q] - 1.e-20));
      }
  }
  if (threadIdx.x == 0) {
    double r = relax;
    if (iter % 600 == 0) r = 1.02 * r;
    st->relax = cmin(r, 0.90);
    st->iter = iter + 1;
  }
}

int cfail(mrsph_handle* h, int code, const std::string& msg) {
  h->err = msg;
  return code;
}

#define CV_CK(call)                                                                     \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess) { rc = cfail(h, MRSPH_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); goto done; } \
  } while (0)

// Core loop on device points (xyz n x 3, pm n), id order.  d_ps (surface
// mass per point) not NULL: the level-set partition with ghost VPs on the
// handle's level set; ghost_xyz (K x 3) / nghost (may be NULL) receive the
// last iteration's ghosts.
int cvp_run(mrsph_handle* h, long long n, double* d_xyz, double* d_pm, const mrsph_cvp_params* p, double* vp_xyz,
            int* labels, double* vp_mass, mrsph_cvp_result* res, const double* d_ps = nullptr,
            double* ghost_xyz = nullptr, int* nghost = nullptr) {
  const int K = p->num_vp, D = h->prm.dim;
  const bool ghosts = d_ps != nullptr;
  CvpGeo G;
  G.dim = D;
  G.K = K;
  G.GM = ghosts ? K : 0;
  G.NP = K + G.GM + 2 * D;
  for (int q = 0; q < 3; q++) {
    G.box_l[q] = h->prm.box_l[q];
    G.box_r[q] = h->prm.box_r[q];
  }
  const long long nchunk = (n + CVP_CHUNK - 1) / CVP_CHUNK;
  cudaStream_t s = h->stream;
  int rc = 0;
  std::vector<void*> mem;
  double *d_vp = nullptr, *d_part = nullptr, *d_face = nullptr, *d_k = nullptr, *d_tm = nullptr, *d_planes = nullptr;
  double* d_src = nullptr;  // VPs then ghost VPs (level-set partition)
  unsigned char* d_flag = nullptr;
  float4* d_planes_f = nullptr;
  int* d_label = nullptr;
  const size_t PS = (size_t)K + G.GM;
  CvpState* d_st = nullptr;
  CvpState hs;
  std::memset(&hs, 0, sizeof(hs));
  hs.relax = p->relax_ratio;
  auto A = [&](void** ptr, size_t bytes) -> cudaError_t {
    cudaError_t e = cudaMalloc(ptr, bytes);
    if (e == cudaSuccess) mem.push_back(*ptr);
    return e;
  };
  CV_CK(A((void**)&d_vp, sizeof(double) * 3 * K));
  CV_CK(A((void**)&d_part, sizeof(double) * 5 * K * nchunk));
  CV_CK(A((void**)&d_face, sizeof(double) * 6 * (size_t)K * G.NP));
  CV_CK(A((void**)&d_planes, sizeof(double) * 4 * (size_t)K * PS));
  CV_CK(A((void**)&d_planes_f, sizeof(float4) * (size_t)K * PS));
  if (ghosts) {
    CV_CK(A((void**)&d_src, sizeof(double) * 3 * PS));
    CV_CK(A((void**)&d_flag, (size_t)K));
    CV_CK(cudaMemsetAsync(d_flag, 0, (size_t)K, h->stream));
  }
  CV_CK(A((void**)&d_k, sizeof(double) * 12 * K));  // mass, mc(3), energy, P, err, f(3), hk, pad
  CV_CK(A((void**)&d_tm, sizeof(double) * nchunk));
  CV_CK(A((void**)&d_label, sizeof(int) * n));
  CV_CK(A((void**)&d_st, sizeof(CvpState)));
  {
    double* vp3 = nullptr;
    CV_CK(A((void**)&vp3, sizeof(double) * 3 * K));  // shift
    CV_CK(cudaMemcpyAsync(d_vp, vp_xyz, sizeof(double) * 3 * K, cudaMemcpyHostToDevice, s));
    CV_CK(cudaMemcpyAsync(d_st, &hs, sizeof(hs), cudaMemcpyHostToDevice, s));
    double *mass = d_k, *mc = d_k + K, *energy = d_k + 4 * K, *P = d_k + 5 * K, *err = d_k + 6 * K,
           *f = d_k + 7 * K, *hk = d_k + 10 * K;
    k_cvp_chunk_mass<<<(int)((nchunk + 127) / 128), 128, 0, s>>>(n, d_pm, nchunk, d_tm);
    k_cvp_target<<<1, 1, 0, s>>>(nchunk, d_tm, K, d_st);
    const int nb = (int)((n + 255) / 256);
    const int ftot = K * G.NP;
    const double* pts = ghosts ? d_src : d_vp;  // the points that bound the cells
    // Voronoi_lset::Initialize: points coloured by their nearest VP
    if (ghosts) k_cvp_assign<<<nb, 256, 0, s>>>(n, d_xyz, K, d_vp, D, d_label, nullptr);
    int it = 0;
    for (; it <= p->max_iter; it++) {
      if (ghosts) {
        k_cvp_flags<<<nb, 256, 0, s>>>(n, d_ps, d_label, d_flag);
        if (D == 3) k_cvp_ghosts<3><<<1, 256, 0, s>>>(h->ls, K, d_vp, d_flag, d_src, d_st);
        else k_cvp_ghosts<2><<<1, 256, 0, s>>>(h->ls, K, d_vp, d_flag, d_src, d_st);
      }
      k_cvp_assign<<<nb, 256, 0, s>>>(n, d_xyz, K, pts, D, d_label, d_st);
      k_cvp_partials<<<(unsigned)nchunk, 256, 0, s>>>(n, d_xyz, d_pm, d_label, K, d_vp, D, d_part);
      k_cvp_reduce<<<(K + 127) / 128, 128, 0, s>>>(nchunk, K, D, d_part, d_st, d_vp, mass, mc, energy, P, err);
      k_cvp_planes<<<(int)((K * PS + 255) / 256), 256, 0, s>>>(G, pts, d_planes, d_planes_f, d_st);
      k_cvp_faces<<<(ftot + 127) / 128, 128, 0, s>>>(G, pts, d_planes, d_planes_f, d_face, d_st);
      k_cvp_update<<<1, (K + 31) / 32 * 32, 0, s>>>(G, d_vp, d_face, mass, mc, energy, P, err, f, hk, vp3, d_st,
                                                   p->error_tolerance, p->pressure_step);
      CV_CK(cudaGetLastError());
      CV_CK(cudaMemcpyAsync(&hs, d_st, sizeof(hs), cudaMemcpyDeviceToHost, s));
      CV_CK(cudaStreamSynchronize(s));
      if (hs.converged) { it++; break; }
    }
    CV_CK(cudaMemcpyAsync(vp_xyz, d_vp, sizeof(double) * 3 * K, cudaMemcpyDeviceToHost, s));
    if (labels) CV_CK(cudaMemcpyAsync(labels, d_label, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
    if (vp_mass) CV_CK(cudaMemcpyAsync(vp_mass, mass, sizeof(double) * K, cudaMemcpyDeviceToHost, s));
    if (ghosts && ghost_xyz)
      CV_CK(cudaMemcpyAsync(ghost_xyz, d_src + 3 * (size_t)K, sizeof(double) * 3 * K, cudaMemcpyDeviceToHost, s));
    CV_CK(cudaStreamSynchronize(s));
    if (nghost) *nghost = ghosts ? hs.nghost : 0;
    if (res) {
      res->iterations = it;
      res->converged = hs.converged;
      res->error_max = hs.error_max;
      res->total_energy = hs.total_energy;
    }
  }
done:
  for (void* q : mem) cudaFree(q);
  return rc;
}

}  // namespace
}  // namespace mrsph

using namespace mrsph;

static int cvp_check(mrsph_handle* h, const mrsph_cvp_params* p, double* vp_xyz) {
  if (!h) return MRSPH_ERR_ARG;
  if (!p || !vp_xyz) return cfail(h, MRSPH_ERR_ARG, "null argument");
  if (p->num_vp < 1 || p->num_vp > CVP_MAX_K) return cfail(h, MRSPH_ERR_RANGE, "num_vp must be 1..1024");
  if (p->max_iter < 0) return cfail(h, MRSPH_ERR_ARG, "max_iter must be >= 0");
  return 0;
}

extern "C" int mrsph_cvp_points(mrsph_handle* h, long long n, const double* xyz, const double* mass,
                                const mrsph_cvp_params* p, double* vp_xyz, int* labels, double* vp_mass,
                                mrsph_cvp_result* res) {
  int rc = cvp_check(h, p, vp_xyz);
  if (rc) return rc;
  if (n <= 0 || !xyz) return cfail(h, MRSPH_ERR_ARG, "no points");
  if (cudaSetDevice(h->prm.device) != cudaSuccess) return cfail(h, MRSPH_ERR_CUDA, "cudaSetDevice failed");
  double *d_xyz = nullptr, *d_pm = nullptr;
  if (cudaMalloc(&d_xyz, sizeof(double) * 3 * n) != cudaSuccess ||
      cudaMalloc(&d_pm, sizeof(double) * n) != cudaSuccess) {
    cudaFree(d_xyz);
    return cfail(h, MRSPH_ERR_OOM, "cudaMalloc failed");
  }
  std::vector<double> ones;
  const double* pm = mass;
  if (!pm) { ones.assign(n, 1.0); pm = ones.data(); }
  cudaMemcpyAsync(d_xyz, xyz, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, h->stream);
  cudaMemcpyAsync(d_pm, pm, sizeof(double) * n, cudaMemcpyHostToDevice, h->stream);
  rc = cvp_run(h, n, d_xyz, d_pm, p, vp_xyz, labels, vp_mass, res);
  cudaFree(d_xyz);
  cudaFree(d_pm);
  return rc;
}

extern "C" int mrsph_cvp_lset(mrsph_handle* h, long long n, const double* xyz, const double* mass,
                              const double* mass_surface, const mrsph_cvp_params* p, double* vp_xyz, int* labels,
                              double* vp_mass, double* ghost_xyz, int* num_ghost, mrsph_cvp_result* res) {
  int rc = cvp_check(h, p, vp_xyz);
  if (rc) return rc;
  if (n <= 0 || !xyz || !mass || !mass_surface) return cfail(h, MRSPH_ERR_ARG, "no points or masses");
  if (2 * p->num_vp > CVP_MAX_K) return cfail(h, MRSPH_ERR_RANGE, "num_vp must be 1..512 with ghost VPs");
  if (h->nls < 1) return cfail(h, MRSPH_ERR_STATE, "mrsph_set_levelset must come first");
  if (cudaSetDevice(h->prm.device) != cudaSuccess) return cfail(h, MRSPH_ERR_CUDA, "cudaSetDevice failed");
  double *d_xyz = nullptr, *d_pm = nullptr, *d_ps = nullptr;
  if (cudaMalloc(&d_xyz, sizeof(double) * 3 * n) != cudaSuccess || cudaMalloc(&d_pm, sizeof(double) * n) != cudaSuccess ||
      cudaMalloc(&d_ps, sizeof(double) * n) != cudaSuccess) {
    cudaFree(d_xyz);
    cudaFree(d_pm);
    return cfail(h, MRSPH_ERR_OOM, "cudaMalloc failed");
  }
  cudaMemcpyAsync(d_xyz, xyz, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, h->stream);
  cudaMemcpyAsync(d_pm, mass, sizeof(double) * n, cudaMemcpyHostToDevice, h->stream);
  cudaMemcpyAsync(d_ps, mass_surface, sizeof(double) * n, cudaMemcpyHostToDevice, h->stream);
  rc = cvp_run(h, n, d_xyz, d_pm, p, vp_xyz, labels, vp_mass, res, d_ps, ghost_xyz, num_ghost);
  cudaFree(d_xyz);
  cudaFree(d_pm);
  cudaFree(d_ps);
  return rc;
}

extern "C" int mrsph_cvp(mrsph_handle* h, const mrsph_cvp_params* p, double* vp_xyz, int* labels, double* vp_mass,
                         mrsph_cvp_result* res) {
  int rc = cvp_check(h, p, vp_xyz);
  if (rc) return rc;
  if (!h->eng) return cfail(h, MRSPH_ERR_STATE, "no particles");
  if (cudaSetDevice(h->prm.device) != cudaSuccess) return cfail(h, MRSPH_ERR_CUDA, "cudaSetDevice failed");
  long long n = h->eng->num_particles();
  if (n <= 0) return cfail(h, MRSPH_ERR_STATE, "no particles");
  double *d_xyz = nullptr, *d_pm = nullptr;
  if (cudaMalloc(&d_xyz, sizeof(double) * 3 * n) != cudaSuccess ||
      cudaMalloc(&d_pm, sizeof(double) * n) != cudaSuccess) {
    cudaFree(d_xyz);
    return cfail(h, MRSPH_ERR_OOM, "cudaMalloc failed");
  }
  rc = h->eng->world_positions(d_xyz);  // particle mass 1 (Particle_mesh_generation::Initialize)
  if (rc) { h->err = h->eng->err; cudaFree(d_xyz); cudaFree(d_pm); return rc; }
  std::vector<double> ones(n, 1.0);
  cudaMemcpyAsync(d_pm, ones.data(), sizeof(double) * n, cudaMemcpyHostToDevice, h->stream);
  rc = cvp_run(h, n, d_xyz, d_pm, p, vp_xyz, labels, vp_mass, res);
  cudaFree(d_xyz);
  cudaFree(d_pm);
  return rc;
}
