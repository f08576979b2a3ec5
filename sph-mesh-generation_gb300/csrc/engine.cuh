// engine.cuh — the relaxation step as CUDA kernels, templated on dimension D
// and arithmetic type R (double: FP64-plain, float: FP32-split).  Included by
// mrsph_fp64.cu (compiled without FMA contraction so FP64 results follow the
// reference's operation order) and mrsph_fp32.cu.
//
// One step (SPH_mesh_generation::SPH_run_mesh_generation,
// sph_mesh_generation.cpp:1371-1463) is 11 launches on one stream, replayed as
// a CUDA graph:
//   k_begin_step   scalars of the step
//   k_map          A1 advect + A2 sample + A3 surface map/re-seed + A4 spacing
//                  + scale/level refresh + cell key + cell histogram
//   scan x3, scatter, rank      A5 counting sort into (level, cell) order
//   k_reorder      gather persistent state into the sorted order
//   k_density      A6 neighbour search over the cell table + A7 kernel sum,
//                  writes the neighbour list (one row per particle)
//   k_force<1>     A8 stage 1 + A9 dt/max|v| grid reduction (FP64 bit atomics)
//   k_force<2>     A8 stage 2 + A9 + A10 (stage-1 kick folded in; the stage-2
//                  kick is folded into the next k_map)
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

#include "engine_iface.h"

namespace mrsph {

using std::max;
using std::min;

// ---------------------------------------------------------------------------
// device data
// ---------------------------------------------------------------------------
template <class R>
struct Buf {  // persistent per-particle state, one ping-pong half
  typename V4<R>::T* posh;  // FP64: (x, y, z, h); FP32: (offset in anchor cell, h)
  typename V4<R>::T* nr;    // (nx, ny, nz, rho)
  typename V4<R>::T* v1;    // velocity after the stage-1 kick
  typename V4<R>::T* a2;    // stage-2 acceleration
  int* key;                 // FP32 anchor cell, packed (FP64: unused)
  int* meta;                // type | level << 8
  int* id;
  R* nu;                    // viscosity read by stage 2
  R* nu_next;               // viscosity written by stage 2
  R* phi;
  R* curv;
  int* cellkey;             // (level, cell) table index
  typename V4<R>::T* rec;   // packed neighbour-pass record, 2 words per particle
};

// Neighbour-list layout: blocks of 32 particles (one warp); inside a block,
// chunks of 8 consecutive entries (one 32-byte sector) per particle,
// interleaved over the 32 particles.  A particle's appends fill whole sectors
// in turn (as a row-major list would), and the lanes of a warp reading their
// q-th entries touch 8 lines instead of 32.  cap is a multiple of 8.
__host__ __device__ inline long long nb_slot(long long s, int q, int cap) {
  return (((((s >> 5) * (cap >> 3) + (q >> 3)) << 5) + (s & 31)) << 3) + (q & 7);
}

template <class R>
struct Work {  // per-step arrays in sorted order
  R* sum;
  typename V4<R>::T* a1;
  int* cnt;
  int* nbl;  // neighbour lists, entry q < cap of particle s at nbl[nb_slot(s, q, cap)]
  R* pc;     // stage-1 pair coefficients aw * (1/rho_i^2 + 1/rho_j^2), 0 for a skipped pair; nbl's layout
  int cap;
  int* counts;
  unsigned* lhmax;  // [level][level-0 cell]: largest h (FP32 bits, rounded up) this step, 0 if none
  int* cstart;
  int* perm;
  int* perm2;
  int* blocksums;
  int* slot_of_id;
  int* fixq;    // FP32-split: particles whose density phase is re-decided exactly (count sc->nfix)
  int* spillq;  // particles whose list spilled (count sc->nspill)
};

// Neighbour-list entries: the neighbour's storage slot in the low 30 bits;
// bits 30-31 carry the surface filter |n_i . n_j| > cos(angle_thres) where
// the FP32-split density fix-up decided it in FP64 (0: decide in FP32).
constexpr int NB_IDX = 0x3FFFFFFF;
constexpr unsigned NB_COS_OK = 1u, NB_COS_NO = 2u;
__host__ __device__ inline int nb_index(int e) { return e & NB_IDX; }
__host__ __device__ inline unsigned nb_mark(int e) { return (unsigned)e >> 30; }

// FP32-split decisions.  Three decisions of a step must come out as the
// reference's FP64 arithmetic on the world positions makes them: the cell of
// a particle (get_cell_id, glbfunc.h:196-208), the neighbour criterion
// r <= h cutoff + 1e-10 for h_i or h_j (level_infor.cpp:491-500) and the
// surface filter |n_i . n_j| > cos(angle_thres) (particle_mesh_generation.cpp:
// 719, 747, 937).  Each is made in FP32 with a band around its threshold that
// is wider than the FP32 error, and inside the band in FP64 with the
// reference's operation order on the world coordinates the position taps
// report.  Bands: the half-cell coordinate of the sort key, 2^-16 of a half
// cell; the squared distance, 2^-15 of the squared cut-off radius (the
// +1e-10 moves the radius by at most 2^-18.9 for radii of at least 1e-4,
// which mrsph_create enforces for FP32-split handles); the cosine, 2^-16.
constexpr float kBandKey = 1.0f / 65536.0f;
constexpr float kD2Accept = 1.0f + 1.0f / 32768.0f;  // FP32 d2 above R^2 * this: certainly not a neighbour
constexpr float kD2Sure = 1.0f - 1.0f / 32768.0f;    // FP32 d2 below R^2 * this: certainly a neighbour
constexpr float kBandCos = 1.0f / 65536.0f;

// Warp-aggregated append of val to queue q (counter *cnt); every lane of the
// warp calls it.
__device__ inline void queue_push(bool pred, unsigned* cnt, int* q, int val) {
  const unsigned m = __ballot_sync(0xffffffffu, pred);
  if (!m) return;
  const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
  unsigned base = 0;
  if (lane == leader) base = atomicAdd(cnt, (unsigned)__popc(m));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (pred) q[base + __popc(m & ((1u << lane) - 1u))] = val;
}

struct KCtx {
  Params prm;
  CellGeo geo;
  LsSet ls;
  long long n;
  DevScalars* sc;
};

// One FP32-split geometry of a batch as the batch kernels (mrsph_persist.cu)
// see it: the handle's context, both state buffers, its per-step arrays, the
// size of its cell table and the buffer that holds its state when the batch
// launch starts.
struct BatchSlot {
  KCtx c;
  Buf<float> buf[2];
  Work<float> w;
  long long ncells;
  int dim;
  int cur;
};

enum { MAP_STEP = 0, MAP_PRE = 1 };

// Tuning of the FP32 map and neighbour passes: resident 256-thread blocks per SM the
// register allocation must allow, and the unroll of the tile loop.
#ifndef MRSPH_DENSITY_MIN_BLOCKS
#define MRSPH_DENSITY_MIN_BLOCKS 6
#endif
#ifndef MRSPH_FORCE_MIN_BLOCKS
#define MRSPH_FORCE_MIN_BLOCKS 5
#endif
#ifndef MRSPH_FORCE2_MIN_BLOCKS
#define MRSPH_FORCE2_MIN_BLOCKS 6
#endif
// list entries (indices, pair coefficients) moved per vector access in the force passes: 1 or 4
#ifndef MRSPH_FORCE_VEC
#define MRSPH_FORCE_VEC 4
#endif
#ifndef MRSPH_MAP_MIN_BLOCKS
#define MRSPH_MAP_MIN_BLOCKS 4
#endif
#ifndef MRSPH_TILE_UNROLL
#define MRSPH_TILE_UNROLL 1
#endif
constexpr int kTileUnroll = MRSPH_TILE_UNROLL;
// largest spread of a warp's half cells (max - min per axis) for which the
// warp scans the union of its lanes' rows through shared-memory tiles
#ifndef MRSPH_TILE_SPAN_X
#define MRSPH_TILE_SPAN_X 3
#endif
#ifndef MRSPH_TILE_SPAN_YZ
#define MRSPH_TILE_SPAN_YZ 1
#endif

// ---------------------------------------------------------------------------
// position representations
// ---------------------------------------------------------------------------
template <int D, class R> struct PosOps;

template <int D>
struct PosOps<D, double> {
  using T4 = double4;
  __device__ static void world(const KCtx&, const T4& p, int, double* x) { x[0] = p.x; x[1] = p.y; x[2] = (D == 3) ? p.z : 0.0; }
  __device__ static void set_world(const KCtx&, T4& p, int&, const double* x) { p.x = x[0]; p.y = x[1]; p.z = (D == 3) ? x[2] : 0.0; }
  // x = x + d  (the reference's coord + delta, component-wise)
  __device__ static void add(const KCtx&, T4& p, int&, const double* d) {
    p.x = p.x + d[0];
    p.y = p.y + d[1];
    if (D == 3) p.z = p.z + d[2];
  }
  // get_cell_id, glbfunc.h:196-208 (_NON_SYM_: [0, num_cell))
  __device__ static void cell(const KCtx& c, int L, const T4& p, int, int* cc) {
    double x[3] = {p.x, p.y, p.z};
    cc[2] = 0;
    for (int d = 0; d < D; d++) {
      int q = (int)floor((x[d] - c.geo.box_l[d]) / c.geo.dcell[L][d]);
      cc[d] = max(0, min(q, c.geo.n[L][d] - 1));
    }
  }
  // box-relative position (the operand of get_cell_id)
  __device__ static void xrel(const KCtx& c, const T4& p, int, double* xr) {
    xr[0] = p.x - c.geo.box_l[0];
    xr[1] = p.y - c.geo.box_l[1];
    xr[2] = (D == 3) ? p.z - c.geo.box_l[2] : 0.0;
  }
  __device__ static void rel(const KCtx&, const T4& pi, int, const T4& pj, int, double* dr) {
    dr[0] = pi.x - pj.x;
    dr[1] = pi.y - pj.y;
    dr[2] = (D == 3) ? pi.z - pj.z : 0.0;
  }
};

// FP32-split: position = anchor cell (finest cell-list cell) + FP32 offset.
template <int D>
struct PosOps<D, float> {
  using T4 = float4;
  __device__ static void unpack(int key, int* k) {
    unsigned u = (unsigned)key;
    if (D == 2) { k[0] = u & 0xFFFF; k[1] = (u >> 16) & 0xFFFF; k[2] = 0; }
    else { k[0] = u & 0x7FF; k[1] = (u >> 11) & 0x7FF; k[2] = (u >> 22) & 0x3FF; }
  }
  __device__ static int pack(const int* k) {
    if (D == 2) return (int)((unsigned)k[0] | ((unsigned)k[1] << 16));
    return (int)((unsigned)k[0] | ((unsigned)k[1] << 11) | ((unsigned)k[2] << 22));
  }
  // world coordinate box_l + (k A + o): one fused multiply-add and one add,
  // both explicit, so every kernel (and the position taps) gets the same bits
  __device__ static double world1(const KCtx& c, int d, int k, float o) {
    return __dadd_rn(c.geo.box_l[d], __fma_rn((double)k, c.geo.A[d], (double)o));
  }
  __device__ static void world(const KCtx& c, const T4& p, int key, double* x) {
    int k[3];
    unpack(key, k);
    float o[3] = {p.x, p.y, p.z};
    x[2] = 0.0;
    for (int d = 0; d < D; d++) x[d] = world1(c, d, k[d], o[d]);
  }
  __device__ static void set_world(const KCtx& c, T4& p, int& key, const double* x) {
    int k[3] = {0, 0, 0};
    float o[3] = {0.f, 0.f, 0.f};
    const int lm = c.geo.ncl - 1;
    for (int d = 0; d < D; d++) {
      double rel = x[d] - c.geo.box_l[d];
      int q = (int)floor(rel / c.geo.A[d]);
      q = max(0, min(q, c.geo.n[lm][d] - 1));
      k[d] = q;
      o[d] = (float)(rel - (double)q * c.geo.A[d]);
    }
    p.x = o[0]; p.y = o[1]; p.z = o[2];
    key = pack(k);
  }
  __device__ static void add(const KCtx& c, T4& p, int& key, const float* dlt) {
    int k[3];
    unpack(key, k);
    float o[3] = {p.x, p.y, p.z};
    const int lm = c.geo.ncl - 1;
    for (int d = 0; d < D; d++) {
      o[d] = o[d] + dlt[d];
      float q = floorf(o[d] / c.geo.Af[d]);
      if (q != 0.f) {
        int kn = max(0, min(k[d] + (int)q, c.geo.n[lm][d] - 1));
        o[d] -= (float)(kn - k[d]) * c.geo.Af[d];
        k[d] = kn;
      }
    }
    p.x = o[0]; p.y = o[1]; p.z = o[2];
    key = pack(k);
  }
  __device__ static void cell(const KCtx& c, int L, const T4&, int key, int* cc) {
    int k[3];
    unpack(key, k);
    int sh = c.geo.ncl - 1 - L;
    cc[2] = 0;
    for (int d = 0; d < D; d++) cc[d] = k[d] >> sh;
  }
  __device__ static void xrel(const KCtx& c, const T4& p, int key, double* xr) {
    int k[3];
    unpack(key, k);
    const float o[3] = {p.x, p.y, p.z};
    xr[2] = 0.0;
    for (int d = 0; d < D; d++) xr[d] = (double)k[d] * c.geo.A[d] + (double)o[d];
  }
  __device__ static void rel(const KCtx& c, const T4& pi, int ki, const T4& pj, int kj, float* dr) {
    int a[3], b[3];
    unpack(ki, a);
    unpack(kj, b);
    dr[0] = (float)(a[0] - b[0]) * c.geo.Af[0] + (pi.x - pj.x);
    dr[1] = (float)(a[1] - b[1]) * c.geo.Af[1] + (pi.y - pj.y);
    dr[2] = (D == 3) ? (float)(a[2] - b[2]) * c.geo.Af[2] + (pi.z - pj.z) : 0.f;
  }
};

// Packed record j (two 16-byte halves, 32-byte aligned; 64 bytes in FP64)
// read through the read-only path with 256-bit loads (sm_100 and later):
// one load instruction per FP32 record instead of two.
__device__ __forceinline__ void ld_rec(const float4* rec, long long j, float4& b0, float4& b1) {
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(b0.x), "=f"(b0.y), "=f"(b0.z), "=f"(b0.w), "=f"(b1.x), "=f"(b1.y), "=f"(b1.z), "=f"(b1.w)
      : "l"(rec + 2 * j));
}
__device__ __forceinline__ void ld_rec(const double4* rec, long long j, double4& b0, double4& b1) {
  asm("ld.global.nc.v4.f64 {%0, %1, %2, %3}, [%4];"
      : "=d"(b0.x), "=d"(b0.y), "=d"(b0.z), "=d"(b0.w) : "l"(rec + 2 * j));
  asm("ld.global.nc.v4.f64 {%0, %1, %2, %3}, [%4];"
      : "=d"(b1.x), "=d"(b1.y), "=d"(b1.z), "=d"(b1.w) : "l"(rec + 2 * j + 1));
}

// Load policies of the step's device functions.  LdNC: the read-only data
// path (ld.global.nc, __ldg) for the per-handle kernels, which never write
// what they read this way.  LdPlain: ordinary global loads for the persistent
// batch kernel, where a buffer read in one phase was written by other blocks
// in an earlier phase of the same launch (after a grid barrier whose fences
// make those writes visible).  The pointers reach the batch kernel through a
// shared-memory copy of the geometry's slot, never as const __restrict__
// kernel parameters, so these loads are not turned into read-only ones.
struct LdNC {
  __device__ static void rec(const float4* r, long long j, float4& b0, float4& b1) { ld_rec(r, j, b0, b1); }
  __device__ static void rec(const double4* r, long long j, double4& b0, double4& b1) { ld_rec(r, j, b0, b1); }
  template <class T> __device__ static T ld(const T* p) { return __ldg(p); }
};
struct LdPlain {
  __device__ static void rec(const float4* r, long long j, float4& b0, float4& b1) {
    b0 = r[2 * j];
    b1 = r[2 * j + 1];
  }
  __device__ static void rec(const double4* r, long long j, double4& b0, double4& b1) {
    b0 = r[2 * j];
    b1 = r[2 * j + 1];
  }
  template <class T> __device__ static T ld(const T* p) { return *p; }
};

template <class R> __device__ inline typename V4<R>::T mk4(R a, R b, R c, R d);
template <> __device__ inline double4 mk4<double>(double a, double b, double c, double d) { return make_double4(a, b, c, d); }
template <> __device__ inline float4 mk4<float>(float a, float b, float c, float d) { return make_float4(a, b, c, d); }

template <int D, class R>
__device__ inline R dot3(const R* a, const R* b) {
  R s = 0;
  s += a[0] * b[0];
  s += a[1] * b[1];
  if (D == 3) s += a[2] * b[2];
  return s;
}

// Set_particle_info, particle_mesh_generation.cpp:361-381 (mass = 1)
template <int D, class R>
__device__ inline void set_info(const KCtx& c, R phi, R curv, R& h, R& rho) {
  R h_tmp = get_scale<R>(c.ls, phi, curv);
  h = h_tmp * pick<R>(c.prm.cell_ratio, c.prm.cell_ratio_f) / pick<R>(c.prm.cutoff, c.prm.cutoff_f);
  R vol;
  if constexpr (std::is_same<R, float>::value) vol = (D == 2) ? h_tmp * h_tmp : h_tmp * h_tmp * h_tmp;
  else vol = (D == 2) ? h_tmp * h_tmp : pow(h_tmp, 3.0);  // pow(h, DIM) as the reference
  rho = (R)1.0 / vol;
}

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------
__device__ inline void begin_step_body(DevScalars* sc, int inc) {
  sc->dt_adv = sc->dt2;
  sc->dt_adv_f = (float)bitsd(sc->dt2);
  sc->hdt_adv_f = (float)(0.5 * bitsd(sc->dt2));
  sc->dt1 = 0x7FF0000000000000ull;  // +inf
  sc->dt2 = 0x7FF0000000000000ull;
  sc->vmax1 = 0;
  sc->vmax2 = 0;
  sc->pairs = 0;
  sc->remap = 0;
  sc->nsurf = 0;
  sc->maxcnt = 0;
  sc->nfix = 0;
  sc->nspill = 0;
  for (int l = 0; l < MAX_CL; l++) {
    sc->hmax[l] = 0;
    sc->lcount[l] = 0;
  }
  sc->step += inc;
}
static __global__ void k_begin_step(DevScalars* sc, int inc) { begin_step_body(sc, inc); }

// clears n words (a step's per-level h maxima) as block blk of 256 threads
__device__ inline void fill_block(unsigned* p, long long n, long long blk) {
  const long long i = blk * blockDim.x + threadIdx.x;
  if (i < n) p[i] = 0u;
}

// Random_particle_distribution, sph_mesh_generation.cpp:1302-1367 (one rank)
template <int D, class R>
__global__ void k_seed(KCtx c, Buf<R> b, unsigned max_att) {
  using P = PosOps<D, R>;
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.n) return;
  const LsLevel& L0 = c.ls.lv[0];
  double padding = L0.dpkg[0];
  R phi = 0, n[3] = {0, 0, 0}, curv = 0, h = 0, rho = 0;
  double x[3] = {0, 0, 0};
  bool ok = false;
  for (unsigned att = 0; att < max_att && !ok; att++) {
    for (int d = 0; d < D; d++) {
      U4 r = philox((uint32_t)i, 0u, att, (RNG_SEED << 8) | d, c.prm.seed);
      double u1 = u53(r.v[0], r.v[1]), u2 = u53(r.v[2], r.v[3]);
      double box = c.prm.box_r[d] - c.prm.box_l[d];
      double lbl = L0.box_l[d], lbr = L0.box_l[d] + L0.dpkg[d] * L0.num_pkg[d];
      double xd = u1 * box + u2 * 1.e-3 + c.prm.box_l[d];
      xd = AMAX1(c.prm.box_l[d] + 1.e-10, AMIN1(xd, c.prm.box_r[d] - 1.e-10));
      xd = AMAX1(lbl + padding, AMIN1(lbr - padding, xd));
      x[d] = xd;
    }
    ls_sample<D, R>(c.ls, x, phi, n, curv);
    set_info<D, R>(c, phi, curv, h, rho);
    if (phi > h) ok = true;
  }
  if (!ok) atomicOr(&c.sc->flags, (unsigned)FLAG_SEED);
  typename V4<R>::T p = mk4<R>(0, 0, 0, h);
  int key = 0;
  P::set_world(c, p, key, x);
  b.posh[i] = p;
  if (b.key) b.key[i] = key;
  b.nr[i] = mk4<R>(n[0], n[1], n[2], rho);
  b.meta[i] = REAL_P;  // level 0: scale = max_scale (Particle_mesh_generation::Initialize)
  b.id[i] = (int)i;
  b.nu[i] = 0;
  b.nu_next[i] = 0;
  b.phi[i] = phi;
  b.curv[i] = curv;
  b.v1[i] = mk4<R>(0, 0, 0, 0);
  b.a2[i] = mk4<R>(0, 0, 0, 0);
}

// A1-A4 + scale refresh + cell key (see file header).  mode MAP_PRE is the
// map part of Pre_run (sph_mesh_generation.cpp:1010-1050): no advection,
// Set_particle_info before Find_and_map.
template <int D, class R>
__device__ inline void map_block(const KCtx& c, const Buf<R>& b, int* counts, unsigned* lhmax, int mode,
                                 unsigned max_att, long long blk) {
  using P = PosOps<D, R>;
  constexpr bool F32 = std::is_same<R, float>::value;
  __shared__ unsigned long long s_hmax[MAX_CL];
  __shared__ unsigned s_lcount[MAX_CL];
  if (threadIdx.x < MAX_CL) {
    s_hmax[threadIdx.x] = 0;
    s_lcount[threadIdx.x] = 0;
  }
  __syncthreads();
  long long i = blk * blockDim.x + threadIdx.x;
  unsigned surf = 0;
  if (i < c.n) {
    int meta = b.meta[i];
    int type = meta & 0xFF;
    int e = (int)(signed char)((meta >> 8) & 0xFF);
    typename V4<R>::T p = b.posh[i];
    int key = b.key ? b.key[i] : 0;
    const int id = b.id[i];
    R h = p.w;
    // A1 Update_coord_full_step (particle_mesh_generation.cpp:1139-1179), with
    // the stage-2 half kick of the previous step folded in (:1130-1135)
    if (mode == MAP_STEP && type != SINGULARITY_P) {
      typename V4<R>::T v1 = b.v1[i], a2 = b.a2[i];
      R hdt, dtr;
      if constexpr (F32) {
        hdt = c.sc->hdt_adv_f;
        dtr = c.sc->dt_adv_f;
      } else {
        const double dt2 = bitsd(c.sc->dt_adv);
        hdt = (R)(0.5 * dt2);
        dtr = (R)dt2;
      }
      R v[3] = {v1.x + a2.x * hdt, v1.y + a2.y * hdt, v1.z + a2.z * hdt};
      R dl[3] = {v[0] * dtr, v[1] * dtr, (D == 3) ? v[2] * dtr : (R)0};
      P::add(c, p, key, dl);
    }
    // A2 at the particle's position: from FP64 world coordinates (FP64-plain)
    // or in FP32 from the anchor representation (FP32-split)
    auto sample_here = [&](R& ph, R* nn, R& cv) {
      if constexpr (F32) {
        int k[3];
        P::unpack(key, k);
        const float o[3] = {p.x, p.y, p.z};
        ls_sample_anchor<D>(c.ls, k, o, ph, nn, cv);
      } else {
        double xw[3];
        P::world(c, p, key, xw);
        ls_sample<D, R>(c.ls, xw, ph, nn, cv);
      }
    };
    auto tag_here = [&](int* chr) -> int {
      if constexpr (F32) {
        // the cell in FP32 unless a cell face lies within the band, then
        // the reference's FP64 lookup of the world position
        int k[3];
        P::unpack(key, k);
        const float o[3] = {p.x, p.y, p.z};
        bool near = false;
        const int t = ls_tag_anchor<D>(c.ls, k, o, chr, &near);
        if (!near) return t;
        double xw[3];
        P::world(c, p, key, xw);
        return ls_tag<D, double>(c.ls, xw, chr);
      } else {
        double xw[3];
        P::world(c, p, key, xw);
        return ls_tag<D, R>(c.ls, xw, chr);
      }
    };
    R phi, n[3], curv, rho = 0;
    sample_here(phi, n, curv);  // A2 Get_particle_info
    if (mode == MAP_PRE) set_info<D, R>(c, phi, curv, h, rho);
    // A3 Find_and_map_particle (:408-467) + driver loop (sph_mesh_generation.cpp:1506-1545)
    int chr = 0;  // characteristic cell: k + 1 on segment k, -(k + 1) at singularity k
    int tag = tag_here(&chr);
    R nl = r_sqrt(dot3<D, R>(n, n));
    if (tag == CUT_CELL && (type == REAL_P || type == SURFACE_P) && chr == 0) {
      type = SURFACE_P;
      R dist = r_fabs(phi);
      R div = (R)1.0 / (nl + (R)1.0e-15);
      R dl[3] = {0, 0, 0};
      for (int d = 0; d < D; d++) {
        R nn = n[d] * div;
        R nd = phi < (R)0 ? nn : -nn;
        dl[d] = nd * dist;
      }
      P::add(c, p, key, dl);
    } else if (chr > 0) {
      // SEGMENT: onto the segment's line (:439-455), in FP64 on the world
      // position: e = (p2 - p1) / max(|p2 - p1|, 1e-15), x = p1 + e ((x - p1) . e)
      type = SEGMENT_P;
      const double* p1 = c.ls.seg + 6 * (chr - 1);
      const double* p2 = p1 + 3;
      double xw[3];
      P::world(c, p, key, xw);
      double Pv[3] = {0.0, 0.0, 0.0}, Nv[3] = {0.0, 0.0, 0.0};
      for (int d = 0; d < D; d++) {
        Pv[d] = __dsub_rn(p2[d], p1[d]);
        Nv[d] = __dsub_rn(xw[d], p1[d]);
      }
      double len = __dmul_rn(Pv[0], Pv[0]);
      len = __dadd_rn(len, __dmul_rn(Pv[1], Pv[1]));
      if (D == 3) len = __dadd_rn(len, __dmul_rn(Pv[2], Pv[2]));
      const double inv = __ddiv_rn(1.0, fmax(__dsqrt_rn(len), 1.e-15));
      double e[3] = {0.0, 0.0, 0.0};
      for (int d = 0; d < D; d++) e[d] = __dmul_rn(Pv[d], inv);
      double dist = __dmul_rn(Nv[0], e[0]);
      dist = __dadd_rn(dist, __dmul_rn(Nv[1], e[1]));
      if (D == 3) dist = __dadd_rn(dist, __dmul_rn(Nv[2], e[2]));
      for (int d = 0; d < D; d++) xw[d] = __dadd_rn(p1[d], __dmul_rn(e[d], dist));
      P::set_world(c, p, key, xw);
    } else if (chr < 0) {
      // SINGULARITY: at the point (:456-465)
      type = SINGULARITY_P;
      const double* ps = c.ls.sing + 3 * (-chr - 1);
      double xw[3] = {ps[0], ps[1], D == 3 ? ps[2] : 0.0};
      P::set_world(c, p, key, xw);
    } else {
      type = REAL_P;
    }
    if (type == SURFACE_P || type == SEGMENT_P) {  // Get_dispersed_position(0.00001*h), :385-404
      R dx = (R)0.00001 * h;
      R div = (R)1.0 / (nl + (R)1.0e-15);
      R dl[3] = {0, 0, 0};
      for (int d = 0; d < D; d++) {
        R nn = n[d] * div;
        R nd = phi < (R)0 ? nn : -nn;
        dl[d] = nd * dx;
      }
      P::add(c, p, key, dl);
    }
    sample_here(phi, n, curv);
    if (phi < (R)0 && type == REAL_P) {
      double x[3];
      // Remap_this_particle_to_positive_phase, sph_mesh_generation.cpp:1885-1928
      atomicAdd(&c.sc->remap, 1u);
      bool ok = false;
      for (unsigned att = 0; att < max_att && !ok; att++) {
        for (int d = 0; d < D; d++) {
          U4 r = philox((uint32_t)id, c.sc->step, att, (RNG_REMAP << 8) | d, c.prm.seed);
          double u1 = u53(r.v[0], r.v[1]), u2 = u53(r.v[2], r.v[3]);
          double bl = c.prm.box_l[d], br = c.prm.box_r[d], box = br - bl;
          double xd = u1 * box + u2 * 1.e-3 + bl;
          x[d] = AMAX1(bl + 1.e-10, AMIN1(xd, br - 1.e-10));
        }
        ls_sample<D, R>(c.ls, x, phi, n, curv);
        if (phi > h) ok = true;
      }
      if (!ok) atomicOr(&c.sc->flags, (unsigned)FLAG_REMAP);
      P::set_world(c, p, key, x);
      type = REAL_P;
      set_info<D, R>(c, phi, curv, h, rho);
    }
    // A4 Set_particle_scale (:361-381)
    if (mode == MAP_STEP) set_info<D, R>(c, phi, curv, h, rho);
    // Particle_base::Set_particle_scale, particle.cpp:957-975 (scale = max_scale*2^-e)
    {
      R sc = F32 ? (R)ldexpf(c.geo.max_scale_f, -e) : (R)ldexp(c.geo.max_scale, -e);
      R hc = h * pick<R>(c.prm.cutoff, c.prm.cutoff_f);
      for (int it = 0; it < 64; it++) {
        if (hc > sc + (R)1.e-15) { sc *= 2; e--; }
        else if (hc < sc / 2 - (R)1.e-15) { sc /= 2; e++; }
        else break;
      }
    }
    int L = e;
    if (L < 0 || L >= c.geo.ncl) {
      atomicOr(&c.sc->flags, (unsigned)FLAG_LEVEL);
      L = max(0, min(L, c.geo.ncl - 1));
      e = L;
    }
    // sort key: level-L half cell (get_cell_id, glbfunc.h:196-208, at dcell/2)
    int hq[3] = {0, 0, 0};
    long long c0 = 0;  // level-0 cell, for the local h maximum of level L
    if constexpr (F32) {
      // a level-L cell is 2^sh anchor cells: the half cell follows from the
      // anchor index and the FP32 position inside the level-L cell
      int k[3];
      P::unpack(key, k);
      const float o[3] = {p.x, p.y, p.z};
      const int sh = c.geo.ncl - 1 - L;
      bool near_edge = false;
      for (int d = 0; d < D; d++) {
        const int cc = k[d] >> sh;
        const float pos = fmaf((float)(k[d] - (cc << sh)), c.geo.Af[d], o[d]);
        const float u = pos * c.geo.ihs_f[L][d];
        const float fl = floorf(u);
        const float fr = u - fl;
        near_edge = near_edge || fr < kBandKey || fr > 1.f - kBandKey;
        hq[d] = max(0, min(2 * cc + (int)fl, c.geo.hn[L][d] - 1));
      }
      if (near_edge) {
        // within the band of a half-cell face: the reference's FP64 binning,
        // floor((x - box_l) / dcell), of the world position.  Half cells are
        // dcell / 2 exactly, so floor((x - box_l) / (dcell / 2)) >> 1 is that
        // cell.
        for (int d = 0; d < D; d++) {
          const double rel = __dsub_rn(P::world1(c, d, k[d], o[d]), c.geo.box_l[d]);
          const double u = floor(__ddiv_rn(rel, c.geo.hs[L][d]));
          hq[d] = (int)fmax(0.0, fmin(u, (double)(c.geo.hn[L][d] - 1)));
        }
      }
      for (int d = D - 1; d >= 0; d--) c0 = c0 * c.geo.n[0][d] + (k[d] >> (c.geo.ncl - 1));
    } else {
      double xr[3];
      P::xrel(c, p, key, xr);
      for (int d = 0; d < D; d++) {
        double u = floor(xr[d] / c.geo.hs[L][d]);
        u = fmax(0.0, fmin(u, (double)(c.geo.hn[L][d] - 1)));
        hq[d] = (int)u;
      }
      for (int d = D - 1; d >= 0; d--) {
        int q0 = (int)fmax(0.0, fmin(floor(xr[d] * c.geo.idc0[d]), (double)(c.geo.n[0][d] - 1)));
        c0 = c0 * c.geo.n[0][d] + q0;
      }
    }
    int ck = (int)(c.geo.hoff[L] + ((long long)hq[2] * c.geo.hn[L][1] + hq[1]) * c.geo.hn[L][0] + hq[0]);
    atomicAdd(&counts[ck], 1);
    atomicMax(&lhmax[L * c.geo.nc0 + c0], __float_as_uint(F32 ? (float)h : __double2float_ru((double)h)));
    atomicMax(&s_hmax[L], dbits((double)h));
    atomicAdd(&s_lcount[L], 1u);
    p.w = h;
    b.posh[i] = p;
    if (b.key) b.key[i] = key;
    b.nr[i] = mk4<R>(n[0], n[1], n[2], rho);
    b.meta[i] = type | ((e & 0xFF) << 8);
    b.phi[i] = phi;
    b.curv[i] = curv;
    b.cellkey[i] = ck;
    surf = (type == SURFACE_P) ? 1u : 0u;
  }
  unsigned ws = __popc(__ballot_sync(0xffffffffu, surf != 0));
  if ((threadIdx.x & 31) == 0 && ws) atomicAdd(&c.sc->nsurf, ws);
  __syncthreads();
  if (threadIdx.x < MAX_CL && s_lcount[threadIdx.x]) {
    atomicMax(&c.sc->hmax[threadIdx.x], s_hmax[threadIdx.x]);
    atomicAdd(&c.sc->lcount[threadIdx.x], s_lcount[threadIdx.x]);
  }
}

template <int D, class R>
__global__ void __launch_bounds__(256, (std::is_same<R, float>::value ? MRSPH_MAP_MIN_BLOCKS : 1))
k_map(KCtx c, Buf<R> b, int* counts, unsigned* lhmax, int mode, unsigned max_att) {
  map_block<D, R>(c, b, counts, lhmax, mode, max_att, blockIdx.x);
}

// Packed record read by the neighbour passes, two V4 words per particle so
// that one candidate costs one 32-byte sector (FP32):
//   FP32: w0 = (offset x, y, z, h), w1 = (anchor x, y, z as exact floats, +-1/rho^2)
//   FP64: w0 = (x, y, z, h),        w1 = (0, 0, 0, +-1/rho^2)
// The sign carries the type: negative for a particle that is not REAL.  1/rho^2 is the
// neighbour's share of the pair coefficient of the force stages, computed once
// per particle (as 1 / (rho * rho), the forces' own expression).
template <int D, class R> struct RecOps;
template <int D>
struct RecOps<D, double> {
  __device__ static void pack(const KCtx&, const double4& p, int, int type, double rho, double4& w0, double4& w1) {
    w0 = p;
    const double vol = r_rcp(rho * rho);
    w1 = make_double4(0.0, 0.0, 0.0, type != REAL_P ? -vol : vol);
  }
  __device__ static void rel(const KCtx&, const double4& a0, const double4&, const double4& b0, const double4&,
                             double* dr) {
    dr[0] = a0.x - b0.x;
    dr[1] = a0.y - b0.y;
    dr[2] = (D == 3) ? a0.z - b0.z : 0.0;
  }
};
template <int D>
struct RecOps<D, float> {
  __device__ static void pack(const KCtx&, const float4& p, int key, int type, float rho, float4& w0, float4& w1) {
    int k[3];
    PosOps<D, float>::unpack(key, k);
    w0 = p;
    const float vol = r_rcp(rho * rho);
    w1 = make_float4((float)k[0], (float)k[1], (float)k[2], type != REAL_P ? -vol : vol);
  }
  __device__ static void rel(const KCtx& c, const float4& a0, const float4& a1, const float4& b0, const float4& b1,
                             float* dr) {
    dr[0] = (a1.x - b1.x) * c.geo.Af[0] + (a0.x - b0.x);
    dr[1] = (a1.y - b1.y) * c.geo.Af[1] + (a0.y - b0.y);
    dr[2] = (D == 3) ? (a1.z - b1.z) * c.geo.Af[2] + (a0.z - b0.z) : 0.f;
  }
};

// The reference's neighbour criterion in FP64 for two FP32-split records
// (w0 = offset, h; w1 = anchor index): world coordinates as the position taps
// compute them, dr = x_i - x_j, dist = sqrt(dr.dr) summed in axis order, and
// dist <= h cutoff + 1e-10 for h_i or h_j (level_infor.cpp:491-500).
template <int D>
__device__ __noinline__ bool exact_neighbor(const KCtx& c, const float4& a0, const float4& a1, const float4& b0,
                                            const float4& b1) {
  const float ao[3] = {a0.x, a0.y, a0.z}, bo[3] = {b0.x, b0.y, b0.z};
  const float ak[3] = {a1.x, a1.y, a1.z}, bk[3] = {b1.x, b1.y, b1.z};
  double d2 = 0.0;
  for (int d = 0; d < D; d++) {
    const double xi = PosOps<D, float>::world1(c, d, (int)ak[d], ao[d]);
    const double xj = PosOps<D, float>::world1(c, d, (int)bk[d], bo[d]);
    const double dr = __dsub_rn(xi, xj);
    d2 = (d == 0) ? __dmul_rn(dr, dr) : __dadd_rn(d2, __dmul_rn(dr, dr));
  }
  const double dist = __dsqrt_rn(d2);
  const double ri = __dadd_rn(__dmul_rn((double)a0.w, c.prm.cutoff), 1.e-10);
  const double rj = __dadd_rn(__dmul_rn((double)b0.w, c.prm.cutoff), 1.e-10);
  return (dist <= ri) || (dist <= rj);
}

// The surface filter |n_i . n_j| > cos(angle_thres) in FP64, products summed
// in axis order (particle_mesh_generation.cpp:719, 747, 937).
template <int D>
__device__ __noinline__ bool exact_cos(const KCtx& c, const float* ni, const float* nj) {
  double ca = __dmul_rn((double)ni[0], (double)nj[0]);
  ca = __dadd_rn(ca, __dmul_rn((double)ni[1], (double)nj[1]));
  if (D == 3) ca = __dadd_rn(ca, __dmul_rn((double)ni[2], (double)nj[2]));
  return fabs(ca) > c.prm.cos_thres;
}

template <int D, class R>
__device__ inline void reorder_block(const Buf<R>& src, const Buf<R>& dst, const KCtx& c, const int* perm2,
                                     int* slot_of_id, long long n, int partial, long long blk) {
  long long s = blk * blockDim.x + threadIdx.x;
  if (s >= n) return;
  int o = perm2[s];
  const auto p = src.posh[o];
  const int key = src.key ? src.key[o] : 0;
  const auto nr = src.nr[o];
  const int meta = src.meta[o];
  dst.posh[s] = p;
  if (src.key) dst.key[s] = key;
  dst.nr[s] = nr;
  dst.meta[s] = meta;
  typename V4<R>::T w0, w1;
  RecOps<D, R>::pack(c, p, key, meta & 0xFF, nr.w, w0, w1);
  dst.rec[2 * s] = w0;
  dst.rec[2 * s + 1] = w1;
  int id = src.id[o];
  dst.id[s] = id;
  dst.nu[s] = src.nu_next[o];
  dst.phi[s] = src.phi[o];
  dst.curv[s] = src.curv[o];
  dst.cellkey[s] = src.cellkey[o];
  if (partial) {  // a step that stops before stage 2 keeps these consistent
    dst.nu_next[s] = src.nu_next[o];
    dst.v1[s] = src.v1[o];
    dst.a2[s] = src.a2[o];
  }
  slot_of_id[id] = (int)s;
}

template <int D, class R>
__global__ void k_reorder(Buf<R> src, Buf<R> dst, KCtx c, const int* __restrict__ perm2,
                          int* __restrict__ slot_of_id, long long n, int partial) {
  reorder_block<D, R>(src, dst, c, perm2, slot_of_id, n, partial, blockIdx.x);
}

// Largest h of level-L particles (lhmax entries) over the level-0 cells
// lo..hi (0: none).
template <class LD = LdNC>
__device__ inline float lhmax_over(const KCtx& c, const unsigned* __restrict__ lhmax, int L, const int* lo,
                                   const int* hi) {
  const unsigned* o = lhmax + (long long)L * c.geo.nc0;
  unsigned m = 0;
  for (int z = lo[2]; z <= hi[2]; z++)
    for (int y = lo[1]; y <= hi[1]; y++)
      for (int x = lo[0]; x <= hi[0]; x++)
        m = max(m, LD::ld(&o[((long long)z * c.geo.n[0][1] + y) * c.geo.n[0][0] + x]));
  return __uint_as_float(m);
}

// Search origin of a particle: its box-relative FP64 position (FP64-plain) or
// its anchor cell and FP32 offset (FP32-split).
template <int D, class R> struct SOrigin;
template <int D> struct SOrigin<D, double> {
  double xr[3];
  __device__ SOrigin(const KCtx& c, const double4& p, int key) { PosOps<D, double>::xrel(c, p, key, xr); }
};
template <int D> struct SOrigin<D, float> {
  int k[3];
  float o[3];
  __device__ SOrigin(const KCtx&, const float4& p, int key) {
    PosOps<D, float>::unpack(key, k);
    o[0] = p.x; o[1] = p.y; o[2] = p.z;
  }
};

// Level L of the candidate search from origin so with smoothing length hi:
// R_L = cutoff * max(hi, local h maximum of level L) + 1e-10 with a relative
// pad (1e-5 FP64, 3e-5 FP32-split; 0 when no level-L particle can pair with the origin), and the
// origin's half-cell coordinate q + fr on level L.  The local h maximum is
// the largest lhmax entry over the level-0 cells overlapping the cube of the
// level-wide bound (every level-L particle that can pair with the origin lies
// in one of them).  FP64-plain keeps the box-relative FP64 arithmetic;
// FP32-split works in FP32 relative to the anchor: a level-L cell is
// 2^(finest - L) anchor cells, so the position inside the origin's level-L
// (or level-0) cell is (anchor index - cell's first anchor) * A + offset.
template <int D, class LD = LdNC>
__device__ inline float level_origin(const KCtx& c, const unsigned* __restrict__ lhmax, int L,
                                     const SOrigin<D, double>& so, double hi, bool active, int* q, float* fr) {
  const double hic = hi * c.prm.cutoff;
  const double Rg = (fmax(hic, bitsd(c.sc->hmax[L]) * c.prm.cutoff) + 1.e-10) * (1.0 + 1.e-5);
  float hloc = 0.f;
  if (active) {
    int lo[3] = {0, 0, 0}, up[3] = {0, 0, 0};
    for (int d = 0; d < D; d++) {
      const double top = (double)(c.geo.n[0][d] - 1);
      lo[d] = (int)fmax(0.0, fmin(floor((so.xr[d] - Rg) * c.geo.idc0[d]), top));
      up[d] = (int)fmax(0.0, fmin(floor((so.xr[d] + Rg) * c.geo.idc0[d]), top));
    }
    hloc = lhmax_over<LD>(c, lhmax, L, lo, up);
  }
  if (!(hloc > 0.f)) return 0.f;
  const double Rw = fmax(hic, (double)hloc * c.prm.cutoff) + 1.e-10;
  for (int d = 0; d < D; d++) {
    double u = so.xr[d] / c.geo.hs[L][d];
    u = fmax(-1.0e6, fmin(u, 1.0e9));
    const double fl = floor(u);
    q[d] = (int)fl;
    fr[d] = (float)(u - fl);
  }
  return (float)(Rw * (1.0 + 1.e-5));
}
template <int D, class LD = LdNC>
__device__ inline float level_origin(const KCtx& c, const unsigned* __restrict__ lhmax, int L,
                                     const SOrigin<D, float>& so, float hi, bool active, int* q, float* fr) {
  const float cut = c.prm.cutoff_f;
  const float hic = hi * cut;
  const float Rg = (fmaxf(hic, (float)bitsd(c.sc->hmax[L]) * cut) + 1.e-10f) * (1.f + 3.e-5f);
  float hloc = 0.f;
  if (active) {
    const int sh0 = c.geo.ncl - 1;
    int lo[3] = {0, 0, 0}, up[3] = {0, 0, 0};
    for (int d = 0; d < D; d++) {
      const int c0 = so.k[d] >> sh0;
      const float u0 = fmaf((float)(so.k[d] - (c0 << sh0)), c.geo.Af[d], so.o[d]) * c.geo.idc0_f[d];
      const float r0 = Rg * c.geo.idc0_f[d];
      const int top = c.geo.n[0][d] - 1;
      lo[d] = max(0, min(c0 + (int)floorf(fmaxf(u0 - r0, -1.0e6f)), top));
      up[d] = max(0, min(c0 + (int)floorf(fminf(u0 + r0, 1.0e6f)), top));
    }
    hloc = lhmax_over<LD>(c, lhmax, L, lo, up);
  }
  if (!(hloc > 0.f)) return 0.f;
  const int sh = c.geo.ncl - 1 - L;
  for (int d = 0; d < D; d++) {
    const int cc = so.k[d] >> sh;
    float u = fmaf((float)(so.k[d] - (cc << sh)), c.geo.Af[d], so.o[d]) * c.geo.ihs_f[L][d];
    u = fmaxf(-1.0e6f, fminf(u, 1.0e6f));
    const float fl = floorf(u);
    q[d] = 2 * cc + (int)fl;
    fr[d] = u - fl;
  }
  return (fmaxf(hic, hloc * cut) + 1.e-10f) * (1.f + 3.e-5f);
}

// Candidates of particle i over all cell-list levels.  The reference walks
// the 3^D cells of i's level, whose lists hold the particles of that level and
// of every finer one, and links i and j when r <= 2 h_i or r <= 2 h_j
// (level_infor.cpp:407-506).  The same relation is found here per level L
// among the level-L particles within R_L = cutoff * max(h_i, hmax_L) + 1e-10
// of x_i, hmax_L being the largest h on level L this step: only the half cells
// of the sort table that the sphere of radius R_L reaches are read.  Each
// (z, y) row of half cells is one contiguous range of the sorted arrays; rows
// farther than R_L are skipped and the x range of each row is cut to the
// sphere.  Edge rows extend to infinity (keys are clamped into the table).
// R_L carries a relative pad for the rounding of the keys and of the row
// arithmetic (FP64: 1e-5; FP32-split: 3e-5, which also covers the FP32
// test's acceptance band of 2^-15 on R^2, so the per-lane and the warp-tile
// scans accept the same candidates); the candidate test decides membership.
template <int D, class R, class LD = LdNC, class F>
__device__ inline void scan_candidates(const KCtx& c, const int* __restrict__ cstart,
                                       const unsigned* __restrict__ lhmax, const SOrigin<D, R>& so, R hi, F&& f) {
  for (int L = 0; L < c.geo.ncl; L++) {
    if (c.sc->lcount[L] == 0) continue;
    int q[3] = {0, 0, 0}, lo[3] = {0, 0, 0}, up[3] = {0, 0, 0}, hn[3];
    float fr[3] = {0.f, 0.f, 0.f}, hs[3] = {1.f, 1.f, 1.f};
    const float R = level_origin<D, LD>(c, lhmax, L, so, hi, true, q, fr);
    if (!(R > 0.f)) continue;
    for (int d = 0; d < 3; d++) hn[d] = c.geo.hn[L][d];
    for (int d = 0; d < D; d++) {
      hs[d] = c.geo.hs_f[L][d];
      const float rr = R / hs[d];
      lo[d] = max(q[d] + (int)floorf(fr[d] - rr), 0);
      up[d] = min(q[d] + (int)floorf(fr[d] + rr), hn[d] - 1);
    }
    const long long base = c.geo.hoff[L];
    const float R2 = R * R;
    for (int z = lo[2]; z <= up[2]; z++) {
      float gz = 0.f;
      if (D == 3) {
        const int m = z - q[2];
        if (z > 0) gz = fmaxf(gz, (float)m - fr[2]);
        if (z < hn[2] - 1) gz = fmaxf(gz, fr[2] - (float)(m + 1));
        gz *= hs[2];
      }
      for (int y = lo[1]; y <= up[1]; y++) {
        const int m = y - q[1];
        float gy = 0.f;
        if (y > 0) gy = fmaxf(gy, (float)m - fr[1]);
        if (y < hn[1] - 1) gy = fmaxf(gy, fr[1] - (float)(m + 1));
        gy *= hs[1];
        const float rem = R2 - gy * gy - gz * gz;
        if (rem < 0.f) continue;
        const float w = sqrtf(rem) / hs[0];
        const int xl = max(q[0] + (int)floorf(fr[0] - w), 0);
        const int xh = min(q[0] + (int)floorf(fr[0] + w), hn[0] - 1);
        if (xl > xh) continue;
        const long long rb = base + ((long long)z * hn[1] + y) * hn[0];
        const int s0 = LD::ld(&cstart[rb + xl]), e0 = LD::ld(&cstart[rb + xh + 1]);
        for (int j = s0; j < e0; j++) f(j);
      }
    }
  }
}

// Warp-cooperative form of scan_candidates, called by all 32 lanes of a warp
// (inactive lanes pass active = false).  Per level, when the warp's particles
// sit within a 4 x 2 x 2 block of half cells (dense regions), the warp walks the
// union of its lanes' rows: each 32-candidate chunk of a row is loaded once,
// coalesced, into the warp's shared-memory tile and every lane tests the
// chunk from there.  Otherwise each lane walks its own rows from global
// memory.  Either way a lane visits its own candidates in the same order
// (levels, rows, storage order), so its accepted neighbours and their order
// do not depend on the mode; lanes also see extra candidates of the union,
// which the candidate test rejects.
// load(k) builds the tile entry of candidate k (uniform mode),
// vchunk(t0, m, tile) visits the m candidates t0 .. t0 + m - 1 held in the
// tile, in that order, vglob(j) visits candidate j straight from global
// memory (per-lane mode).
// origin() gives the search origin (built per level from memory rather than
// held in registers across the scan).
template <int D, class R, class LD = LdNC, class E, class SO, class FL, class FT, class FG>
__device__ inline void warp_scan(const KCtx& c, const int* __restrict__ cstart, const unsigned* __restrict__ lhmax,
                                 bool active, SO&& origin, R hi, E* tile, FL&& load, FT&& vchunk,
                                 FG&& vglob) {
  const int lane = threadIdx.x & 31;
  const unsigned FULL = 0xffffffffu;
  for (int L = 0; L < c.geo.ncl; L++) {
    if (c.sc->lcount[L] == 0) continue;
    int q[3] = {0, 0, 0}, lo[3] = {0, 0, 0}, up[3] = {-1, -1, -1}, hn[3];
    float fr[3] = {0.f, 0.f, 0.f}, hs[3] = {1.f, 1.f, 1.f};
    const float R = level_origin<D, LD>(c, lhmax, L, origin(), hi, active, q, fr);
    const bool need = R > 0.f;
    if (!__any_sync(FULL, need)) continue;
    const float R2 = R * R;
    for (int d = 0; d < 3; d++) hn[d] = c.geo.hn[L][d];
    if (D == 2) { lo[2] = 0; up[2] = 0; }
    if (need) {
      for (int d = 0; d < D; d++) {
        hs[d] = c.geo.hs_f[L][d];
        const float rr = R / hs[d];
        lo[d] = max(q[d] + (int)floorf(fr[d] - rr), 0);
        up[d] = min(q[d] + (int)floorf(fr[d] + rr), hn[d] - 1);
      }
    }
    // own x range of row (z, y); empty when the row is outside the lane's sphere
    auto row_range = [&](int z, int y, int& xl, int& xh) {
      xl = 0x7fffffff;
      xh = -1;
      if (!need || z < lo[2] || z > up[2] || y < lo[1] || y > up[1]) return;
      float gz = 0.f;
      if (D == 3) {
        const int m = z - q[2];
        if (z > 0) gz = fmaxf(gz, (float)m - fr[2]);
        if (z < hn[2] - 1) gz = fmaxf(gz, fr[2] - (float)(m + 1));
        gz *= hs[2];
      }
      const int m = y - q[1];
      float gy = 0.f;
      if (y > 0) gy = fmaxf(gy, (float)m - fr[1]);
      if (y < hn[1] - 1) gy = fmaxf(gy, fr[1] - (float)(m + 1));
      gy *= hs[1];
      const float rem = R2 - gy * gy - gz * gz;
      if (rem < 0.f) return;
      const float w = sqrtf(rem) / hs[0];
      xl = max(q[0] + (int)floorf(fr[0] - w), 0);
      xh = min(q[0] + (int)floorf(fr[0] + w), hn[0] - 1);
    };
    const long long base = c.geo.hoff[L];
    // warp compactness at this level
    const int BIG = 0x3fffffff;
    bool uni = true;
    for (int d = 0; d < D; d++) {
      const int qmin = __reduce_min_sync(FULL, need ? q[d] : BIG);
      const int qmax = __reduce_max_sync(FULL, need ? q[d] : -BIG);
      uni = uni && (qmax - qmin <= (d == 0 ? MRSPH_TILE_SPAN_X : MRSPH_TILE_SPAN_YZ));
    }
    if (uni) {
      const int zl = __reduce_min_sync(FULL, need ? lo[2] : BIG), zu = __reduce_max_sync(FULL, need ? up[2] : -BIG);
      const int yl = __reduce_min_sync(FULL, need ? lo[1] : BIG), yu = __reduce_max_sync(FULL, need ? up[1] : -BIG);
      for (int z = zl; z <= zu; z++)
        for (int y = yl; y <= yu; y++) {
          int xl, xh;
          row_range(z, y, xl, xh);
          const int ul = __reduce_min_sync(FULL, xl), uh = __reduce_max_sync(FULL, xh);
          if (ul > uh) continue;
          const long long rb = base + ((long long)z * hn[1] + y) * hn[0];
          const int s0 = LD::ld(&cstart[rb + ul]), e0 = LD::ld(&cstart[rb + uh + 1]);
          for (int t0 = s0; t0 < e0; t0 += 32) {
            const int k = t0 + lane;
            if (k < e0) tile[lane] = load(k);
            __syncwarp();
            const int m = min(32, e0 - t0);
            if (need) vchunk(t0, m, (const E*)tile);
            __syncwarp();
          }
        }
    } else if (need) {
      for (int z = lo[2]; z <= up[2]; z++)
        for (int y = lo[1]; y <= up[1]; y++) {
          int xl, xh;
          row_range(z, y, xl, xh);
          if (xl > xh) continue;
          const long long rb = base + ((long long)z * hn[1] + y) * hn[0];
          const int s0 = LD::ld(&cstart[rb + xl]), e0 = LD::ld(&cstart[rb + xh + 1]);
          for (int j = s0; j < e0; j++) vglob(j);
        }
    }
  }
}

// Neighbour criterion, level_infor.cpp:491-500.
__device__ inline bool nb_test(double d2, double hi, double hj, double cutoff, double& dist) {
  double R = fmax(hi, hj) * cutoff + 1.e-10;
  if (d2 > R * R * (1.0 + 1.e-9)) return false;  // conservative pre-reject
  dist = sqrt(d2);
  return (dist <= (hi * cutoff + 1.e-10)) || (dist <= (hj * cutoff + 1.e-10));
}

// pair distance of the force passes: IEEE square root in FP32 (see wendland_aw)
__device__ inline double force_dist(double d2) { return sqrt(d2); }
__device__ inline float force_dist(float d2) { return sqrtf(d2); }

template <class R> __device__ inline R d2_of(const R* dr, int D) {
  R d2 = 0;
  d2 += dr[0] * dr[0];
  d2 += dr[1] * dr[1];
  if (D == 3) d2 += dr[2] * dr[2];
  return d2;
}

// How a SURFACE or SEGMENT particle i pairs with a neighbour j that is not
// REAL, in the kernel sum (particle_mesh_generation.cpp:717-759) and the
// forces (:769-991): 1 = through the normal-angle filter (j of i's own type),
// 2 = without the filter, 0 = not at all.  A SURFACE particle takes SURFACE,
// SEGMENT and SINGULARITY neighbours; a SEGMENT particle SEGMENT and
// SINGULARITY neighbours.  Both skip REAL neighbours.
__device__ inline int char_pair(int ti, int tj) {
  if (ti == SURFACE_P) return tj == SURFACE_P ? 1 : 2;
  return tj == SEGMENT_P ? 1 : (tj == SINGULARITY_P ? 2 : 0);
}

// A6 + A7: Refresh_neighbor_info (level_infor.cpp:469-506) and
// Get_kernel_summation (particle_mesh_generation.cpp:690-765).  The
// neighbour list is written in the fixed scan order.
template <class R> struct RecPair { typename V4<R>::T a, b; };


// KK: the kernel kind fixed at compile time (FP32 Wendland C2), or -1
template <int D, class R, int KK, class LD = LdNC>
__device__ inline void density_block(const KCtx& c, const Buf<R>& b, const Work<R>& w, long long blk) {
  using P = PosOps<D, R>;
  using Q = RecOps<D, R>;
  using T4 = typename V4<R>::T;
  constexpr bool F32 = std::is_same<R, float>::value;
  // FP32 tile entry: position relative to the warp's anchor cell and
  // (cutoff*h)^2, negative for a particle that is not REAL; FP64: the packed record
  using E = typename std::conditional<F32, float4, RecPair<R>>::type;
  __shared__ E s_tile[8][32];
  long long i = blk * blockDim.x + threadIdx.x;
  const bool active = i < c.n;
  unsigned long long pairs = 0;
  T4 a0 = mk4<R>(0, 0, 0, 0), a1 = mk4<R>(0, 0, 0, 0);
  int ti = REAL_P;
  R ni[3] = {0, 0, 0};
  if (active) {
    a0 = b.rec[2 * i];
    a1 = b.rec[2 * i + 1];
    ti = b.meta[i] & 0xFF;
    if (!F32 && ti != REAL_P) {
      const T4 nri = b.nr[i];
      ni[0] = nri.x; ni[1] = nri.y; ni[2] = nri.z;
    }
  }
  auto origin = [&]() {
    return SOrigin<D, R>(c, active ? b.posh[i] : mk4<R>(0, 0, 0, 0), (active && b.key) ? b.key[i] : 0);
  };
  const R hi = a0.w;
  const R inv_hi = active ? r_rcp(hi) : (R)0;
  const int kind = KK >= 0 ? KK : c.prm.kernel;
  // FP32 Wendland C2: a REAL particle sums (1 - s/2)^4 (1 + 2s), s = r/h,
  // clamped at s = 2, and applies the normalisation C/h^D once at the end
  constexpr bool WEN32 = F32 && KK == K_WEN;
  const R cos_t = pick<R>(c.prm.cos_thres, c.prm.cos_thres_f);
  const R cut = pick<R>(c.prm.cutoff, c.prm.cutoff_f);
  R sum = 0;
  int ncount = 0, cnt = 0;
  bool unc = false;  // FP32-split: a decision of this particle lies in its band (exact re-decision follows)
  const R R2i = (hi * cut) * (hi * cut);
  int* row = w.nbl + nb_slot(active ? i : 0, 0, w.cap);  // entry q at row[(q >> 3) * 256 + (q & 7)]
  // accepted neighbour j at distance vector dr (i - j), |dr| = dist; char_j:
  // j is not REAL.  A SEGMENT particle sums in 3D only (:740-759).
  const bool char_i = ti == SURFACE_P || (D == 3 && ti == SEGMENT_P);
  auto accept = [&](int j, const R* dr, R dist, bool char_j) {
    if (cnt < w.cap) row[((cnt >> 3) << 8) + (cnt & 7)] = j;
    cnt++;
    if (ti == REAL_P) {
      if constexpr (WEN32) {
        const float s = (float)dist * (float)inv_hi;
        const float t = fmaxf(fmaf(-0.5f, s, 1.f), 0.f), t2 = t * t;
        sum += (t2 * t2) * fmaf(2.f, s, 1.f);
      } else {
        sum += pair_W(kind, D, dist, hi, inv_hi);
        ncount++;
      }
    } else if (char_i && char_j) {  // the tangential kernel sum of a surface or segment particle
      const int rule = char_pair(ti, b.meta[j] & 0xFF);
      if (rule == 0) return;
      if constexpr (F32) {  // the normal is not kept in registers across the scan
        const T4 nri = b.nr[i];
        ni[0] = nri.x; ni[1] = nri.y; ni[2] = nri.z;
      }
      R dn = dot3<D, R>(dr, ni);
      R pr[3] = {dr[0] - ni[0] * dn, dr[1] - ni[1] * dn, dr[2] - ni[2] * dn};
      R pd = pair_dist(dot3<D, R>(pr, pr));
      bool ok = true;
      if (rule == 1) {
        const T4 nrj = b.nr[j];
        const R nj[3] = {nrj.x, nrj.y, nrj.z};
        const R ca = r_fabs(dot3<D, R>(ni, nj));
        if (F32 && fabsf((float)ca - (float)cos_t) <= kBandCos) unc = true;
        ok = ca > cos_t;
      }
      if (ok) {
        sum += pair_W(kind, ti == SEGMENT_P ? 1 : D - 1, pd, hi, inv_hi);
        ncount++;
      }
    }
  };
  if constexpr (F32) {
    // Positions relative to the warp's anchor (lane 0's anchor cell; lane 0
    // is active whenever any lane is), in the tile and in the per-lane path
    // alike, so the particle's own record is not kept across the scan.
    const float wa[3] = {__shfl_sync(0xffffffffu, (float)a1.x, 0), __shfl_sync(0xffffffffu, (float)a1.y, 0),
                         __shfl_sync(0xffffffffu, (float)a1.z, 0)};
    const float pi[3] = {((float)a1.x - wa[0]) * c.geo.Af[0] + (float)a0.x,
                         ((float)a1.y - wa[1]) * c.geo.Af[1] + (float)a0.y,
                         D == 3 ? ((float)a1.z - wa[2]) * c.geo.Af[2] + (float)a0.z : 0.f};
    auto load = [&](int k) {
      float4 b0, b1;
      LD::rec(b.rec, k, b0, b1);
      const float rj = b0.w * (float)cut;
      const float r2 = rj * rj;
      return make_float4((b1.x - wa[0]) * c.geo.Af[0] + b0.x, (b1.y - wa[1]) * c.geo.Af[1] + b0.y,
                         D == 3 ? (b1.z - wa[2]) * c.geo.Af[2] + b0.z : 0.f, b1.w < 0.f ? -r2 : r2);
    };
    auto vglob = [&](int j) {
      const float4 e = load(j);
      float dr[3] = {pi[0] - e.x, pi[1] - e.y, D == 3 ? pi[2] - e.z : 0.f};
      const float d2 = d2_of(dr, D);
      const float Rm = fmaxf((float)R2i, fabsf(e.w));
      if (d2 > Rm * kD2Accept) return;
      if (d2 >= Rm * kD2Sure) unc = true;
      accept(j, (R*)dr, (R)pair_dist(d2), e.w < 0.f);
    };
    // A chunk of 32 tile entries in two parts: every entry is tested without
    // branches into a bit mask, then the lane walks only its own set bits in
    // ascending order (the candidates' order) to accept them.  Accepting in
    // the test loop made the whole warp run the accept path for almost every
    // entry (some lane accepts nearly every candidate), with a third of the
    // lanes idle.
    auto test = [&](const float4& e) -> bool {
      const float dr[3] = {pi[0] - e.x, pi[1] - e.y, D == 3 ? pi[2] - e.z : 0.f};
      return d2_of(dr, D) <= fmaxf((float)R2i, fabsf(e.w)) * kD2Accept;
    };
    auto vchunk = [&](int t0, int m, const float4* tile) {
      unsigned mask = 0u;
      if (m == 32) {
#pragma unroll
        for (int t = 0; t < 32; t++) mask |= test(tile[t]) ? (1u << t) : 0u;
      } else {
        for (int t = 0; t < m; t++) mask |= test(tile[t]) ? (1u << t) : 0u;
      }
      while (mask) {
        const int t = __ffs(mask) - 1;
        mask &= mask - 1u;
        const float4 e = tile[t];
        float dr[3] = {pi[0] - e.x, pi[1] - e.y, D == 3 ? pi[2] - e.z : 0.f};
        const float d2 = d2_of(dr, D);
        const float Rm = fmaxf((float)R2i, fabsf(e.w));
        if (d2 >= Rm * kD2Sure) unc = true;
        accept(t0 + t, (R*)dr, (R)pair_dist(d2), e.w < 0.f);
      }
    };
    warp_scan<D, R, LD>(c, w.cstart, w.lhmax, active, origin, hi, s_tile[threadIdx.x >> 5], load, vchunk, vglob);
  } else {
    auto vglob = [&](int j) {
      T4 b0, b1;
      LD::rec(b.rec, j, b0, b1);
      R dr[3];
      Q::rel(c, a0, a1, b0, b1, dr);
      R dist;
      if (!nb_test(d2_of(dr, D), hi, b0.w, c.prm.cutoff, dist)) return;
      accept(j, dr, dist, b1.w < (R)0);
    };
    auto load = [&](int k) {
      RecPair<R> e;
      LD::rec(b.rec, k, e.a, e.b);
      return e;
    };
    auto vchunk = [&](int t0, int m, const RecPair<R>* tile) {
      for (int t = 0; t < m; t++) {
        const RecPair<R>& e = tile[t];
        R dr[3];
        Q::rel(c, a0, a1, e.a, e.b, dr);
        R dist;
        if (!nb_test(d2_of(dr, D), hi, e.a.w, c.prm.cutoff, dist)) continue;
        accept(t0 + t, dr, dist, e.b.w < (R)0);
      }
    };
    warp_scan<D, R, LD>(c, w.cstart, w.lhmax, active, origin, hi, s_tile[threadIdx.x >> 5], load, vchunk, vglob);
  }
  if (active) {
    if (WEN32 && ti == REAL_P) {
      sum *= (R)((float)kern_norm(K_WEN, D) * (D == 3 ? inv_hi * inv_hi * inv_hi : inv_hi * inv_hi));
      ncount = cnt;
    }
    if (ncount > 1) sum = (R)1. / (sum + (R)1.e-15);
    w.sum[i] = sum;
    w.cnt[i] = cnt;
    if (cnt > w.cap) atomicOr(&c.sc->flags, (unsigned)FLAG_SPILL);
    pairs = (unsigned long long)(cnt - 1);
  }
  queue_push(active && cnt > w.cap, &c.sc->nspill, w.spillq, (int)i);
  if (F32) queue_push(active && unc, &c.sc->nfix, w.fixq, (int)i);
  unsigned mc = (unsigned)(pairs + 1);
  for (int o = 16; o > 0; o >>= 1) mc = max(mc, __shfl_xor_sync(0xffffffffu, mc, o));
  if ((threadIdx.x & 31) == 0 && mc > 1) atomicMax(&c.sc->maxcnt, mc);
  block_sum_u64_to_global(pairs, &c.sc->pairs);
}

template <int D, class R, int KK>
__global__ void __launch_bounds__(256, (std::is_same<R, float>::value ? MRSPH_DENSITY_MIN_BLOCKS : 1)) k_density(KCtx c, Buf<R> b, Work<R> w) {
  density_block<D, R, KK>(c, b, w, blockIdx.x);
}

// FP32-split density fix-up, one warp per queued particle (grid-stride over
// warps): every pair of the particle is decided again (FP32 outside the
// bands, FP64 inside), its list is compacted to the accepted pairs in scan
// order (the lanes take 32 entries at a time; a ballot gives each accepted
// entry its new position), surface-filter decisions made in FP64 are marked
// on their entries (the force passes read the marks), and its kernel sum,
// count and share of the step's pair total are redone.  The sum has one
// fixed order whatever the path: the accepted pairs' terms in list order,
// term p into lane p mod 32's partial sum, the partials folded by a butterfly
// (xor 16, 8, 4, 2, 1).  The list path stores the terms in the pair
// coefficient array (which stage 1 overwrites) and sums them strided; a
// particle whose list spilled re-scans its cells on lane 0, which keeps the
// 32 partial sums itself and folds them the same way.
template <int D, int KK, class LD = LdNC>
__device__ inline void density_fix_items(const KCtx& c, const Buf<float>& b, const Work<float>& w, long long blk,
                                         long long nblk) {
  using Q = RecOps<D, float>;
  constexpr bool WEN = KK == K_WEN;
  const unsigned FULL = 0xffffffffu;
  const unsigned nq = c.sc->nfix;
  const long long wpb = blockDim.x >> 5;
  if (blk * wpb >= (long long)nq) return;  // block-uniform: nothing queued for this block
  const int lane = threadIdx.x & 31;
  const int kind = KK >= 0 ? KK : c.prm.kernel;
  const float cut = c.prm.cutoff_f, cos_t = c.prm.cos_thres_f;
  for (long long t = blk * wpb + (threadIdx.x >> 5); t < nq; t += nblk * wpb) {  // warp-uniform
    const int i = w.fixq[t];
    const float4 a0 = b.rec[2 * i], a1 = b.rec[2 * i + 1];
    const int ti = b.meta[i] & 0xFF;
    float ni[3] = {0.f, 0.f, 0.f};
    if (ti != REAL_P) {
      const float4 q = b.nr[i];
      ni[0] = q.x; ni[1] = q.y; ni[2] = q.z;
    }
    const bool char_i = ti == SURFACE_P || (D == 3 && ti == SEGMENT_P);
    const float hi = a0.w, inv_hi = r_rcp(hi);
    const float R2i = (hi * cut) * (hi * cut);
    const int old = w.cnt[i];
    const long long base = nb_slot(i, 0, w.cap);
    int* row = w.nbl + base;
    float* prow = w.pc + base;
    // decision of pair (i, j): false if j is no neighbour; else e = j with
    // the surface-filter mark, term its kernel-sum term and counted whether
    // it counts towards ncount (generic kernels)
    auto visit = [&](int j, int& e, float& term, bool& counted) -> bool {
      float4 b0, b1;
      LD::rec(b.rec, j, b0, b1);
      float dr[3];
      Q::rel(c, a0, a1, b0, b1, dr);
      const float d2 = d2_of(dr, D);
      const float rj = b0.w * cut;
      const float Rm = fmaxf(R2i, rj * rj);
      if (d2 > Rm * kD2Accept) return false;
      if (d2 >= Rm * kD2Sure && !exact_neighbor<D>(c, a0, a1, b0, b1)) return false;
      e = j;
      term = 0.f;
      counted = false;
      const float dist = pair_dist(d2);
      if (ti == REAL_P) {
        if (WEN) {
          const float s = dist * inv_hi;
          const float tt = fmaxf(fmaf(-0.5f, s, 1.f), 0.f), t2 = tt * tt;
          term = (t2 * t2) * fmaf(2.f, s, 1.f);
        } else {
          term = pair_W(kind, D, dist, hi, inv_hi);
          counted = true;
        }
      } else if (char_i && b1.w < 0.f) {
        const int rule = char_pair(ti, b.meta[j] & 0xFF);
        if (rule == 0) return true;
        const float dn = dot3<D, float>(dr, ni);
        float pr[3] = {dr[0] - ni[0] * dn, dr[1] - ni[1] * dn, dr[2] - ni[2] * dn};
        const float pd = pair_dist(dot3<D, float>(pr, pr));
        bool ok = true;
        if (rule == 1) {
          const float4 q = b.nr[j];
          const float nj[3] = {q.x, q.y, q.z};
          const float ca = fabsf(dot3<D, float>(ni, nj));
          if (fabsf(ca - cos_t) <= kBandCos) {
            ok = exact_cos<D>(c, ni, nj);
            e |= (int)((ok ? NB_COS_OK : NB_COS_NO) << 30);
          } else {
            ok = ca > cos_t;
          }
        }
        if (ok) {
          term = pair_W(kind, ti == SEGMENT_P ? 1 : D - 1, pd, hi, inv_hi);
          counted = true;
        }
      }
      return true;
    };
    int cnt = 0, ncount = 0;
    float sum = 0.f;
    if (old <= w.cap) {
      // the list holds every candidate the FP32 test did not certainly
      // reject; each chunk of 32 entries is read before any of it is written,
      // and an accepted entry moves to a position <= its own
      for (int q0 = 0; q0 < old; q0 += 32) {
        const int q = q0 + lane;
        int e = 0;
        float term = 0.f;
        bool acc = false, counted = false;
        if (q < old) acc = visit(nb_index(LD::ld(&row[((q >> 3) << 8) + (q & 7)])), e, term, counted);
        const unsigned m = __ballot_sync(FULL, acc);
        ncount += __popc(__ballot_sync(FULL, acc && counted));
        if (acc) {
          const int pos = cnt + __popc(m & ((1u << lane) - 1u));
          const int o = ((pos >> 3) << 8) + (pos & 7);
          row[o] = e;
          prow[o] = term;
        }
        cnt += __popc(m);
        __syncwarp();
      }
      for (int p = lane; p < cnt; p += 32) sum += LD::ld(&prow[((p >> 3) << 8) + (p & 7)]);
      for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(FULL, sum, o);
    } else {
      if (lane == 0) {
        float part[32];
        for (int l = 0; l < 32; l++) part[l] = 0.f;
        const SOrigin<D, float> so(c, b.posh[i], b.key[i]);
        scan_candidates<D, float, LD>(c, w.cstart, w.lhmax, so, hi, [&](int j) {
          int e = 0;
          float term = 0.f;
          bool counted = false;
          if (!visit(j, e, term, counted)) return;
          if (cnt < w.cap) row[((cnt >> 3) << 8) + (cnt & 7)] = e;
          part[cnt & 31] += term;
          ncount += counted ? 1 : 0;
          cnt++;
        });
        for (int o = 16; o > 0; o >>= 1) {
          float nxt[32];
          for (int l = 0; l < 32; l++) nxt[l] = part[l] + part[l ^ o];
          for (int l = 0; l < 32; l++) part[l] = nxt[l];
        }
        sum = part[0];
      }
      cnt = __shfl_sync(FULL, cnt, 0);
      ncount = __shfl_sync(FULL, ncount, 0);
    }
    if (lane == 0) {
      if (WEN && ti == REAL_P) {
        sum *= (float)kern_norm(K_WEN, D) * (D == 3 ? inv_hi * inv_hi * inv_hi : inv_hi * inv_hi);
        ncount = cnt;
      }
      if (ncount > 1) sum = 1.f / (sum + 1.e-15f);
      w.sum[i] = sum;
      w.cnt[i] = cnt;
      atomicAdd(&c.sc->pairs, (unsigned long long)(long long)(cnt - old));
    }
    __syncwarp();
  }
}

template <int D, int KK>
__global__ void __launch_bounds__(256) k_density_fix(KCtx c, Buf<float> b, Work<float> w) {
  density_fix_items<D, KK>(c, b, w, blockIdx.x, gridDim.x);
}

__device__ inline void accum_pairs_body(DevScalars* sc) { sc->pairs_total += sc->pairs; }
static __global__ void k_accum_pairs(DevScalars* sc) { accum_pairs_body(sc); }

// four consecutive pair coefficients (16-byte aligned)
__device__ inline void store4(float* p, const float* v) {
  *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ inline void store4(double* p, const double* v) {
  reinterpret_cast<double2*>(p)[0] = make_double2(v[0], v[1]);
  reinterpret_cast<double2*>(p)[1] = make_double2(v[2], v[3]);
}
template <class LD>
__device__ inline void load4(const float* p, float* v) {
  const float4 t = LD::ld(reinterpret_cast<const float4*>(p));
  v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
}
template <class LD>
__device__ inline void load4(const double* p, double* v) {
  const double2 t0 = LD::ld(reinterpret_cast<const double2*>(p)), t1 = LD::ld(reinterpret_cast<const double2*>(p) + 1);
  v[0] = t0.x; v[1] = t0.y; v[2] = t1.x; v[3] = t1.y;
}

// A8 force stages + A9 timestep (Set_timestep(stage), particle_mesh_generation.cpp:127-145).
// Stage 1 evaluates each pair's kernel gradient aw and stores, in the
// neighbour list's layout, the pair coefficient c_ij = aw * (1/rho_i^2 +
// 1/rho_j^2) (0 for a pair the forces skip), and per particle (a1, eta),
// eta = nu * rho, negated for a particle that is not REAL.  The stage-2 viscous term
// of a pair is c_ij * eta_ij * (v_i - v_j) (:1021-1049), so stage 2 reads the
// coefficient and one vector per neighbour; a particle whose list spilled
// re-scans its cells and recomputes c_ij in both stages.
// FP32 Wendland C2 gradient over distance in DK dimensions (0 in 1D, the
// reference's quirk), Derivative_kernel_function (particle.cpp:732-750):
// -5 C (1 - s/2)^3 s / h / (r + 1e-15) with C = norm / h^DK and s = r / h,
// which is -5 norm (1 - s/2)^3 / h^(DK+2) for r > 0 in FP32, and 0 at r = 0.
// 1/h is rounded correctly (__frcp_rn): the hardware approximation's error
// is a smooth function of h, so pairs of similar h_ij share it and a
// near-balanced sum of hundreds of pair forces does not average it out (it
// acts as a slightly different kernel); the force passes take the distance
// from an IEEE square root for the same reason (force_dist).
template <int DK>
__device__ inline float wendland_aw(float dist, float h) {
  if (DK == 1) return 0.f;
  const float ih = __frcp_rn(h);
  const float t = fmaxf(fmaf(-0.5f * ih, dist, 1.f), 0.f);
  float ihp = (ih * ih) * (ih * ih);
  if (DK == 3) ihp *= ih;
  return dist > 0.f ? (-5.f * (float)kern_norm(K_WEN, DK)) * ihp * (t * t * t) : 0.f;
}

// One particle of a force stage.  SPILL = false: the particle's list is
// complete (cnt <= cap); SPILL = true: it spilled and re-scans its cells,
// making the neighbour and surface-filter decisions as the density pass does
// (FP32-split: exact inside the bands).  my_dt / my_v take the min / max.
template <int D, class R, int STAGE, int KK, bool SPILL, class LD = LdNC>
__device__ inline void force_particle(const KCtx& c, const Buf<R>& b, const Work<R>& w, long long i, double& my_dt,
                                      double& my_v) {
  using Q = RecOps<D, R>;
  constexpr bool F32 = std::is_same<R, float>::value;
  constexpr bool WEN32 = F32 && KK == K_WEN;
  using T4 = typename V4<R>::T;
  const T4 a0 = b.rec[2 * i], a1r = b.rec[2 * i + 1];
  const int mi = b.meta[i];
  const int ti = mi & 0xFF;
  R ni[3] = {0, 0, 0};
  if (ti != REAL_P) {
    const T4 nri = b.nr[i];
    ni[0] = nri.x; ni[1] = nri.y; ni[2] = nri.z;
  }
  const R rho = b.nr[i].w, h = a0.w;
  const R cos_t = pick<R>(c.prm.cos_thres, c.prm.cos_thres_f);
  const R sum = (STAGE == 1) ? w.sum[i] : (R)0;
  R nu = 0, eta_i = 0;
  R hdt1 = 0;
  R vi[3] = {0, 0, 0};
  if (STAGE == 2) {
    hdt1 = (R)(0.5 * bitsd(c.sc->dt1));
    T4 an = w.a1[i];
    vi[0] = an.x * hdt1; vi[1] = an.y * hdt1; vi[2] = an.z * hdt1;
    eta_i = r_fabs(an.w);
  } else {
    nu = b.nu[i];
  }
  // FP32-split accumulates a particle's pair forces in groups of four list
  // entries (a candidate scan groups its accepted neighbours the same way)
  // and adds each group's sum into F with compensated (Kahan) summation.  The
  // list is in scan order (levels, then z, y rows), so a plain running sum
  // first collects every same-signed term of one side and reaches about half
  // of sum |terms| before the other side cancels it; rounding at that
  // magnitude, not the terms, dominated the FP32 error.  FP64-plain sums
  // plainly, in the reference's expression order.
  R F[3] = {0, 0, 0}, Fb[3] = {0, 0, 0}, Fc[3] = {0, 0, 0};
  auto accum = [&](int d, R v) {
    if constexpr (F32) Fb[d] = Fb[d] + v;
    else F[d] = F[d] + v;
  };
  auto flush = [&]() {
    if constexpr (F32) {
      for (int d = 0; d < D; d++) {
        const float y = Fb[d] - Fc[d];
        const float t = F[d] + y;
        Fc[d] = (t - F[d]) - y;
        F[d] = t;
        Fb[d] = 0.f;
      }
    }
  };
  const R vol_i = (R)1.0 / (rho * rho);
  // pair (i, j) at relative position vec: the skip rules of :1019-1031 and
  // :904-920, the direction dr the force acts along and the coefficient.
  // mark: the surface filter's FP64 decision from the density fix-up (0: none)
  auto coef = [&](int j, const T4& b0, const T4& b1, const R* vec, R* dr, R& cij, unsigned mark) -> bool {
    if (j == (int)i) return false;
    int rule = 0;
    if (ti != REAL_P) {  // SURFACE or SEGMENT: j must not be REAL
      if (!(b1.w < (R)0)) return false;
      rule = char_pair(ti, b.meta[j] & 0xFF);
      if (rule == 0) return false;
    }
    R aw;
    const R hij = (R)0.5 * (h + b0.w);
    if (ti == REAL_P) {
      dr[0] = vec[0]; dr[1] = vec[1]; dr[2] = vec[2];
      R dist = force_dist(dot3<D, R>(dr, dr));
      if constexpr (WEN32) aw = wendland_aw<D>(dist, hij);
      else aw = pair_dW(c.prm.kernel, D, dist, hij);
    } else {
      R dn = dot3<D, R>(vec, ni);
      dr[0] = vec[0] - ni[0] * dn; dr[1] = vec[1] - ni[1] * dn; dr[2] = vec[2] - ni[2] * dn;
      R dist = force_dist(dot3<D, R>(dr, dr));
      bool ok = true;
      if (rule == 1) {
        if (mark == NB_COS_OK) {
          ok = true;
        } else if (mark == NB_COS_NO) {
          ok = false;
        } else {
          const T4 nrj = b.nr[j];
          const R nj[3] = {nrj.x, nrj.y, nrj.z};
          const R ca = r_fabs(dot3<D, R>(ni, nj));
          ok = ca > cos_t;
          if constexpr (F32 && SPILL) {
            if (fabsf(ca - cos_t) <= kBandCos) ok = exact_cos<D>(c, (const float*)ni, (const float*)nj);
          }
        }
      }
      if (!ok) return false;
      if (ti == SEGMENT_P) {  // the 1D kernel gradient in 3D, none in 2D (:769-879)
        if constexpr (WEN32) aw = wendland_aw<1>(dist, hij);
        else aw = (D == 3) ? pair_dW(c.prm.kernel, 1, dist, hij) : (R)0;
      } else {
        if constexpr (WEN32) aw = wendland_aw<D - 1>(dist, hij);
        else aw = pair_dW(c.prm.kernel, D - 1, dist, hij);
      }
    }
    const R vol_ij = vol_i + r_fabs(b1.w);
    if (STAGE == 1) {
      const R P_ij = sum * vol_ij;
      for (int d = 0; d < D; d++) accum(d, (dr[d] * aw) * -P_ij);
    }
    cij = aw * vol_ij;
    return true;
  };
  auto visc = [&](int j, R cij) {
    const T4 anj = w.a1[j];
    const bool char_j = signbit(anj.w);  // j is not REAL
    R vj[3];
    if (ti == REAL_P && char_j) {
      vj[0] = vi[0] * (R)-1.0; vj[1] = vi[1] * (R)-1.0; vj[2] = vi[2] * (R)-1.0;
    } else {
      vj[0] = anj.x * hdt1; vj[1] = anj.y * hdt1; vj[2] = anj.z * hdt1;
    }
    const R eta_j = r_fabs(anj.w);
    const R eta_ij = r_div((R)2. * eta_j * eta_i, eta_i + eta_j + (R)1.e-15);
    const R temp0 = cij * eta_ij;
    for (int d = 0; d < D; d++) accum(d, (vi[d] - vj[d]) * temp0);
  };
  if (ti != SINGULARITY_P) {  // a SINGULARITY particle has no force
    if constexpr (!SPILL) {
      const int cnt = w.cnt[i];
      const long long base = nb_slot(i, 0, w.cap);
      const int* row = w.nbl + base;
      R* crow = w.pc + base;
      if (MRSPH_FORCE_VEC == 4) {
        // four entries per access: q0 is a multiple of 4, so row + o and
        // crow + o are 16-byte aligned; entries past cnt inside the group
        // lie within the particle's cap and are ignored (stage 1 stores 0)
        for (int q0 = 0; q0 < cnt; q0 += 4) {
          const int o = ((q0 >> 3) << 8) + (q0 & 7);
          const int4 j4 = LD::ld(reinterpret_cast<const int4*>(row + o));
          const int jj[4] = {j4.x, j4.y, j4.z, j4.w};
          R cc[4];
          if (STAGE == 1) {
#pragma unroll
            for (int k = 0; k < 4; k++) {
              cc[k] = 0;
              if (q0 + k < cnt) {
                const int j = nb_index(jj[k]);
                T4 b0, b1;
                LD::rec(b.rec, j, b0, b1);
                R vec[3], dr[3];
                Q::rel(c, a0, a1r, b0, b1, vec);
                coef(j, b0, b1, vec, dr, cc[k], nb_mark(jj[k]));
              }
            }
            store4(crow + o, cc);
          } else {
            load4<LD>(crow + o, cc);
#pragma unroll
            for (int k = 0; k < 4; k++)
              if (q0 + k < cnt && cc[k] != (R)0) visc(nb_index(jj[k]), cc[k]);
          }
          flush();
        }
      } else {
        for (int q = 0; q < cnt; q++) {
          const int o = ((q >> 3) << 8) + (q & 7);
          if (STAGE == 1) {
            const int e = LD::ld(&row[o]);
            const int j = nb_index(e);
            T4 b0, b1;
            LD::rec(b.rec, j, b0, b1);
            R vec[3], dr[3], cij = 0;
            Q::rel(c, a0, a1r, b0, b1, vec);
            coef(j, b0, b1, vec, dr, cij, nb_mark(e));
            crow[o] = cij;
          } else {
            const R cij = LD::ld(&crow[o]);
            if (cij != (R)0) visc(nb_index(LD::ld(&row[o])), cij);
          }
          if ((q & 3) == 3 || q == cnt - 1) flush();
        }
      }
    } else {
      const R cut = pick<R>(c.prm.cutoff, c.prm.cutoff_f);
      const R R2i = (h * cut) * (h * cut);
      const SOrigin<D, R> so(c, b.posh[i], b.key ? b.key[i] : 0);
      int q = 0;  // accepted neighbours so far (the list entries this scan replaces)
      scan_candidates<D, R, LD>(c, w.cstart, w.lhmax, so, h, [&](int j) {
        T4 b0, b1;
        LD::rec(b.rec, j, b0, b1);
        R vec[3], dr[3], cij = 0;
        Q::rel(c, a0, a1r, b0, b1, vec);
        if constexpr (F32) {
          const float d2 = d2_of(vec, D);
          const float rj = b0.w * cut;
          const float Rm = fmaxf(R2i, rj * rj);
          if (d2 > Rm * kD2Accept) return;
          if (d2 >= Rm * kD2Sure && !exact_neighbor<D>(c, a0, a1r, b0, b1)) return;
        } else {
          R dist;
          if (!nb_test(d2_of(vec, D), h, b0.w, c.prm.cutoff, dist)) return;
        }
        if (coef(j, b0, b1, vec, dr, cij, 0u) && STAGE == 2 && cij != (R)0) visc(j, cij);
        if ((q & 3) == 3) flush();
        q++;
      });
      if (q & 3) flush();
    }
  }
  R a[3] = {0, 0, 0};
  if (ti != SINGULARITY_P) {
    if constexpr (F32)
      for (int d = 0; d < D; d++) F[d] = F[d] - Fc[d];
    for (int d = 0; d < D; d++) a[d] = F[d];
    if (STAGE == 2)
      for (int d = 0; d < D; d++) a[d] = a[d] + vi[d] * pick<R>(c.prm.damp_coeff, c.prm.damp_coeff_f);
    if (ti == SURFACE_P || ti == SEGMENT_P) {  // Map_surface_particle_force, :1122-1126
      R nf = dot3<D, R>(a, ni);
      for (int d = 0; d < D; d++) a[d] = a[d] - ni[d] * nf;
    }
  }
  R U = r_sqrt(dot3<D, R>(vi, vi));
  R A = r_sqrt(dot3<D, R>(a, a));
  R ts = (R)0.25 * r_sqrt(h / (A + (R)1.e-15));
  ts = AMIN1(ts, h / (R)40. / (U + (R)1.e-15));
  if (STAGE == 2) {
    R nu_new = pick<R>(c.prm.nu_coeff, c.prm.nu_coeff_f) * h * U;
    ts = AMIN1(ts, (R)0.125 * h * h / (nu_new + (R)1.e-15));
    b.nu_next[i] = nu_new;
    b.v1[i] = mk4<R>(vi[0], vi[1], vi[2], U);
    b.a2[i] = mk4<R>(a[0], a[1], a[2], 0);
  } else {
    const R eta = nu * rho;
    w.a1[i] = mk4<R>(a[0], a[1], a[2], ti != REAL_P ? -eta : eta);
  }
  my_dt = fmin(my_dt, (double)ts);
  my_v = fmax(my_v, (double)U);
}

// KK: the kernel kind fixed at compile time (FP32 Wendland C2), or -1.
// Particles whose list spilled are left to k_force_spill.
template <int D, class R, int STAGE, int KK, class LD = LdNC>
__device__ inline void force_block(const KCtx& c, const Buf<R>& b, const Work<R>& w, long long blk) {
  long long i = blk * blockDim.x + threadIdx.x;
  double my_dt = 1.e300, my_v = 0.0;
  if (i < c.n && w.cnt[i] <= w.cap) force_particle<D, R, STAGE, KK, false, LD>(c, b, w, i, my_dt, my_v);
  if (STAGE == 1) block_minmax_to_global(my_dt, my_v, &c.sc->dt1, &c.sc->vmax1);
  else block_minmax_to_global(my_dt, my_v, &c.sc->dt2, &c.sc->vmax2);
}

template <int D, class R, int STAGE, int KK>
__global__ void __launch_bounds__(256, (std::is_same<R, float>::value ? (STAGE == 1 ? MRSPH_FORCE_MIN_BLOCKS : MRSPH_FORCE2_MIN_BLOCKS) : 1)) k_force(KCtx c, Buf<R> b, Work<R> w) {
  force_block<D, R, STAGE, KK>(c, b, w, blockIdx.x);
}

// The force stage of the particles whose list spilled (queued by the density
// pass; grid-stride), re-scanning their cells.
template <int D, class R, int STAGE, int KK, class LD = LdNC>
__device__ inline void force_spill_items(const KCtx& c, const Buf<R>& b, const Work<R>& w, long long blk,
                                         long long nblk) {
  double my_dt = 1.e300, my_v = 0.0;
  const unsigned nq = c.sc->nspill;
  if (blk * blockDim.x >= (long long)nq) return;  // block-uniform: nothing queued for this block
  for (long long t = blk * blockDim.x + threadIdx.x; t < nq; t += nblk * blockDim.x) {
    const int i = w.spillq[t];
    if (w.cnt[i] > w.cap) force_particle<D, R, STAGE, KK, true, LD>(c, b, w, i, my_dt, my_v);
  }
  if (STAGE == 1) block_minmax_to_global(my_dt, my_v, &c.sc->dt1, &c.sc->vmax1);
  else block_minmax_to_global(my_dt, my_v, &c.sc->dt2, &c.sc->vmax2);
}

template <int D, class R, int STAGE, int KK>
__global__ void __launch_bounds__(256) k_force_spill(KCtx c, Buf<R> b, Work<R> w) {
  force_spill_items<D, R, STAGE, KK>(c, b, w, blockIdx.x, gridDim.x);
}

// ----------------------------------------------------------------- taps
template <int D, class R>
__global__ void k_tap(KCtx c, Buf<R> b, Work<R> w, const int* __restrict__ slot_of_id, double* out, int field,
                      int have_work) {
  using P = PosOps<D, R>;
  long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= c.n) return;
  int s = slot_of_id[k];
  double* o3 = out + 3 * k;
  switch (field) {
    case 0: { double x[3]; P::world(c, b.posh[s], b.key ? b.key[s] : 0, x); o3[0] = x[0]; o3[1] = x[1]; o3[2] = x[2]; break; }
    case 1: {  // velocity after the last complete step
      double dt2 = bitsd(c.sc->dt2);
      auto v1 = b.v1[s]; auto a2 = b.a2[s];
      R hdt = (R)(0.5 * dt2);
      o3[0] = (double)(v1.x + a2.x * hdt); o3[1] = (double)(v1.y + a2.y * hdt);
      o3[2] = (D == 3) ? (double)(v1.z + a2.z * hdt) : 0.0;
      break;
    }
    case 2: { auto q = b.nr[s]; o3[0] = q.x; o3[1] = q.y; o3[2] = q.z; break; }
    case 3: { auto q = have_work ? w.a1[s] : mk4<R>(0, 0, 0, 0); o3[0] = q.x; o3[1] = q.y; o3[2] = q.z; break; }
    case 4: { auto q = b.a2[s]; o3[0] = q.x; o3[1] = q.y; o3[2] = q.z; break; }
    case 5: out[k] = (double)b.posh[s].w; break;
    case 6: out[k] = (double)b.phi[s]; break;
    case 7: out[k] = (double)b.curv[s]; break;
    case 8: out[k] = have_work ? (double)w.sum[s] : 0.0; break;
    case 9: out[k] = (double)b.nr[s].w; break;
    case 10: out[k] = (double)b.nu_next[s]; break;
    case 11: out[k] = (double)(b.meta[s] & 0xFF); break;
    case 12: out[k] = (double)(signed char)((b.meta[s] >> 8) & 0xFF); break;
  }
}

// triangulation inputs by particle id; rows translated to ids and sorted
template <int D, class R>
__global__ void k_export_tri(KCtx c, Buf<R> b, Work<R> w, double* __restrict__ xyz, int* __restrict__ type,
                             double* __restrict__ phi, int* __restrict__ rows, int* __restrict__ cnt, int rowcap,
                             unsigned* flags, double* __restrict__ hout, bool sort_rows) {
  using P = PosOps<D, R>;
  long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= c.n) return;
  int s = w.slot_of_id[k];
  double x[3];
  P::world(c, b.posh[s], b.key ? b.key[s] : 0, x);
  xyz[3 * k] = x[0]; xyz[3 * k + 1] = x[1]; xyz[3 * k + 2] = x[2];
  type[k] = b.meta[s] & 0xFF;
  phi[k] = (double)b.phi[s];
  if (hout) hout[k] = (double)b.posh[s].w;
  int m = w.cnt[s];
  if (m > w.cap || m > rowcap) { atomicOr(flags, 4u); m = min(w.cap, rowcap); }
  cnt[k] = m;
  const int* src = w.nbl + nb_slot(s, 0, w.cap);
  int* dst = rows + k * rowcap;
  if (!sort_rows) {
    for (int q = 0; q < m; q++) dst[q] = b.id[nb_index(src[((q >> 3) << 8) + (q & 7)])];
    return;
  }
  for (int q = 0; q < m; q++) {  // insertion sort by id
    int v = b.id[nb_index(src[((q >> 3) << 8) + (q & 7)])];
    int p = q;
    while (p > 0 && dst[p - 1] > v) { dst[p] = dst[p - 1]; p--; }
    dst[p] = v;
  }
}

template <int D, class R>
__global__ void k_upload(KCtx c, Buf<R> b, const double* __restrict__ xyz) {
  using P = PosOps<D, R>;
  long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= c.n) return;
  int id = b.id[s];
  double x[3] = {xyz[3 * (long long)id], xyz[3 * (long long)id + 1], xyz[3 * (long long)id + 2]};
  auto p = b.posh[s];
  int key = b.key ? b.key[s] : 0;
  P::set_world(c, p, key, x);
  b.posh[s] = p;
  if (b.key) b.key[s] = key;
}

template <int D, class R>
__global__ void k_set_state(KCtx c, Buf<R> b, const double* __restrict__ in, int has_v, int has_h, int has_nu,
                            int has_level, const int* __restrict__ type, const int* __restrict__ level) {
  using P = PosOps<D, R>;
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.n) return;
  const long long n = c.n;
  double x[3] = {in[3 * i], in[3 * i + 1], in[3 * i + 2]};
  typename V4<R>::T p = mk4<R>(0, 0, 0, has_h ? (R)in[9 * n + i] : (R)0);
  int key = 0;
  P::set_world(c, p, key, x);
  b.posh[i] = p;
  if (b.key) b.key[i] = key;
  R v[3] = {0, 0, 0};
  if (has_v) for (int d = 0; d < 3; d++) v[d] = (R)in[3 * n + 3 * i + d];
  b.v1[i] = mk4<R>(v[0], v[1], v[2], 0);
  b.a2[i] = mk4<R>(0, 0, 0, 0);
  R nu = has_nu ? (R)in[6 * n + i] : (R)0;
  b.nu[i] = nu;
  b.nu_next[i] = nu;
  int t = type ? type[i] : REAL_P;
  int e = has_level ? level[i] : 0;
  b.meta[i] = t | ((e & 0xFF) << 8);
  b.id[i] = (int)i;
  b.nr[i] = mk4<R>(0, 0, 0, 0);
  b.phi[i] = 0;
  b.curv[i] = 0;
}

static __global__ void k_iota(int* a, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = (int)i;
}

template <int D, class R>
__global__ void k_sample_points(KCtx c, long long n, const double* __restrict__ xyz, double* out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double x[3] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
  R phi, nn[3], curv;
  ls_sample<D, R>(c.ls, x, phi, nn, curv);
  out[6 * i + 0] = phi;
  out[6 * i + 1] = nn[0];
  out[6 * i + 2] = nn[1];
  out[6 * i + 3] = nn[2];
  out[6 * i + 4] = curv;
  out[6 * i + 5] = (double)ls_tag<D, R>(c.ls, x);
}

// ---------------------------------------------------------------------------
// host engine
// ---------------------------------------------------------------------------
#define MR_CK(call)                                                                     \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess) {                                                            \
      err = std::string(#call) + ": " + cudaGetErrorString(e_);                         \
      return MRSPH_ERR_CUDA;                                                            \
    }                                                                                   \
  } while (0)

template <int D, class R>
class Engine : public EngineBase {
  using T4 = typename V4<R>::T;

 public:
  explicit Engine(const EngineConfig& cfg) : cfg_(cfg) {
    kc_.prm = cfg.prm;
    kc_.geo = cfg.geo;
    kc_.ls = cfg.ls;
    kc_.n = 0;
    kc_.sc = nullptr;
    st_ = cfg.stream;
    // FP32 copies of the run parameters, read by the FP32-split kernels
    kc_.prm.cell_ratio_f = (float)kc_.prm.cell_ratio;
    kc_.prm.cutoff_f = (float)kc_.prm.cutoff;
    kc_.prm.cos_thres_f = (float)kc_.prm.cos_thres;
    kc_.prm.nu_coeff_f = (float)kc_.prm.nu_coeff;
    kc_.prm.damp_coeff_f = (float)kc_.prm.damp_coeff;
    kc_.ls.max_phi_f = (float)kc_.ls.max_phi;
    kc_.ls.dl0_f = (float)kc_.ls.dl0;
    kc_.ls.min_dl_f = (float)kc_.ls.min_dl;
    kc_.ls.max_dl_f = (float)kc_.ls.max_dl;
    kc_.ls.middle_dl_f = (float)kc_.ls.middle_dl;
    kc_.ls.max_curv_f = (float)kc_.ls.max_curv;
    kc_.ls.min_curv_f = (float)kc_.ls.min_curv;
    kc_.geo.max_scale_f = (float)kc_.geo.max_scale;
    if (std::is_same<R, float>::value) init_rc_ = anchor_tables();
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, dev);
    cudaGetLastError();
    if (sms_ < 1) sms_ = 1;
  }
  ~Engine() override {
    release();
    for (void* p : anc_allocs_) cudaFree(p);
  }

  int seed(long long n) override {
    int rc = alloc(n);
    if (rc) return rc;
    MR_CK(cudaMemsetAsync(kc_.sc, 0, sizeof(DevScalars), st_));
    k_seed<D, R><<<grid(n), 256, 0, st_>>>(kc_, buf_[cur_], 1000000u);
    MR_CK(cudaGetLastError());
    return pre_run();
  }

  int set_state(long long n, const mrsph_state_in* s, int pre) override {
    int rc = alloc(n);
    if (rc) return rc;
    std::vector<double> host((size_t)10 * n, 0.0);
    for (long long i = 0; i < 3 * n; i++) host[i] = s->xyz[i];
    if (s->v) for (long long i = 0; i < 3 * n; i++) host[3 * n + i] = s->v[i];
    if (s->nu) for (long long i = 0; i < n; i++) host[6 * n + i] = s->nu[i];
    if (s->h) for (long long i = 0; i < n; i++) host[9 * n + i] = s->h[i];
    double* dbuf = nullptr;
    int* dint = nullptr;
    MR_CK(cudaMalloc(&dbuf, sizeof(double) * 10 * n));
    MR_CK(cudaMalloc(&dint, sizeof(int) * 2 * n));
    MR_CK(cudaMemcpyAsync(dbuf, host.data(), sizeof(double) * 10 * n, cudaMemcpyHostToDevice, st_));
    if (s->type) MR_CK(cudaMemcpyAsync(dint, s->type, sizeof(int) * n, cudaMemcpyHostToDevice, st_));
    if (s->level) MR_CK(cudaMemcpyAsync(dint + n, s->level, sizeof(int) * n, cudaMemcpyHostToDevice, st_));
    MR_CK(cudaMemsetAsync(kc_.sc, 0, sizeof(DevScalars), st_));
    k_set_state<D, R><<<grid(n), 256, 0, st_>>>(kc_, buf_[cur_], dbuf, s->v != nullptr, s->h != nullptr,
                                                 s->nu != nullptr, s->level != nullptr,
                                                 s->type ? dint : nullptr, dint + n);
    MR_CK(cudaGetLastError());
    DevScalars h{};
    h.dt2 = dbits_host(s->dt);
    h.step = (unsigned)s->step;
    MR_CK(cudaMemcpyAsync(kc_.sc, &h, sizeof(h), cudaMemcpyHostToDevice, st_));
    k_iota<<<grid(n), 256, 0, st_>>>(w_.slot_of_id, n);
    MR_CK(cudaStreamSynchronize(st_));
    cudaFree(dbuf);
    cudaFree(dint);
    have_work_ = false;
    if (pre) return pre_run();
    return 0;  // state stays in id order (slot_of_id = identity) until the next step
  }

  int run_phase(int phase) override {
    if (!n_) { err = "no particles"; return MRSPH_ERR_STATE; }
    int rc = launch_step(phase);
    if (rc) return rc;
    MR_CK(cudaStreamSynchronize(st_));
    MR_CK(cudaGetLastError());
    return 0;
  }

  // Graph replay.  The neighbour-list capacity follows the largest list
  // seen: every 32 steps (and on the first call) the device max count is read
  // and the list grown, within a memory budget; particles whose list does not
  // fit are handled by re-scanning their cells in the force kernels.
  int step(int nsteps) override {
    if (!n_) { err = "no particles"; return MRSPH_ERR_STATE; }
    if (nsteps <= 0) return 0;
    for (int k = 0; k < nsteps; k++) {
      int rc = build_graphs();
      if (rc) return rc;
      MR_CK(cudaGraphLaunch(graph_[cur_], st_));
      cur_ ^= 1;
      have_work_ = true;
      if (--countdown_ <= 0) {
        rc = maybe_grow_cap();
        if (rc) return rc;
        countdown_ = 32;
      }
    }
    return 0;
  }

  // Reads the largest neighbour count of the last step and grows the list
  // capacity (graphs are rebuilt).  Stays with the re-scan fallback when the
  // allocation fails or exceeds the budget (half of the device memory free
  // beside the current lists, at least 48 GB), or when the caller fixed the
  // cap; a growth that falls short raises MRSPH_FLAG_CAPACITY_CLAMPED in the
  // next stats.
  int maybe_grow_cap() {
    unsigned mc = 0;
    MR_CK(cudaMemcpyAsync(&mc, &kc_.sc->maxcnt, sizeof(unsigned), cudaMemcpyDeviceToHost, st_));
    MR_CK(cudaStreamSynchronize(st_));
    if ((int)mc <= w_.cap || cfg_.neighbor_cap > 0) return 0;
    long long want = ((long long)mc * 5 / 4 + 31) / 32 * 32;
    const long long n32 = (n_ + 31) / 32 * 32;  // nb_slot blocks of 32 particles
    const long long per_entry = (long long)(sizeof(int) + sizeof(R)) * n32;
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
      cudaGetLastError();
      free_b = 0;
    }
    // the current lists are freed only once the new ones are in place, so the
    // new ones must fit beside them
    const long long avail = (long long)free_b + per_entry * w_.cap;
    const long long budget = std::max(48ll << 30, std::min(avail / 2, (long long)free_b));  // lists + pair coefficients
    long long maxcap = budget / per_entry / 8 * 8;
    if (want > maxcap) {
      want = maxcap;
      cap_clamped_ = true;
    }
    if (want <= w_.cap) return 0;
    int* nb = nullptr;
    R* pc = nullptr;
    cudaError_t e = cudaMalloc(&nb, sizeof(int) * (size_t)want * n32);
    if (e == cudaSuccess) {
      e = cudaMalloc(&pc, sizeof(R) * (size_t)want * n32);
      if (e != cudaSuccess) cudaFree(nb);
    }
    if (e != cudaSuccess) {
      cudaGetLastError();
      cap_clamped_ = true;
      return 0;
    }
    for (auto& p : allocs_) {
      if (p == w_.nbl) { cudaFree(p); p = nb; }
      else if (p == w_.pc) { cudaFree(p); p = pc; }
    }
    w_.nbl = nb;
    w_.pc = pc;
    w_.cap = (int)want;
    drop_graphs();
    return 0;
  }

  int build_graphs() {
    for (int p = 0; p < 2; p++) {
      if (!graph_[p]) {
        int saved = cur_;
        cur_ = p;
        MR_CK(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
        int rc = launch_step(MRSPH_PHASE_FORCE2);
        cudaGraph_t g;
        cudaError_t ee = cudaStreamEndCapture(st_, &g);
        cur_ = saved;
        if (rc) return rc;
        if (ee != cudaSuccess) { err = cudaGetErrorString(ee); return MRSPH_ERR_CUDA; }
        cudaError_t ie = cudaGraphInstantiate(&graph_[p], g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) { graph_[p] = nullptr; err = cudaGetErrorString(ie); return MRSPH_ERR_CUDA; }
        MR_CK(cudaGraphUpload(graph_[p], st_));  // upload now, not at the first (timed) launch
      }
    }
    return 0;
  }

  void drop_graphs() {
    for (int p = 0; p < 2; p++) {
      if (graph_[p]) { cudaGraphExecDestroy(graph_[p]); graph_[p] = nullptr; }
    }
  }

  // One step of a batch: the step graph of the current parity launched on the
  // handle's stream, without the periodic capacity check (the batch makes it).
  int step_batched() override {
    if (!n_) { err = "no particles"; return MRSPH_ERR_STATE; }
    int rc = build_graphs();
    if (rc) return rc;
    MR_CK(cudaGraphLaunch(graph_[cur_], st_));
    cur_ ^= 1;
    have_work_ = true;
    return 0;
  }

  int prepare_steps() override { return n_ ? build_graphs() : 0; }

  int check_capacity() override { return have_work_ ? maybe_grow_cap() : 0; }

  int stats(mrsph_stats* o) override {
    DevScalars h;
    MR_CK(cudaMemcpyAsync(&h, kc_.sc, sizeof(h), cudaMemcpyDeviceToHost, st_));
    MR_CK(cudaStreamSynchronize(st_));
    // cleared on the engine stream, ordered before the next step's kernels
    MR_CK(cudaMemsetAsync(&kc_.sc->flags, 0, sizeof(unsigned), st_));
    o->dt = bitsd_host(h.dt2);
    o->dt_stage1 = bitsd_host(h.dt1);
    o->max_v = bitsd_host(h.vmax2);
    o->step = h.step;
    o->n = n_;
    o->n_surface = h.nsurf;
    o->pairs = (long long)h.pairs;
    o->pairs_total = (long long)h.pairs_total;
    o->remapped = h.remap;
    o->flags = (int)h.flags | (cap_clamped_ ? MRSPH_FLAG_CAPACITY_CLAMPED : 0);
    cap_clamped_ = false;
    o->num_cell_levels = kc_.geo.ncl;
    o->num_cells = kc_.geo.hoff[kc_.geo.ncl];
    o->max_phi = kc_.ls.max_phi;
    return 0;
  }

  int get_particles(const mrsph_particle_view* v) override {
    if (!n_) { err = "no particles"; return MRSPH_ERR_STATE; }
    struct F { void* p; int field; int vec; bool isint; };
    F fs[] = {{v->xyz, 0, 1, false}, {v->v, 1, 1, false}, {v->norm, 2, 1, false}, {v->a1, 3, 1, false},
              {v->a2, 4, 1, false}, {v->h, 5, 0, false}, {v->phi, 6, 0, false}, {v->curv, 7, 0, false},
              {v->sum, 8, 0, false}, {v->rho, 9, 0, false}, {v->nu, 10, 0, false}, {v->type, 11, 0, true},
              {v->level, 12, 0, true}};
    std::vector<double> host((size_t)3 * n_);
    for (auto& f : fs) {
      if (!f.p) continue;
      k_tap<D, R><<<grid(n_), 256, 0, st_>>>(kc_, buf_[cur_], w_, w_.slot_of_id, stage_, f.field, have_work_);
      MR_CK(cudaGetLastError());
      size_t cnt = (size_t)(f.vec ? 3 : 1) * n_;
      MR_CK(cudaMemcpyAsync(host.data(), stage_, sizeof(double) * cnt, cudaMemcpyDeviceToHost, st_));
      MR_CK(cudaStreamSynchronize(st_));
      if (f.isint) {
        int* o = (int*)f.p;
        for (size_t k = 0; k < cnt; k++) o[k] = (int)host[k];
      } else {
        std::memcpy(f.p, host.data(), sizeof(double) * cnt);
      }
    }
    return 0;
  }

  int get_cells(int* level_cell, int* sorted_ids) override {
    if (!n_) { err = "no particles"; return MRSPH_ERR_STATE; }
    std::vector<int> ck(n_), ids(n_);
    MR_CK(cudaMemcpyAsync(ck.data(), buf_[cur_].cellkey, sizeof(int) * n_, cudaMemcpyDeviceToHost, st_));
    MR_CK(cudaMemcpyAsync(ids.data(), buf_[cur_].id, sizeof(int) * n_, cudaMemcpyDeviceToHost, st_));
    MR_CK(cudaStreamSynchronize(st_));
    if (sorted_ids) std::memcpy(sorted_ids, ids.data(), sizeof(int) * n_);
    if (level_cell) {
      for (long long s = 0; s < n_; s++) {
        long long key = ck[s];
        int L = 0;
        while (L + 1 < kc_.geo.ncl && key >= kc_.geo.hoff[L + 1]) L++;
        long long r = key - kc_.geo.hoff[L];  // half cell -> reference cell
        int cx = (int)(r % kc_.geo.hn[L][0]) >> 1;
        r /= kc_.geo.hn[L][0];
        int cy = (int)(r % kc_.geo.hn[L][1]) >> 1;
        int cz = (int)(r / kc_.geo.hn[L][1]) >> 1;
        int* o = level_cell + 4 * (long long)ids[s];
        o[0] = L; o[1] = cx; o[2] = cy; o[3] = cz;
      }
    }
    return 0;
  }

  int get_neighbors(long long* off, int* nb, long long cap, long long* total) override {
    if (!have_work_) { err = "no density phase has run"; return MRSPH_ERR_STATE; }
    std::vector<int> cnt(n_), ids(n_);
    MR_CK(cudaMemcpyAsync(cnt.data(), w_.cnt, sizeof(int) * n_, cudaMemcpyDeviceToHost, st_));
    MR_CK(cudaMemcpyAsync(ids.data(), buf_[cur_].id, sizeof(int) * n_, cudaMemcpyDeviceToHost, st_));
    MR_CK(cudaStreamSynchronize(st_));
    long long tot = 0;
    std::vector<long long> byid_cnt(n_);
    for (long long s = 0; s < n_; s++) {
      if (cnt[s] > w_.cap) { err = "neighbour list spilled; raise neighbor_cap"; return MRSPH_ERR_RANGE; }
      byid_cnt[ids[s]] = cnt[s];
      tot += cnt[s];
    }
    if (total) *total = tot;
    if (!nb) return 0;
    if (cap < tot || !off) { err = "neighbour buffer too small"; return MRSPH_ERR_ARG; }
    const size_t nbl_len = (size_t)w_.cap * ((n_ + 31) / 32 * 32);
    std::vector<int> nbl(nbl_len);
    MR_CK(cudaMemcpy(nbl.data(), w_.nbl, sizeof(int) * nbl_len, cudaMemcpyDeviceToHost));
    off[0] = 0;
    for (long long k = 0; k < n_; k++) off[k + 1] = off[k] + byid_cnt[k];
    for (long long s = 0; s < n_; s++) {
      long long base = off[ids[s]];
      for (int q = 0; q < cnt[s]; q++) nb[base + q] = ids[nb_index(nbl[nb_slot(s, q, w_.cap)])];
      std::sort(nb + base, nb + base + cnt[s]);
    }
    return 0;
  }

  int upload_positions(const double* xyz) override {
    if (!n_) { err = "no particles"; return MRSPH_ERR_STATE; }
    MR_CK(cudaMemcpyAsync(stage_, xyz, sizeof(double) * 3 * n_, cudaMemcpyHostToDevice, st_));
    k_upload<D, R><<<grid(n_), 256, 0, st_>>>(kc_, buf_[cur_], stage_);
    MR_CK(cudaGetLastError());
    return 0;
  }

  int download_positions(double* xyz) override {
    if (!n_) { err = "no particles"; return MRSPH_ERR_STATE; }
    k_tap<D, R><<<grid(n_), 256, 0, st_>>>(kc_, buf_[cur_], w_, w_.slot_of_id, stage_, 0, have_work_);
    MR_CK(cudaGetLastError());
    MR_CK(cudaMemcpyAsync(xyz, stage_, sizeof(double) * 3 * n_, cudaMemcpyDeviceToHost, st_));
    MR_CK(cudaStreamSynchronize(st_));
    return 0;
  }

  int sample(long long n, const double* xyz, double* phi, double* norm, double* curv, int* tag) override {
    double *din = nullptr, *dout = nullptr;
    MR_CK(cudaMalloc(&din, sizeof(double) * 3 * n));
    MR_CK(cudaMalloc(&dout, sizeof(double) * 6 * n));
    MR_CK(cudaMemcpyAsync(din, xyz, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st_));
    k_sample_points<D, R><<<grid(n), 256, 0, st_>>>(kc_, n, din, dout);
    std::vector<double> h((size_t)6 * n);
    cudaError_t e = cudaMemcpyAsync(h.data(), dout, sizeof(double) * 6 * n, cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
    cudaFree(din);
    cudaFree(dout);
    if (e != cudaSuccess) { err = cudaGetErrorString(e); return MRSPH_ERR_CUDA; }
    for (long long i = 0; i < n; i++) {
      if (phi) phi[i] = h[6 * i];
      if (norm) for (int d = 0; d < 3; d++) norm[3 * i + d] = h[6 * i + 1 + d];
      if (curv) curv[i] = h[6 * i + 4];
      if (tag) tag[i] = (int)h[6 * i + 5];
    }
    return 0;
  }

  int sample_device(long long n, const double* d_xyz, double* d_out) override {
    k_sample_points<D, R><<<grid(n), 256, 0, st_>>>(kc_, n, d_xyz, d_out);
    MR_CK(cudaGetLastError());
    return 0;
  }

  cudaStream_t stream() const override { return st_; }
  long long num_particles() const override { return n_; }

  int world_positions(double* d_out) override {
    if (!n_) { err = "no particles"; return MRSPH_ERR_STATE; }
    k_tap<D, R><<<grid(n_), 256, 0, st_>>>(kc_, buf_[cur_], w_, w_.slot_of_id, d_out, 0, have_work_);
    MR_CK(cudaGetLastError());
    return 0;
  }

  int export_tri(double* d_xyz, int* d_type, double* d_phi, int* d_rows, int* d_cnt, int rowcap,
                 unsigned* d_flags, double* d_h = nullptr, bool sort_rows = true) override {
    if (!n_) { err = "no particles"; return MRSPH_ERR_STATE; }
    if (!have_work_) { err = "no density phase has run"; return MRSPH_ERR_STATE; }
    k_export_tri<D, R><<<grid(n_), 256, 0, st_>>>(kc_, buf_[cur_], w_, d_xyz, d_type, d_phi, d_rows, d_cnt, rowcap,
                                                   d_flags, d_h, sort_rows);
    MR_CK(cudaGetLastError());
    return 0;
  }

  int neighbor_capacity() const override { return w_.cap; }

  // The batch kernels' view of this handle (FP32-split only).
  int batch_slot(BatchSlot* out) override {
    if (!std::is_same<R, float>::value) { err = "batched kernels take FP32-split handles"; return MRSPH_ERR_ARG; }
    if (!n_) { err = "no particles"; return MRSPH_ERR_STATE; }
    BatchSlot s{};
    s.c = kc_;
    std::memcpy((void*)&s.buf[0], (const void*)&buf_[0], sizeof(Buf<float>));
    std::memcpy((void*)&s.buf[1], (const void*)&buf_[1], sizeof(Buf<float>));
    std::memcpy((void*)&s.w, (const void*)&w_, sizeof(Work<float>));
    s.ncells = ncells_;
    s.dim = D;
    s.cur = cur_;
    *out = s;
    return 0;
  }
  // nsteps whole steps ran on this handle's state in a batch launch
  void batch_advance(int nsteps) override {
    cur_ ^= (nsteps & 1);
    have_work_ = true;
  }

 private:
  static unsigned long long dbits_host(double x) { unsigned long long u; std::memcpy(&u, &x, 8); return u; }
  static double bitsd_host(unsigned long long u) { double x; std::memcpy(&x, &u, 8); return x; }
  static int grid(long long n) { return (int)((n + 255) / 256); }
  // grid of the queue kernels (density fix-up, spilled force stages): the
  // queues' lengths are known on the device only; two blocks per SM at most
  int qgrid() const { return std::max(1, std::min(grid(n_), 2 * sms_)); }

  int pre_run() {
    k_begin_step<<<1, 1, 0, st_>>>(kc_.sc, 0);
    int rc = run_map_and_bin(MAP_PRE);
    if (rc) return rc;
    // Pre_run (sph_mesh_generation.cpp:1010-1050) leaves v = 0 (Reset_particle_force)
    // and nu = 0 (Set_timestep(2) at v = 0), so the first step's
    // Update_coord_full_step moves nothing; the advection step is set to 0
    Buf<R>& b = buf_[cur_];
    MR_CK(cudaMemsetAsync(b.v1, 0, sizeof(T4) * n_, st_));
    MR_CK(cudaMemsetAsync(b.a2, 0, sizeof(T4) * n_, st_));
    MR_CK(cudaMemsetAsync(b.nu, 0, sizeof(R) * n_, st_));
    MR_CK(cudaMemsetAsync(b.nu_next, 0, sizeof(R) * n_, st_));
    MR_CK(cudaMemsetAsync(&kc_.sc->dt2, 0, sizeof(unsigned long long), st_));
    MR_CK(cudaStreamSynchronize(st_));
    have_work_ = false;
    return 0;
  }

  // map (mode) + counting sort + reorder; swaps cur_.
  int run_map_and_bin(int mode) {
    const long long n = n_;
    MR_CK(cudaMemsetAsync(w_.lhmax, 0, sizeof(unsigned) * kc_.geo.nc0 * kc_.geo.ncl, st_));
    k_map<D, R><<<grid(n), 256, 0, st_>>>(kc_, buf_[cur_], w_.counts, w_.lhmax, mode, 1000000u);
    MR_CK(cudaGetLastError());
    return bin(1);
  }

  int bin(int partial) {
    const long long n = n_;
    cell_scan(w_.counts, w_.cstart, w_.blocksums, ncells_, (int)n, st_);
    cell_scatter(buf_[cur_].cellkey, w_.counts, w_.cstart, w_.perm, n, st_);
    cell_rank(buf_[cur_].cellkey, w_.cstart, w_.perm, buf_[cur_].id, w_.perm2, n, st_);
    k_reorder<D, R><<<grid(n), 256, 0, st_>>>(buf_[cur_], buf_[cur_ ^ 1], kc_, w_.perm2, w_.slot_of_id, n, partial);
    MR_CK(cudaGetLastError());
    cur_ ^= 1;
    return 0;
  }

  // ev (optional, 8 events) brackets the timer phases MRSPH_TIMER_*.
  int launch_step(int phase, cudaEvent_t* ev = nullptr) {
    const long long n = n_;
    auto mark = [&](int k) { if (ev) cudaEventRecord(ev[k], st_); };
    mark(0);
    k_begin_step<<<1, 1, 0, st_>>>(kc_.sc, 1);
    MR_CK(cudaMemsetAsync(w_.lhmax, 0, sizeof(unsigned) * kc_.geo.nc0 * kc_.geo.ncl, st_));
    k_map<D, R><<<grid(n), 256, 0, st_>>>(kc_, buf_[cur_], w_.counts, w_.lhmax, MAP_STEP, 1000000u);
    MR_CK(cudaGetLastError());
    mark(1);
    if (phase < MRSPH_PHASE_BIN) {  // the histogram is not consumed by a scatter: clear it
      MR_CK(cudaMemsetAsync(w_.counts, 0, sizeof(int) * ncells_, st_));
      return 0;
    }
    cell_scan(w_.counts, w_.cstart, w_.blocksums, ncells_, (int)n, st_);
    mark(2);
    cell_scatter(buf_[cur_].cellkey, w_.counts, w_.cstart, w_.perm, n, st_);
    cell_rank(buf_[cur_].cellkey, w_.cstart, w_.perm, buf_[cur_].id, w_.perm2, n, st_);
    mark(3);
    k_reorder<D, R><<<grid(n), 256, 0, st_>>>(buf_[cur_], buf_[cur_ ^ 1], kc_, w_.perm2, w_.slot_of_id, n,
                                              phase < MRSPH_PHASE_FORCE2 ? 1 : 0);
    MR_CK(cudaGetLastError());
    cur_ ^= 1;
    mark(4);
    if (phase < MRSPH_PHASE_DENSITY) return 0;
    const bool wen32 = sizeof(R) == 4 && kc_.prm.kernel == K_WEN;
    if (wen32)
      k_density<D, R, (sizeof(R) == 4 ? K_WEN : -1)><<<grid(n), 256, 0, st_>>>(kc_, buf_[cur_], w_);
    else
      k_density<D, R, -1><<<grid(n), 256, 0, st_>>>(kc_, buf_[cur_], w_);
    if constexpr (std::is_same<R, float>::value) {
      // one warp per queued particle: as many warps as particles / 32
      if (wen32) k_density_fix<D, K_WEN><<<grid(n), 256, 0, st_>>>(kc_, buf_[cur_], w_);
      else k_density_fix<D, -1><<<grid(n), 256, 0, st_>>>(kc_, buf_[cur_], w_);
    }
    k_accum_pairs<<<1, 1, 0, st_>>>(kc_.sc);
    have_work_ = true;
    mark(5);
    if (phase < MRSPH_PHASE_FORCE1) return 0;
    if (wen32) {
      k_force<D, R, 1, (sizeof(R) == 4 ? K_WEN : -1)><<<grid(n), 256, 0, st_>>>(kc_, buf_[cur_], w_);
      k_force_spill<D, R, 1, (sizeof(R) == 4 ? K_WEN : -1)><<<qgrid(), 256, 0, st_>>>(kc_, buf_[cur_], w_);
    } else {
      k_force<D, R, 1, -1><<<grid(n), 256, 0, st_>>>(kc_, buf_[cur_], w_);
      k_force_spill<D, R, 1, -1><<<qgrid(), 256, 0, st_>>>(kc_, buf_[cur_], w_);
    }
    mark(6);
    if (phase < MRSPH_PHASE_FORCE2) return 0;
    if (wen32) {
      k_force<D, R, 2, (sizeof(R) == 4 ? K_WEN : -1)><<<grid(n), 256, 0, st_>>>(kc_, buf_[cur_], w_);
      k_force_spill<D, R, 2, (sizeof(R) == 4 ? K_WEN : -1)><<<qgrid(), 256, 0, st_>>>(kc_, buf_[cur_], w_);
    } else {
      k_force<D, R, 2, -1><<<grid(n), 256, 0, st_>>>(kc_, buf_[cur_], w_);
      k_force_spill<D, R, 2, -1><<<qgrid(), 256, 0, st_>>>(kc_, buf_[cur_], w_);
    }
    mark(7);
    MR_CK(cudaGetLastError());
    return 0;
  }

 public:
  int step_timed(int nsteps, double* ms) override {
    cudaEvent_t a, b;
    MR_CK(cudaEventCreate(&a));
    MR_CK(cudaEventCreate(&b));
    int rc = 0;
    if (have_work_) rc = maybe_grow_cap();  // settle the list capacity first
    if (!rc) rc = build_graphs();            // instantiate outside the timed region
    if (rc) return rc;
    const int saved = countdown_;
    countdown_ = 1 << 30;                    // no capacity checks while timing
    MR_CK(cudaEventRecord(a, st_));
    rc = step(nsteps);
    MR_CK(cudaEventRecord(b, st_));
    countdown_ = saved;
    MR_CK(cudaEventSynchronize(b));
    float f = 0.f;
    MR_CK(cudaEventElapsedTime(&f, a, b));
    *ms = f;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return rc;
  }

  int profile_steps(int nsteps, double* phase_ms, int nphase) override {
    if (!n_) { err = "no particles"; return MRSPH_ERR_STATE; }
    cudaEvent_t ev[8];
    for (int k = 0; k < 8; k++) MR_CK(cudaEventCreate(&ev[k]));
    double acc[8] = {0};
    for (int s = 0; s < nsteps; s++) {
      int rc = launch_step(MRSPH_PHASE_FORCE2, ev);
      if (rc) return rc;
      MR_CK(cudaEventSynchronize(ev[7]));
      for (int k = 0; k < 7; k++) {
        float f = 0.f;
        MR_CK(cudaEventElapsedTime(&f, ev[k], ev[k + 1]));
        acc[k] += f;
      }
    }
    for (int k = 0; k < nphase && k < 7; k++) phase_ms[k] = acc[k] / (nsteps > 0 ? nsteps : 1);
    for (int k = 0; k < 8; k++) cudaEventDestroy(ev[k]);
    return 0;
  }

 private:

  // FP32-split level-set location: per level-set level and axis, the
  // package of each anchor cell's lower corner and the corner's FP32 offset
  // inside it (computed here in FP64, once per level set)
  int anchor_tables() {
    const int lm = kc_.geo.ncl - 1;
    for (int l = 0; l < kc_.ls.nls; l++) {
      LsLevel& L = kc_.ls.lv[l];
      for (int d = 0; d < 3; d++) {
        L.anc[d] = nullptr;
        L.dpkg_f[d] = (float)L.dpkg[d];
        L.inv_dpkg_f[d] = (float)L.inv_dpkg[d];
        L.inv_dcell_f[d] = (float)L.inv_dcell[d];
        if (d >= D) continue;
        const int na = kc_.geo.n[lm][d];
        std::vector<int2> t(na);
        for (int k = 0; k < na; k++) {
          const double base = (kc_.geo.box_l[d] - L.box_l[d]) + (double)k * kc_.geo.A[d];
          const double p0 = std::floor(base / L.dpkg[d]);
          const float rem = (float)(base - p0 * L.dpkg[d]);
          t[k].x = (int)p0;
          std::memcpy(&t[k].y, &rem, sizeof(float));
        }
        int2* dv = nullptr;
        if (cudaMalloc(&dv, sizeof(int2) * na) != cudaSuccess) {
          err = "cudaMalloc failed (anchor tables)";
          return MRSPH_ERR_OOM;
        }
        anc_allocs_.push_back(dv);
        // on the engine stream (the kernels that read the table run there) and
        // complete before the host vector goes out of scope
        if (cudaMemcpyAsync(dv, t.data(), sizeof(int2) * na, cudaMemcpyHostToDevice, st_) != cudaSuccess ||
            cudaStreamSynchronize(st_) != cudaSuccess) {
          err = "cudaMemcpy failed (anchor tables)";
          return MRSPH_ERR_CUDA;
        }
        L.anc[d] = dv;
      }
    }
    return 0;
  }

  int alloc(long long n) {
    if (init_rc_) return init_rc_;
    if (n <= 0 || n > (1ll << 30)) { err = "particle count out of range"; return MRSPH_ERR_RANGE; }
    release();
    n_ = n;
    kc_.n = n;
    ncells_ = kc_.geo.hoff[kc_.geo.ncl];
    int cap = cfg_.neighbor_cap > 0 ? (cfg_.neighbor_cap + 7) / 8 * 8 : (D == 2 ? 64 : 192);
    w_.cap = cap;
    auto A = [&](void** p, size_t bytes) -> int {
      cudaError_t e = cudaMalloc(p, bytes);
      if (e != cudaSuccess) { err = std::string("cudaMalloc: ") + cudaGetErrorString(e); return MRSPH_ERR_OOM; }
      allocs_.push_back(*p);
      return 0;
    };
    int rc = 0;
    for (int k = 0; k < 2 && !rc; k++) {
      Buf<R>& b = buf_[k];
      rc |= A((void**)&b.posh, sizeof(T4) * n);
      rc |= A((void**)&b.nr, sizeof(T4) * n);
      rc |= A((void**)&b.v1, sizeof(T4) * n);
      rc |= A((void**)&b.a2, sizeof(T4) * n);
      if (sizeof(R) == 4) rc |= A((void**)&b.key, sizeof(int) * n); else b.key = nullptr;
      rc |= A((void**)&b.meta, sizeof(int) * n);
      rc |= A((void**)&b.id, sizeof(int) * n);
      rc |= A((void**)&b.nu, sizeof(R) * n);
      rc |= A((void**)&b.nu_next, sizeof(R) * n);
      rc |= A((void**)&b.phi, sizeof(R) * n);
      rc |= A((void**)&b.curv, sizeof(R) * n);
      rc |= A((void**)&b.cellkey, sizeof(int) * n);
      rc |= A((void**)&b.rec, sizeof(T4) * 2 * n);
    }
    if (!rc) {
      rc |= A((void**)&w_.sum, sizeof(R) * n);
      rc |= A((void**)&w_.a1, sizeof(T4) * n);
      rc |= A((void**)&w_.cnt, sizeof(int) * n);
      rc |= A((void**)&w_.nbl, sizeof(int) * (size_t)cap * ((n + 31) / 32 * 32));
      rc |= A((void**)&w_.pc, sizeof(R) * (size_t)cap * ((n + 31) / 32 * 32));
      rc |= A((void**)&w_.counts, sizeof(int) * ncells_);
      rc |= A((void**)&w_.lhmax, sizeof(unsigned) * kc_.geo.nc0 * kc_.geo.ncl);
      rc |= A((void**)&w_.cstart, sizeof(int) * (ncells_ + 1));
      rc |= A((void**)&w_.perm, sizeof(int) * n);
      rc |= A((void**)&w_.perm2, sizeof(int) * n);
      rc |= A((void**)&w_.blocksums, sizeof(int) * scan_blocksums_size(ncells_));
      rc |= A((void**)&w_.slot_of_id, sizeof(int) * n);
      rc |= A((void**)&w_.fixq, sizeof(int) * n);
      rc |= A((void**)&w_.spillq, sizeof(int) * n);
      rc |= A((void**)&stage_, sizeof(double) * 3 * n);
      rc |= A((void**)&kc_.sc, sizeof(DevScalars));
    }
    if (rc) { release(); return rc; }
    MR_CK(cudaMemsetAsync(w_.counts, 0, sizeof(int) * ncells_, st_));
    MR_CK(cudaMemsetAsync(w_.cnt, 0, sizeof(int) * n, st_));
    MR_CK(cudaMemsetAsync(kc_.sc, 0, sizeof(DevScalars), st_));
    cur_ = 0;
    countdown_ = 0;
    return 0;
  }

  void release() {
    drop_graphs();
    for (void* p : allocs_) cudaFree(p);
    allocs_.clear();
    n_ = 0;
    kc_.n = 0;
    kc_.sc = nullptr;
    stage_ = nullptr;
  }

  EngineConfig cfg_;
  KCtx kc_;
  cudaStream_t st_;
  Buf<R> buf_[2]{};
  Work<R> w_{};
  double* stage_ = nullptr;
  long long n_ = 0, ncells_ = 0;
  int cur_ = 0;
  bool have_work_ = false;
  int countdown_ = 0;
  cudaGraphExec_t graph_[2] = {nullptr, nullptr};
  std::vector<void*> allocs_;
  std::vector<void*> anc_allocs_;  // anchor tables, kept across re-allocations
  int init_rc_ = 0;
  int sms_ = 1;  // multiprocessors of the engine's device
  bool cap_clamped_ = false;  // a list-capacity growth fell short since the last stats
};

}  // namespace mrsph
