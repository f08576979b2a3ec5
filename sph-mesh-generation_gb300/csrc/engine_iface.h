// engine_iface.h — host-side interface between the C ABI (mrsph_api.cu) and
// the precision-specific engines (mrsph_fp64.cu, mrsph_fp32.cu).
#pragma once
#include <string>

#include "../../include/mrsph_relax.h"
#include "mrsph_common.cuh"

namespace mrsph {

struct BatchSlot;  // engine.cuh

struct EngineConfig {
  Params prm;
  CellGeo geo;
  LsSet ls;            // device pointers of the built level set
  int neighbor_cap;
  cudaStream_t stream;
};

class EngineBase {
 public:
  virtual ~EngineBase() {}
  virtual int seed(long long n) = 0;
  virtual int set_state(long long n, const mrsph_state_in* st, int pre_run) = 0;
  virtual int run_phase(int phase) = 0;
  virtual int step(int nsteps) = 0;
  virtual int step_timed(int nsteps, double* ms) = 0;
  virtual int profile_steps(int nsteps, double* phase_ms, int nphase) = 0;
  virtual int stats(mrsph_stats* out) = 0;
  virtual int get_particles(const mrsph_particle_view* v) = 0;
  virtual int get_cells(int* level_cell, int* sorted_ids) = 0;
  virtual int get_neighbors(long long* off, int* nb, long long cap, long long* total) = 0;
  virtual int upload_positions(const double* xyz) = 0;
  virtual int download_positions(double* xyz) = 0;
  virtual int sample(long long n, const double* xyz, double* phi, double* norm, double* curv, int* tag) = 0;
  // Level-set sampling between caller-owned device buffers (xyz n x 3 in,
  // out n x 6: phi, nx, ny, nz, curv, tag); enqueued on the engine stream.
  virtual int sample_device(long long n, const double* d_xyz, double* d_out) = 0;
  virtual cudaStream_t stream() const = 0;
  virtual long long num_particles() const = 0;
  // FP64 world positions in particle-id order into a device buffer (n x 3)
  virtual int world_positions(double* d_out) = 0;
  // Triangulation inputs in particle-id order: FP64 positions (n x 3), type,
  // phi, neighbour rows of the last density phase (n x rowcap ids, ascending,
  // spilled rows clamped with bit 4 set in *d_flags) and their counts;
  // d_h (optional) receives the smoothing lengths; sort_rows = false leaves
  // each row in list order (for consumers whose result is order-independent).
  virtual int export_tri(double* d_xyz, int* d_type, double* d_phi, int* d_rows, int* d_cnt, int rowcap,
                         unsigned* d_flags, double* d_h = nullptr, bool sort_rows = true) = 0;
  virtual int neighbor_capacity() const = 0;
  // Batched stepping: one step launched on the handle's stream without the
  // periodic capacity check; the step graphs built ahead of a timed region;
  // the neighbour-list capacity check a solo step makes every 32 steps (the
  // handle's stream must be idle; the graphs may be rebuilt).
  virtual int step_batched() = 0;
  virtual int prepare_steps() = 0;
  virtual int check_capacity() = 0;
  // The batch kernels' view of the handle (FP32-split engines; see BatchSlot)
  // and the bookkeeping after nsteps steps of a batch launch.
  virtual int batch_slot(BatchSlot* out) = 0;
  virtual void batch_advance(int nsteps) = 0;
  std::string err;
};

EngineBase* make_engine_fp64(const EngineConfig& cfg);
EngineBase* make_engine_fp32(const EngineConfig& cfg);

// level-set grid build (mrsph_levelset.cu)
struct LsBuildDesc {
  int D;
  int num_pkg[3], margin, n[3];
  double dcell[3];
};
cudaError_t ls_build_level(const LsBuildDesc& L, const double* d_phi, double4* g64, double* c64, float4* g32,
                           float* c32, uint8_t* tag, unsigned long long* max_phi_bits, cudaStream_t s);
// Characteristic cells of one built level (L.tag set): chr per cell (0 none,
// k + 1 segment k, -(k + 1) singularity k), mrsph_levelset.cu.
cudaError_t ls_build_characteristics(const LsLevel& L, int D, long long ntot, int* chr, const double* d_sing,
                                     int nsing, const double* d_seg, int nseg, cudaStream_t s);
// Cut-cell volume / area / mass of one built level (mrsph_levelset.cu);
// synchronises s (the CUT cells and the cut sub-cubes size the later
// passes); cnt holds 3 counters.
// ncut_listed_host = {CUT cells, CUT cells in the mass sums}.
cudaError_t ls_volume_mass(const LsSet& ls, int level, int D, double* cvol, double* carea, int* list,
                           double* part, signed char* tab, unsigned long long* cnt, double* tot,
                           long long* ncut_listed_host, cudaStream_t s);

// sort / scan primitives (mrsph_sort.cu)
void cell_scan(int* counts, int* cstart, int* blocksums, long long ncells, int ntotal, cudaStream_t s);
void cell_scatter(const int* cellkey, int* cursor, const int* cstart, int* perm, long long n, cudaStream_t s);
void cell_rank(const int* cellkey, const int* cstart, const int* perm, const int* id, int* perm2, long long n,
               cudaStream_t s);
long long scan_blocksums_size(long long ncells);

}  // namespace mrsph
