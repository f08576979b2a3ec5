// sph_mesh_generation.hpp — C++ host layer over the C ABI of mrsph_relax.h.
//
// It keeps the reference's host-side entry points for the relaxation path,
// so a C++ driver written against the reference reads the same:
//   SPH_mesh_generation (src/sph_mesh_generation/sph_mesh_generation.h:10-154):
//     Initialize_case, SPH_run_mesh_generation, Get_timestep,
//     Save_particle_post_file, Load_data_for_post;
//   Solver::SPH_Mesh_Generation_Solver (src/solver.cpp:257-321): the step loop
//     with periodic particle restarts.
// The particle state lives on the GPU; these classes own one engine handle
// each and translate its status codes into exceptions (the reference prints
// and aborts).  Workloads are built here from analytic signed-distance
// functions, as the Python workloads are (mrsph/cases.py), so the host layer
// runs without Python.
#pragma once

#include <array>
#include <cmath>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/mrsph_relax.h"

namespace mrsph_host {

// A level-set level (see mrsph_levelset_level): cell-centred phi incl.
// margins, x fastest, positive inside; active: per package incl. margins, or
// empty for all active.
struct LevelGrid {
  std::array<double, 3> box_l{{0, 0, 0}};
  std::array<double, 3> dpkg{{1, 1, 1}};
  std::array<int, 3> num_pkg{{1, 1, 1}};
  int margin = 1;
  std::vector<double> phi;
  std::vector<unsigned char> active;
};

struct Case {
  std::string name;
  mrsph_params params{};
  std::vector<LevelGrid> levels;
  long long n_particles = 0;
  int steps = 0;
  // characteristic points (x, y, z each) and segments (x1, y1, z1, x2, y2,
  // z2 each): Levelset::singularity and ::segment (level_set.h:37-41)
  std::vector<double> singularities, segments;
};

// Reference defaults (sph_mesh_generation.cpp:688-703, glbparam.h:171-183).
mrsph_params default_params(int dim);

// Samples sdf(x, y, z) at the cell centres of one level (incl. margin packages).
LevelGrid make_level(const std::function<double(double, double, double)>& sdf, int dim,
                     const std::array<double, 3>& box_l, const std::array<double, 3>& dpkg,
                     const std::array<int, 3>& num_pkg, int margin = 1);

// Particle count from the spacing integral over phi > 0 of the finest level
// (the reference's total_mass = sum vol / scale^D, lset_package.cpp:1283-1397,
// without the cut-cell refinement), tanh spacing law.
long long particle_count(const std::vector<LevelGrid>& levels, const mrsph_params& p);

// True when the reference's level plan (sph.cpp:144-180) gives every cell-list
// level a cell of max_scale / 2^l (the library rejects other domains).
bool cell_levels_consistent(const double* box_l, const double* box_r, int dim, double max_scale,
                            double min_scale);

// Unit square minus a disc (r = 0.2 at (0.5, 0.5)), constant spacing.
Case disc_hole_2d(double spacing = 0.01, int grid = 256, int kernel = MRSPH_KERNEL_WENDLAND,
                  double h_over_dx = 1.3, int precision = MRSPH_FP64_PLAIN, unsigned long long seed = 0);
// Inside of a torus (R = 1, r = 0.35) on nested level sets, tanh spacing law.
Case torus_3d(double dx_min = 0.005, double dx_max = 0.02, int kernel = MRSPH_KERNEL_WENDLAND,
              double h_over_dx = 1.3, int precision = MRSPH_FP32_SPLIT, unsigned long long seed = 0,
              int fine_pkg = 64, int nlevels = 3);

// The box [lo_b, hi_b]^dim of a unit domain with margins: phi is the
// distance to the nearest face inside, its corners are singularity points
// and, in 3D with edges, its 12 edges are segments.  Constant spacing.
Case box_with_corners(int dim = 3, double spacing = 0.04, int grid = 32, int kernel = MRSPH_KERNEL_HYPERBOLIC,
                      double h_over_dx = 1.0, int precision = MRSPH_FP64_PLAIN, unsigned long long seed = 0,
                      double lo_b = 0.1, double hi_b = 0.9, bool edges = true);

class Error : public std::runtime_error {
 public:
  Error(int code, const std::string& what) : std::runtime_error(what), code(code) {}
  int code;
};

class SPH_mesh_generation {
 public:
  // The constructor and the level-set set-up of Initialize_case
  // (sph_mesh_generation.cpp:8-152, 594-712): engine handle, level-set build.
  explicit SPH_mesh_generation(const Case& c, int device = 0);
  ~SPH_mesh_generation();
  SPH_mesh_generation(const SPH_mesh_generation&) = delete;
  SPH_mesh_generation& operator=(const SPH_mesh_generation&) = delete;

  // Random_particle_distribution + Pre_run (sph_mesh_generation.cpp:1302-1367,
  // 1010-1050); n < 0 takes the case's particle count.
  void Initialize_case(long long n = -1);
  // Levelset::Calculate_total_volume_mass (level_set.cpp:930-972) on one
  // level (< 0: the finest): cut-cell volumes, surface areas, masses and the
  // particle numbers of Get_num_particles (sph_mesh_generation.cpp:900-940).
  mrsph_volume_mass_stats Calculate_total_volume_mass(int level = -1);
  // The reference's particle count (glbl_total_num_particle) of that level.
  long long Get_num_particles(int level = -1) { return Calculate_total_volume_mass(level).num_particle; }
  // SPH_run_mesh_generation x nsteps (sph_mesh_generation.cpp:1371-1463).
  void SPH_run_mesh_generation(int nsteps = 1);
  // glbl_timestep after the last step (SPH::Get_timestep, sph.cpp:224-227).
  double Get_timestep();
  mrsph_stats Stats();
  // Particle positions in id order, n x 3.
  std::vector<double> Positions();
  // rstfile_particles/step_<run_time>_rank_0.pst and list.csv under root
  // (Save_particle_post_file, sph_mesh_generation.cpp:2624-2660).
  std::string Save_particle_post_file(const std::string& root, long long run_time, bool first);
  // Positions of a .pst file as the state (Load_data_for_post,
  // sph_mesh_generation.cpp:426-590); with pre_run the map and Pre_run follow.
  void Load_data_for_post(const std::string& pst, bool pre_run = true);

  // One step up to and including a phase (MRSPH_PHASE_*), the groups of the
  // reference's per-particle methods in step order: MAP = Update_coord_full_step,
  // Get_particle_info, Find_and_map_particle, Set_particle_scale; BIN = the
  // cell binning of Prepare_for_the_current_step; DENSITY = neighbour search and
  // Get_kernel_summation; FORCE1 / FORCE2 = Accumulate_particle_force (1 / 2)
  // with Set_timestep and the half-step kicks (sph_mesh_generation.cpp:1371-1463).
  void Run_phase(int phase);

  // Centroidal Voronoi partition of the particles (mass 1), Voronoi::
  // Partitioning (CVP/voronoi.cpp:1376-1446): vp (K x 3) holds the initial
  // VPs and receives the final ones; labels (n, id order) and vp_mass (K).
  mrsph_cvp_result Partitioning(std::vector<double>& vp, const mrsph_cvp_params& p, std::vector<int>* labels = nullptr,
                                std::vector<double>* vp_mass = nullptr);
  // The level-set partition of weighted points with ghost VPs, Voronoi_lset::
  // Partitioning_for_initial_VP_distribution (CVP/voronoi_lset.cpp:824-889);
  // labels -1 for points nearest a ghost; ghosts receive the last
  // iteration's ghost VPs (x, y, z each).
  mrsph_cvp_result Partitioning_for_initial_VP_distribution(const std::vector<double>& xyz,
                                                            const std::vector<double>& mass,
                                                            const std::vector<double>& mass_surface,
                                                            std::vector<double>& vp, const mrsph_cvp_params& p,
                                                            std::vector<int>* labels = nullptr,
                                                            std::vector<double>* vp_mass = nullptr,
                                                            std::vector<double>* ghosts = nullptr);

  // The tet mesh of the current particles (3D): Graphmeshcls::Reconstruct_tets
  // (geometry_tools/graph_mesh.cpp:981-1100) with Tet_quality_statistics
  // (:1967-2400) over mrsph_tetrahedralize; tets receives 4 ascending ids per tet.
  mrsph_tet_quality Reconstruct_tets(std::vector<int>& tets);

  long long num_particles() const { return n_; }
  mrsph_handle* handle() { return h_; }
  const Case& Get_case() const { return case_; }
  // Per-particle arrays of the writers in id order: type, h, normal (n x 3)
  // and neighbour counts of the last density pass (self included).
  void Particle_fields(std::vector<int>& type, std::vector<double>& h, std::vector<double>& norm,
                       std::vector<int>& nn);

 private:
  void check(int rc, const char* what);
  mrsph_handle* h_ = nullptr;
  Case case_;
  long long n_ = 0;
};

// System parameters (Initialization, src/system.cpp:12-32): the run spans
// [start_time, end_time) in steps, with an output every output_dt steps.
struct Initialization {
  double start_time = 0.0;
  double end_time = 20000;
  double output_dt = 100;
  int Get_num_timestep() const { return (int)std::ceil((end_time - start_time) / output_dt); }
  double Get_start_time() const { return start_time; }
  double Get_dt() const { return output_dt; }
};

// Solver::SPH_Mesh_Generation_Solver (src/solver.cpp:257-321): total_steps
// relaxation steps, a particle restart every output_interval steps (and at
// the end) when output_root is not empty.  Returns the device-timed
// milliseconds of the steps.
class Solver {
 public:
  explicit Solver(SPH_mesh_generation& sim) : sim_(sim) {}
  // With VTU output on, every output also writes the particle VTU series
  // (Particle_binary_writer) under <output_root>/outdata.
  void Set_vtu_output(bool on) { write_vtu_ = on; }
  double SPH_Mesh_Generation_Solver(int total_steps, int output_interval = 0, const std::string& output_root = "");
  // Solver::Load_solver (src/solver.cpp:35-101) for the relaxation path:
  // Get_num_timestep() outputs, Get_dt() steps apart, with a particle restart
  // at each.  Returns the device-timed milliseconds of the steps.
  double Load_solver(const Initialization& ini, const std::string& output_root = "");

 private:
  SPH_mesh_generation& sim_;
  bool write_vtu_ = false;
  int n_out_ = 0;
};

// Particle_binary_writer (particle_binary_writer.cpp:12-400) with the
// reference's default fields (id, local_id, type, h, NN, color, norm): per
// output n, outdir/particle_rank_0_step_<n>.vtu (VTK XML UnstructuredGrid,
// raw appended little-endian arrays, each preceded by its UInt32 byte
// count), particle_step_<n>.pvtu and the particle.pvd collection.
struct ParticleFields {
  long long n = 0;
  const double* xyz = nullptr;   // n x 3
  const int* type = nullptr;
  const double* h = nullptr;
  const int* nn = nullptr;       // neighbour count of the last density pass, self included
  const double* norm = nullptr;  // n x 3
};
std::string particle_vtu(const ParticleFields& f);
// Mesh_binary_writer (mesh_binary_writer.cpp:36-390) for the 2D triangle
// mesh: the particle point fields, one triangle cell per triangle and the
// cell fields 'vol' (area) and 'aspect' (longest / shortest edge).
std::string mesh_vtu(const ParticleFields& f, long long ntri, const int* tris);
// Its 3D branch (mesh_binary_writer.cpp:392-640): one VTK_TETRA cell per tet
// and the cell fields 'vol', 'aspect' (longest edge / smallest height),
// 'radius_ratio' (3 r_in / r_circ) and 'mindihedangle' (degrees).
std::string tet_mesh_vtu(const ParticleFields& f, long long ntet, const int* tets);
std::string particle_pvtu(const std::string& piece);
std::string mesh_pvtu(const std::string& piece, bool tets = false);
// Rewrites outdir/<name>.pvd with one DataSet entry per output so far
// (Output_pvd_file, particle_binary_writer.cpp:53-93); n_out = 0 starts it.
void update_pvd(const std::string& path, int n_out, const std::string& timestep, const std::string& dataset);

// Level-set restart rstfile/levelset.rst of one level (Save_restart_file,
// sph_mesh_generation.cpp:2671-2736; Save_lset_restart_file,
// level_set.cpp:1022-1094; Write_level_set_rstfile,
// lset_level_infor.cpp:695-929), little-endian: the same bytes as the Python
// writer (mrsph/io.py save_lset_restart).
struct LsetRestart {
  int dim = 3;
  std::array<double, 3> box_l{{0, 0, 0}}, box_r{{0, 0, 0}};
  std::array<int, 3> num_pkg{{1, 1, 1}}, margin{{0, 0, 0}};
  std::array<double, 3> dpkg{{1, 1, 1}}, dcell{{1, 1, 1}};
  double fac_max = 0, fac_mid = 0, fac_min = 0, curv_artificial = 0;
  double total_mass = 0, total_mass_surface = 0, total_volume = 0, total_area = 0;
  double total_mass_segment = 0, total_length = 0;
  double max_phi = 0, max_dl = 0, mid_dl = 0, min_dl = 0, max_curv = 0, min_curv = 0;
  int num_interface_cell = 0;
  // characteristic points (3 doubles each) and segments (6 doubles each)
  std::vector<double> sing, seg;
  // interior cells, x fastest; chr_tag / chr_idx empty = NORMAL / -1
  std::vector<double> phi, nx, ny, nz, curv, scale;
  std::vector<int> tag, chr_tag, chr_idx;
};
std::string lset_restart_bytes(const LsetRestart& r);
// Gathers the record of one level (< 0: the finest) from the engine and
// writes it to path.
std::string Save_lset_restart(SPH_mesh_generation& sim, const std::string& path, int level = -1);
// Reads a level-set restart of one level, the bytes lset_restart_bytes
// writes (Load_rst_case, sph_mesh_generation.cpp:323-414, with
// Load_lset_restart_file, level_set.cpp:1098-1175, and
// Load_level_set_rstfile, lset_level_infor.cpp:932-1080); throws Error on a
// short, oversized or inconsistent file.
LsetRestart Load_lset_restart(const std::string& path);
// Get_num_particles (sph_mesh_generation.cpp:900-930) over a level set's
// totals: one particle per singularity point; segment, surface and interior
// counts each less half the next-lower-dimensional mass, truncated and at
// least 0; the surface count at most the number of interface cells.
long long restart_num_particles(double total_mass, double total_mass_surface, double total_mass_segment,
                                int num_singularity, int num_interface_cell);
// A runnable case from a level-set restart (the reference's restart run):
// the file's domain, spacing bounds, middle spacing, characteristic points
// and segments, and one level-set level whose interior cells hold the file's
// phi.  The reference fills the margin packages from its analytic geometry;
// here a margin cell holds the nearest interior cell's phi minus its
// distance to that cell.  The count is restart_num_particles of the file's
// totals.  retarget (3 factors, may be NULL; kRetargetFactors are the
// reference's) is the restart run that re-targets the spacing
// (_READ_TARGET_FIELD_, sph_mesh_generation.cpp:658-666): minimum, middle and
// maximum spacing become the factors times the level's cell size
// (level_set.cpp:939-941) and the count the spacing integral of the new law
// (particle_count: the tanh law; with scale_law 1 seed the cut-cell count).
// Throws Error when the domain and spacing give an inconsistent cell-list
// level plan.
constexpr double kRetargetFactors[3] = {2.0, 5.0, 16.0};
Case case_from_lset_restart(const LsetRestart& r, int kernel = MRSPH_KERNEL_WENDLAND, double h_over_dx = 1.3,
                            int precision = MRSPH_FP32_SPLIT, unsigned long long seed = 0, int scale_law = 0,
                            const double* retarget = nullptr);

class Mesh_binary_writer {
 public:
  explicit Mesh_binary_writer(const std::string& outdir = "outdata") : outdir_(outdir) {}
  // 2D: triangulates the current particles (mrsph_triangulate) and writes
  // outdir/mesh_tris_rank_0_step_<n>.vtu, mesh_tris_step_<n>.pvtu and
  // mesh_tris.pvd; 3D: tetrahedralises them (mrsph_tetrahedralize) and
  // writes mesh_tets_rank_0_step_<n>.vtu, mesh_tets_step_<n>.pvtu and
  // mesh_tets.pvd.  Returns the piece's path.
  std::string Output_mesh(int n_out, SPH_mesh_generation& sim, long long run_time = -1);

 private:
  std::string outdir_;
};

class Particle_binary_writer {
 public:
  explicit Particle_binary_writer(const std::string& outdir = "outdata") : outdir_(outdir) {}
  // Output_vtu_file / Output_pvtu_file / Output_pvd_file of output n_out; the
  // timestep entry is run_time (the completed steps when negative).  Returns
  // the piece's path.
  std::string Output_particle(int n_out, SPH_mesh_generation& sim, long long run_time = -1);

 private:
  std::string outdir_;
};

// Level_set_binary_writer (lset_binary_writer.cpp:12-510) for one level:
// outdir/mesh_lset_rank_0_step_<n>.vti (VTK XML ImageData over the level's
// interior cells, raw appended arrays) with phi, curv and scale at the cell
// corners (the mean of the 2^D cells around each corner) and per cell the
// cut-cell tag 'interface', the characteristic tag 'char' (none here), the
// cut-cell volume 'vol' and area 'area' (mrsph_volume_mass), its
// mesh_lset_step_<n>.pvti and the mesh_lset.pvd collection.
struct ImageField {
  std::string name, type;  // type "Float32" or "Int32"
  std::string raw;         // little-endian values, x fastest
};
std::string vti_bytes(const std::array<int, 3>& ncell, const std::array<double, 3>& origin,
                      const std::array<double, 3>& spacing, const std::vector<ImageField>& point_data,
                      const std::vector<ImageField>& cell_data);
// Shortest round-trip decimal of a double, written the way Python's repr writes it.
std::string repr_double(double v);

class Level_set_binary_writer {
 public:
  explicit Level_set_binary_writer(const std::string& outdir = "outdata") : outdir_(outdir) {}
  std::string Output_lset(int n_out, SPH_mesh_generation& sim, int level = 0, long long run_time = -1);

 private:
  std::string outdir_;
};

// .pst restart files: int32 count, then x, y, z (float64) per particle.
void write_pst(const std::string& path, const std::vector<double>& xyz);
std::vector<double> read_pst(const std::string& path);

}  // namespace mrsph_host
