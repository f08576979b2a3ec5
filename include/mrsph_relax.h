/*
 * mrsph_relax.h — C ABI of the GB300 relaxation engine (adaptive SPH particle
 * relaxation driven by a level set, the data-parallel core of the SPH mesh
 * generator Xiangyu-Hu/SPH-mesh-generation).
 *
 * The reference has no plugin or FFI layer: its hot path sits behind the C++
 * class SPH_mesh_generation (src/sph_mesh_generation/sph_mesh_generation.h:10-154)
 * and the per-particle methods of Particle_mesh_generation
 * (src/sph_mesh_generation/particle_mesh_generation.h:78-120), called from
 * Solver (src/solver.cpp:35-321).  Each entry point below names the reference
 * member it replaces.
 *
 * Conventions: every function returns 0 on success or a negative MRSPH_ERR_*
 * code; mrsph_last_error() gives the message.  No exception crosses the ABI.
 * The library owns all device memory; results are copied into caller buffers
 * (host memory, particle-id order).  One host thread per handle; handles are
 * independent.  All pointers are plain host pointers.
 */
#ifndef MRSPH_RELAX_H
#define MRSPH_RELAX_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MRSPH_API_VERSION 1

/* status codes */
#define MRSPH_OK 0
#define MRSPH_ERR_ARG (-1)     /* invalid argument */
#define MRSPH_ERR_CUDA (-2)    /* CUDA runtime error */
#define MRSPH_ERR_STATE (-3)   /* call out of order (e.g. no level set yet) */
#define MRSPH_ERR_OOM (-4)     /* device allocation failed */
#define MRSPH_ERR_RANGE (-5)   /* size beyond a documented limit */
#define MRSPH_ERR_DEVICE (-6)  /* a device-side check failed (see stats.flags) */

/* kernels (Makefile.in:36-40) */
#define MRSPH_KERNEL_HYPERBOLIC 0
#define MRSPH_KERNEL_CUBIC 1
#define MRSPH_KERNEL_WENDLAND 2 /* the reference's _WINDLAND_C4_ (Wendland C2 form) */
#define MRSPH_KERNEL_GAUSSIAN 3
#define MRSPH_KERNEL_QUINTIC 4

/* precision modes */
#define MRSPH_FP64_PLAIN 0 /* absolute FP64 positions, FP64 arithmetic */
#define MRSPH_FP32_SPLIT 1 /* int cell key + FP32 offset, FP32 arithmetic, FP64 reductions */

/* particle types (glbparam.h:53-60) */
#define MRSPH_REAL 0
#define MRSPH_SURFACE 1
#define MRSPH_SINGULARITY 2
#define MRSPH_SEGMENT 3

/* device-side flags reported in mrsph_stats.flags */
#define MRSPH_FLAG_REMAP_EXHAUSTED 1 /* a re-seed loop hit its attempt limit */
#define MRSPH_FLAG_SEED_EXHAUSTED 2  /* a seeding loop hit its attempt limit */
#define MRSPH_FLAG_LEVEL_CLAMPED 4   /* a particle scale left the planned cell-list levels */
#define MRSPH_FLAG_NEIGHBOR_SPILL 8  /* a neighbour list exceeded its capacity (handled by re-scan) */
#define MRSPH_FLAG_CAPACITY_CLAMPED 16 /* host side: the list capacity could not grow to the largest
                                          list (memory budget or allocation), so lists keep spilling */

/* run_phase selectors (a step is MAP -> BIN -> DENSITY -> FORCE1 -> FORCE2) */
#define MRSPH_PHASE_MAP 1
#define MRSPH_PHASE_BIN 2
#define MRSPH_PHASE_DENSITY 3
#define MRSPH_PHASE_FORCE1 4
#define MRSPH_PHASE_FORCE2 5

typedef struct mrsph_handle mrsph_handle;

/* Run parameters.  Replaces the compile-time flags of Makefile.in:14-195 and
 * the constants hard-coded in SPH_mesh_generation::SPH_mesh_generation /
 * Initialize_case (sph_mesh_generation.cpp:8-152, 680-712). */
typedef struct {
  int dim;              /* 2 or 3 */
  int kernel;           /* MRSPH_KERNEL_* */
  int precision;        /* MRSPH_FP64_PLAIN or MRSPH_FP32_SPLIT */
  double cell_ratio;    /* CELL_RATIO: h = scale*cell_ratio/cutoff (glbparam.h:171-183) */
  double cutoff;        /* CUT_OFF (2.0) */
  double angle_thres;   /* surface-neighbour angle threshold, rad (reference 0.4*PI) */
  double nu_coeff;      /* artificial viscosity coefficient (reference 0.1) */
  double damp_coeff;    /* velocity damping (reference 0) */
  double min_dl;        /* minimum target spacing (Levelset::minimum_dl) */
  double max_dl;        /* maximum target spacing (Levelset::maximum_dl) */
  double box_l[3];      /* domain (SPH::box_l, box_r) = level-set level-0 interior box */
  double box_r[3];
  unsigned long long seed; /* Philox4x32-10 key for seeding and re-seeding */
  int neighbor_cap;     /* neighbour-list capacity per particle (rounded up to a multiple of 8); 0 = automatic */
  int device;           /* CUDA device ordinal */
  int scale_law;        /* target spacing: 0 = the reference's tanh law of phi (Levelset::Get_scale,
                           level_set.cpp:311-351); 1 = curvature law: at the surface from min_dl
                           (largest |curvature| of the cut cells) to middle_dl (smallest), then the
                           tanh law of phi up to max_dl */
  double middle_dl;     /* middle spacing of law 1; <= 0: 5 x the level-0 level-set cell (middel_dl) */
} mrsph_params;

/* One level of a (possibly nested) level set: packages of 4^D cells covering
 * [box_l, box_l + num_pkg*dpkg) plus `margin` packages on every side
 * (Levelset_levelinfo::Initialize, lset_level_infor.cpp:17-117).  phi holds
 * cell-centred values incl. margins, x fastest, positive inside the body.
 * active (optional, one byte per package incl. margins, x fastest) marks the
 * packages a finer nested level covers; NULL = all packages active. */
typedef struct {
  double box_l[3];
  double dpkg[3];
  int num_pkg[3];
  int margin;
  const double* phi;
  const unsigned char* active;
} mrsph_levelset_level;

typedef struct {
  double dt;          /* glbl_timestep after the last step (stage 2) */
  double dt_stage1;   /* glbl_timestep of stage 1 of the last step */
  double max_v;       /* glbl_max_v of the last step (stage 2) */
  long long step;     /* completed relaxation steps */
  long long n;        /* particles */
  long long n_surface;/* SURFACE particles after the last map phase */
  long long pairs;    /* ordered neighbour pairs i != j of the last step */
  long long remapped; /* REAL particles re-seeded into phi > h by the last map phase */
  long long pairs_total; /* ordered neighbour pairs summed over all steps since seeding */
  int flags;          /* MRSPH_FLAG_* accumulated since the last mrsph_get_stats */
  int num_cell_levels;/* cell-list levels in use */
  long long num_cells;/* entries of the sort table (half-size cell-list cells, all levels) */
  double max_phi;     /* maximum phi of the level set (Levelset::maximum_phi) */
} mrsph_stats;

/* Host views for particle taps, particle-id order; any pointer may be NULL.
 * Vectors are n x 3 (z = 0 in 2D). */
typedef struct {
  double* xyz;
  double* v;
  int* type;
  double* h;
  int* level;   /* cell-list level (0 = coarsest) */
  double* phi;
  double* curv;
  double* norm;
  double* sum;  /* inverse kernel sum of the last density phase */
  double* rho;
  double* nu;
  double* a1;   /* stage-1 acceleration of the last step */
  double* a2;   /* stage-2 acceleration of the last step */
} mrsph_particle_view;

/* State injection for parity runs (particle-id order).  v, nu, h may be NULL
 * (zero); level NULL = coarsest level (Particle_mesh_generation::Initialize). */
typedef struct {
  const double* xyz;
  const double* v;
  const int* type;
  const double* h;
  const int* level;
  const double* nu;
  double dt;          /* glbl_timestep used by the next advection */
  long long step;     /* completed steps (drives the re-seed random stream) */
} mrsph_state_in;

int mrsph_version(void);

/* SPH_mesh_generation constructor + Define_level_infor_tight (sph.cpp:144-180). */
int mrsph_create(const mrsph_params* params, mrsph_handle** out);
int mrsph_destroy(mrsph_handle* h);
/* Last error message of the handle (or of the last failed mrsph_create when h is NULL). */
int mrsph_last_error(mrsph_handle* h, char* buf, size_t len);

/* Levelset::Initialize + Calculate_level_set (level_set.cpp:51-88, 238-307):
 * copies phi to the device and builds normals, cut-cell tags, curvature and
 * maximum phi there.  nlevels <= 4, finest last. */
int mrsph_set_levelset(mrsph_handle* h, int nlevels, const mrsph_levelset_level* levels);
/* The geometry's characteristic points and segments (Levelset::singularity,
 * ::segment, level_set.h:37-41; the counts and coordinates that Levelset's
 * restart file carries, level_set.cpp:1053-1070).  sing holds nsing points
 * as (x, y, z) and seg holds nseg segments as (x1, y1, z1, x2, y2, z2); z is
 * ignored in 2D.  Must come before mrsph_set_levelset.  That call then tags
 * each level's characteristic cells on the device: Get_singularity_tag
 * (lset_package.cpp:515-555), where the interface cell (tag not NORMAL)
 * whose centre is nearest each point, among the cells of the point's
 * package, becomes a SINGULARITY cell, and Get_segment_tag
 * (lset_package.cpp:559-585), where every other interface cell whose box a
 * segment meets becomes a SEGMENT cell (the first such segment).  Particles in those cells are mapped onto the
 * point (MRSPH_SINGULARITY) or the segment's line (MRSPH_SEGMENT), as in
 * particle_mesh_generation.cpp:439-465.  Counts up to 2^20 each; both zero
 * clears them. */
int mrsph_set_characteristics(mrsph_handle* h, int nsing, const double* sing, int nseg, const double* seg);
/* Tap: the characteristic tag of every cell of one level (sized like phi):
 * 0 for a NORMAL cell, k + 1 for a SEGMENT cell of segment k, -(k + 1) for
 * the SINGULARITY cell of point k (tag_characteristic and
 * idx_characteristic of Levelset_cell, in one int). */
int mrsph_get_characteristics(mrsph_handle* h, int level, int* chr);
/* Tap: the device-built fields of one level (arrays sized like phi; NULL skips). */
int mrsph_get_levelset(mrsph_handle* h, int level, double* nx, double* ny, double* nz, double* curv,
                       unsigned char* tag, double* max_phi);
/* Cut-cell volume, surface area and particle numbers of one level-set level
 * (level < 0: the finest): Levelset::Calculate_total_volume_mass
 * (level_set.cpp:930-972) over Levelset_package::Calculate_volume_mass
 * (lset_package.cpp:1283-1397) and GeometryCalculator
 * (geometry_calculator.cpp:12-570), then
 * SPH_mesh_generation::Get_num_particles (sph_mesh_generation.cpp:900-940),
 * with the segment and singularity terms of a geometry given by
 * mrsph_set_characteristics: in 3D a SEGMENT cell adds the length of its
 * segment inside the cell box (GeometryCalculator::Get_segment_length,
 * geometry_calculator.cpp:571-589, over AABB_calculator.cpp:6-55) over its
 * scale to total_mass_segment.  A cell counts when phi > 0 or
 * |phi| < dl (the level's smallest cell size); CUT cells take their volume
 * fraction from adaptive bisection and their area from marching cubes.
 * cell_vol / cell_area (may be NULL) receive per-cell values sized like phi
 * (zero outside the counted cells). */
typedef struct {
  double total_mass;          /* sum of vol / scale^D (Levelset::total_mass) */
  double total_mass_surface;  /* sum over CUT cells of area / scale^(D-1) */
  double total_volume;
  double total_area;
  long long num_interface_cell;   /* CUT cells (glbl_num_interface_cell) */
  long long num_particle_mesh;    /* max(int(total_mass - total_mass_surface / 2), 0) */
  long long num_particle_surface; /* min(int(total_mass_surface), num_interface_cell) */
  long long num_particle;         /* mesh + surface + segment + singularity (glbl_total_num_particle) */
  double device_ms;           /* device time of the pass */
  double total_mass_segment;  /* 3D: sum over SEGMENT cells of length / scale (Levelset::total_mass_segment) */
  double total_length;        /* 3D: sum of those lengths (Levelset::total_length) */
  long long num_particle_segment;     /* max(int(total_mass_segment - 0.5 x singularity points), 0) */
  long long num_particle_singularity; /* the geometry's singularity points */
} mrsph_volume_mass_stats;
int mrsph_volume_mass(mrsph_handle* h, int level, mrsph_volume_mass_stats* out, double* cell_vol,
                      double* cell_area);
/* Levelset::Get_phi_at_position / Calculate_particle_infor (level_set.cpp:372-436,
 * particle_mesh_generation.cpp:175-265) at n host points (xyz n x 3). */
int mrsph_sample_levelset(mrsph_handle* h, long long n, const double* xyz, double* phi, double* norm,
                          double* curv, int* tag);

/* No counterpart in the reference.  Same results as mrsph_sample_levelset for
 * callers that cannot allocate device memory (cudaMalloc synchronises the
 * device and may be forbidden where another allocator owns the memory or on a
 * latency-critical path): points and results are staged through a fixed
 * scratch array that is part of the library image (held on every GPU that
 * loads the library until exit).  At most 65536 points per call, else
 * MRSPH_ERR_RANGE.  The first call on a device looks up the scratch address
 * and keeps it for the life of the process; make that first call before any
 * stream capture, and do not reset the device (cudaDeviceReset) while the
 * library is loaded.  Every call is synchronous: it returns with the results
 * in the caller's arrays.  All calls on a device share the scratch: calls that
 * overlap on the GPU race. */
int mrsph_sample_levelset_noalloc(mrsph_handle* h, long long n, const double* xyz, double* phi, double* norm,
                                  double* curv, int* tag);

/* Random_particle_distribution (sph_mesh_generation.cpp:1302-1367) + Pre_run
 * (:1010-1050): n particles seeded where phi > h. */
int mrsph_seed(mrsph_handle* h, long long n);
/* Parity entry: particles from given positions (e.g. a reference .pst file),
 * optionally with full state; runs Pre_run when pre_run != 0. */
int mrsph_set_state(mrsph_handle* h, long long n, const mrsph_state_in* st, int pre_run);

/* SPH_run_mesh_generation x nsteps (sph_mesh_generation.cpp:1371-1463),
 * asynchronous on the handle's stream, CUDA-graph replayed. */
int mrsph_step(mrsph_handle* h, int nsteps);
/* One step up to and including `phase` (MRSPH_PHASE_*), for phase-by-phase parity. */
int mrsph_run_phase(mrsph_handle* h, int phase);
int mrsph_sync(mrsph_handle* h);
/* mrsph_step timed on the device: CUDA events recorded on the handle's stream
 * around the graph launches; *ms = elapsed device milliseconds (synchronises). */
int mrsph_step_timed(mrsph_handle* h, int nsteps, double* ms);
/* Per-phase device time of nsteps eagerly launched steps (the reference's
 * time_for_* timers, sph_mesh_generation.cpp:1373-1454).  phase_ms[k] receives
 * the mean milliseconds per step of phase k (MRSPH_TIMER_*), nphase <= 8. */
#define MRSPH_TIMER_MAP 0     /* begin + advect/sample/map/spacing/key */
#define MRSPH_TIMER_SCAN 1    /* cell histogram scan */
#define MRSPH_TIMER_SORT 2    /* scatter + in-cell rank */
#define MRSPH_TIMER_REORDER 3
#define MRSPH_TIMER_DENSITY 4 /* neighbour search + kernel sum */
#define MRSPH_TIMER_FORCE1 5
#define MRSPH_TIMER_FORCE2 6
#define MRSPH_NUM_TIMERS 7
int mrsph_profile_steps(mrsph_handle* h, int nsteps, double* phase_ms, int nphase);

int mrsph_get_stats(mrsph_handle* h, mrsph_stats* out);
int mrsph_get_particles(mrsph_handle* h, const mrsph_particle_view* view);
/* Cell binning tap: per particle (id order) level, cx, cy, cz (n x 4 ints);
 * sorted_ids (n ints) = particle ids in device storage order: levels in
 * turn, half cells (dcell/2) row-major within a level, ascending id inside a
 * half cell.  Either pointer may be NULL. */
int mrsph_get_cells(mrsph_handle* h, int* level_cell, int* sorted_ids);
/* Neighbour lists of the last density phase in CSR form, particle-id order,
 * neighbour ids ascending.  Call with nb == NULL to get *total only. */
int mrsph_get_neighbors(mrsph_handle* h, long long* offsets, int* nb, long long cap, long long* total);

/* Centroidal Voronoi partitioning (row A13): Voronoi::Partitioning
 * (src/CVP/voronoi.cpp:1376-1446) with Get_CPU_id assignment (:480-493),
 * mass / mass-centre / energy sums (:617-631), face-pressure step
 * Update_position (:830-897), Lloyd step Update_position_CVT (:901-992) and
 * the convergence test Check_partition_error (:1228-1262).  voro++ faces are
 * replaced by exact in-box Voronoi faces computed on the GPU. */
typedef struct {
  int num_vp;             /* K partitions, 1..1024 */
  int max_iter;           /* Max_iterate_number (reference 4000; 800 for level-set packages) */
  int pressure_step;      /* 1: face-pressure move before the Lloyd step (reference); 0: Lloyd only */
  double error_tolerance; /* reference 0.05 */
  double relax_ratio;     /* initial relax ratio (reference 0.8) */
} mrsph_cvp_params;

typedef struct {
  int iterations;
  int converged;
  double error_max;     /* max |mass - target| / target of the last iteration */
  double total_energy;  /* sum of mass x distance to the VP */
} mrsph_cvp_result;

/* Partition the handle's particles (mass 1).  vp_xyz (K x 3) holds the
 * initial VP positions and receives the final ones; labels (n, id order) and
 * vp_mass (K) may be NULL. */
int mrsph_cvp(mrsph_handle* h, const mrsph_cvp_params* p, double* vp_xyz, int* labels, double* vp_mass,
              mrsph_cvp_result* res);
/* Same on given host points with masses (e.g. level-set package centres with
 * their total mass, Voronoi_lset); mass NULL = 1.  The box is the handle's domain. */
int mrsph_cvp_points(mrsph_handle* h, long long n, const double* xyz, const double* mass,
                     const mrsph_cvp_params* p, double* vp_xyz, int* labels, double* vp_mass,
                     mrsph_cvp_result* res);
/* Level-set partition with ghost VPs: Voronoi_lset::
 * Partitioning_for_initial_VP_distribution (src/CVP/voronoi_lset.cpp:824-889)
 * on weighted points (the level set's package centres with their total mass
 * and surface mass, lset_package.cpp:1283-1397).  The points start coloured
 * by their nearest VP (Voronoi_lset::Initialize, :147-169).  Each iteration
 * first mirrors, in VP order, every VP k > 0 whose points include one with
 * surface mass across the surface: x - 2 phi n, with phi and the
 * interpolated normal at the VP on the handle's level set, when phi >= 1e-6
 * (Ghost_VP_generation, :250-308; the reference's colour > 0 test leaves VP 0
 * out).  The ghosts then take part in the assignment: a point nearest a
 * ghost belongs to no VP (label -1).  They also bound the VPs' cells like
 * walls: a face with a ghost takes the VP's own pressure (:555-594).  The
 * rest is mrsph_cvp_points.  num_vp <= 512.  ghost_xyz (num_vp x 3) and
 * num_ghost (may be NULL) receive the last iteration's ghosts. */
int mrsph_cvp_lset(mrsph_handle* h, long long n, const double* xyz, const double* mass, const double* mass_surface,
                   const mrsph_cvp_params* p, double* vp_xyz, int* labels, double* vp_mass, double* ghost_xyz,
                   int* num_ghost, mrsph_cvp_result* res);

/* 2D triangulation of the relaxed particles (row A14): the neighbour-graph
 * mesh of Voronoi_construction::Local_VD_generation
 * (src/geometry_tools/voronoi_construction.cpp:6-127: an edge i-j when j is a
 * Voronoi neighbour of i among i's neighbours; voro++ replaced by exact
 * orient2d / incircle signs), Graphmeshcls::Reconstruct_tris
 * (src/geometry_tools/graph_mesh.cpp:37-409: 3-cycles i > j > k; a triangle of
 * three non-REAL particles whose centroid phi <= 1e-4 x the vertex mean loses
 * its longest edge; the graph is rebuilt from the kept triangles; final
 * 3-cycles plus non-manifold / crossing checks) and Tri_quality_statistics
 * (graph_mesh.cpp:411-670).  Uses the neighbour lists of the last density
 * phase and the current positions. */
typedef struct {
  long long ntri;        /* final triangles */
  long long nedge;       /* edges after the rebuild */
  long long nedge_first; /* local-Voronoi edges before pass 1 */
  long long ndeleted;    /* edges removed by the centroid rule */
  long long nerror;      /* edges with > 2 triangles or crossing opposite vertices */
  double max_angle, min_angle, max_aspect, max_edge, min_edge, max_area, min_area;
  double G_min, G_avg;   /* shape factor 2 sqrt(3) A / (l_max s) */
  double min_angle_avg, theta_30; /* mean minimum angle; share of triangles with min angle < 30 deg */
  double total_area;
  long long hist[45];    /* all angles, 4-degree bins (the last bin takes 176..180) */
} mrsph_tri_quality;

/* tris (cap x 3 ints, vertex ids, rows ordered i > j > k, ascending (i, j, k))
 * may be NULL or too small: *ntri is always set and tris is filled only when
 * cap >= *ntri.  quality may be NULL.  2D handles only. */
int mrsph_triangulate(mrsph_handle* h, int* tris, long long cap, long long* ntri, mrsph_tri_quality* quality);

/* 3D tetrahedralisation and tet quality: replaces Graphmeshcls::Reconstruct_tets
 * (graph_mesh.cpp:981-1100, TetGen's Delaunay tetrahedralisation of all
 * particles followed by Check_whether_this_tet_should_be_delete, :675-979)
 * and Tet_quality_statistics (:1967-2400).  The tets are the Delaunay tets
 * of the particles (positions snapped to the grid `grid`, about one ulp of
 * the domain's largest coordinate) whose circumsphere lies inside the
 * neighbour ball (radius cutoff * h) of one of their four particles; tets
 * whose four particles are all not REAL and whose aspect ratio (longest
 * edge / smallest height) exceeds 10 are dropped, as in the reference.
 * Large tets across concavities of the body and on the convex hull, which
 * TetGen keeps, are not produced.  Uses the neighbour rows of the last
 * density phase (spilled rows: MRSPH_ERR_RANGE). */
typedef struct {
  long long ntet;
  long long nopen;     /* particles on the hull of their neighbour row (their star does not close) */
  long long ndeleted;  /* tets dropped by the aspect-ratio rule */
  long long ntie;      /* particles that met five co-spherical particles */
  double grid;         /* the snapping grid */
  double total_volume, min_volume, max_volume;
  double min_edge, max_edge;
  double min_aspect, max_aspect, avg_aspect;
  double min_radius_ratio, max_radius_ratio, avg_radius_ratio; /* 3 r_in / r_circ */
  double min_dihedral, max_dihedral, avg_min_dihedral;         /* degrees */
  long long nsmall_dihedral[4]; /* tets whose smallest dihedral is below 10, 20, 30, 40 degrees */
  long long aspect_hist[12];    /* bins up to 1.5, 2, 2.5, 3, 4, 6, 10, 15, 25, 50, 100, above */
  long long radius_hist[56];    /* radius ratio in bins of 0.02 (the last takes 1.1 and above) */
  long long dihedral_hist[45];  /* all six dihedral angles, 4-degree bins */
  long long ntrunc;             /* particles whose star outgrew 128 tets or 224 link edges: their walk
                                   stopped there, and tets they alone would have emitted are missing */
} mrsph_tet_quality;

/* tets (cap x 4 ints, ascending vertex ids per tet) may be NULL or too
 * small: *ntet is always set and tets is filled only when cap >= *ntet.
 * quality may be NULL.  3D handles only.  MRSPH_ERR_RANGE when a neighbour
 * row spilled.  A star is walked up to 128 tets and 224 link edges (about
 * 27 and 40 on average; ntrunc counts stars cut there).  The device work is
 * synchronous; scratch (about 400 bytes per particle plus the neighbour
 * rows) is allocated and freed by the call. */
int mrsph_tetrahedralize(mrsph_handle* h, int* tets, long long cap, long long* ntet, mrsph_tet_quality* quality);

/* Batched relaxation of independent geometries (no counterpart in the
 * reference, which relaxes one geometry per run, SPH_run_mesh_generation,
 * sph_mesh_generation.cpp:1371-1463, from Solver::SPH_Mesh_Generation_Solver,
 * solver.cpp:257-321).  A batch steps seeded handles of one device together;
 * each handle's results equal those of stepping it alone.  Modes:
 *   MRSPH_BATCH_PERSISTENT (default when every handle is FP32-split): one
 *     cooperative launch of a persistent kernel runs up to 32 whole steps of
 *     every geometry over (geometry, block) work lists with grid-wide
 *     barriers between the phases; a barrier that waits longer than one
 *     second gives up and the batch reports MRSPH_ERR_DEVICE.
 *   MRSPH_BATCH_PHASES: the same work lists, one launch per phase.
 *   MRSPH_BATCH_STREAMS (FP64-plain batches): each handle's own step graph on
 *     the handle's own stream.
 * Work queued on a handle before mrsph_batch_step runs first; work queued on
 * it afterwards runs after the batch's steps.  A handle may be stepped alone
 * between batch calls.  Handles and batches may be destroyed in any order:
 * destroying a handle that a batch holds waits for the batch's queued work
 * and takes the handle out of it, after which the batch's step and sync
 * calls return MRSPH_ERR_STATE (only mrsph_batch_destroy remains).
 * FP32-split results of a batch whose geometries use different smoothing
 * kernels equal those of stepping each alone as well. */
typedef struct mrsph_batch mrsph_batch;
#define MRSPH_BATCH_STREAMS 0
#define MRSPH_BATCH_PERSISTENT 1
#define MRSPH_BATCH_PHASES 2
int mrsph_batch_create(mrsph_handle* const* handles, int count, mrsph_batch** out);
int mrsph_batch_destroy(mrsph_batch* b);
int mrsph_batch_last_error(mrsph_batch* b, char* buf, size_t len);
/* MRSPH_BATCH_PERSISTENT and MRSPH_BATCH_PHASES need FP32-split handles. */
int mrsph_batch_set_mode(mrsph_batch* b, int mode);
/* the mode; graph_captured (may be NULL): 1 when the persistent launches are
 * replayed from CUDA graphs. */
int mrsph_batch_get_mode(mrsph_batch* b, int* mode, int* graph_captured);
/* nsteps steps of every handle (asynchronous; capacity checks every 32 steps). */
int mrsph_batch_step(mrsph_batch* b, int nsteps);
/* Same, device-timed with CUDA events (ms from before the first handle's first
 * step to after every handle's last step). */
int mrsph_batch_step_timed(mrsph_batch* b, int nsteps, double* ms);
int mrsph_batch_sync(mrsph_batch* b);
/* Self-test of the persistent kernel's bounded barrier wait (no counterpart in
 * the reference): a two-block cooperative launch in which one block never
 * arrives; the other must give up after limit_ms (0 < limit_ms <= 10000) and
 * raise the error bit.  *raised = 1 when it did. */
int mrsph_batch_barrier_selftest(int device, double limit_ms, int* raised);

/* e2e helpers: positions in id order (n x 3), host memory (pinned or not). */
int mrsph_upload_positions(mrsph_handle* h, const double* xyz);
int mrsph_download_positions(mrsph_handle* h, double* xyz);

#ifdef __cplusplus
}
#endif
#endif /* MRSPH_RELAX_H */
