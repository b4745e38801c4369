/*
 * hg_gpu.h - C ABI of the GB300-native granular time-step library
 * (libhg_gpu.so).
 *
 * This is the drop-in boundary for the per-timestep core of libHybridGrains:
 * the explicit MPM step of mpmgrains2d, the penalty-DEM disk step of
 * rigidbody2d and the node-node coupling of hybridgrains2dnew. Each entry
 * point names the reference interface it replaces. The reference interfaces
 * are C++ member functions operating on caller-owned Eigen arrays; here state
 * lives on the device between calls and the host exchanges plain arrays in the
 * reference's memory layouts:
 *   - MPM positions/velocities: 2 x N column-major doubles (x0 y0 x1 y1 ...),
 *     like Matrix2Xsc::data();
 *   - be_bar: N column-major 2x2 blocks (b00 b10 b01 b11), like
 *     std::vector<Matrix22sc>;
 *   - DEM q and v: 3 x N doubles (x y theta / vx vy omega), like
 *     RigidBody2DState::q() / v().
 * The library copies; the caller keeps ownership of every host buffer.
 *
 * Conventions: every call returns an hg_status; no C++ exception crosses the
 * ABI; hg_last_error() gives a message for the calling thread's last failure.
 * Calls on one context are asynchronous on that context's CUDA stream until a
 * download, hg_*_status or hg_context_synchronize. One host thread per
 * context. Kernels never trap: device-side faults in the data (NaN, particles
 * leaving the grid, capacity overflow) set bits of a per-object status word.
 */
#ifndef HG_GPU_H
#define HG_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t hg_status;

enum {
  HG_OK = 0,
  HG_ERR_INVALID_ARGUMENT = 1,
  HG_ERR_CUDA = 2,
  HG_ERR_OUT_OF_MEMORY = 3,
  HG_ERR_CAPACITY = 4,
  HG_ERR_UNSUPPORTED = 5,
  HG_ERR_DEVICE_STATUS = 6
};

/* Bits of the device status word (hg_mpm_status / hg_dem_status). */
enum {
  HG_STATUS_NONFINITE = 1u << 0,        /* NaN/Inf produced in particle state */
  HG_STATUS_OUT_OF_GRID = 1u << 1,      /* a particle left the MPM grid */
  HG_STATUS_CONTACT_OVERFLOW = 1u << 2, /* DEM contact capacity exceeded */
  HG_STATUS_CELL_OVERFLOW = 1u << 3,    /* DEM broadphase bucket overflow */
  HG_STATUS_NEGATIVE_MASS = 1u << 4,    /* a grain coupled to an empty node */
  HG_STATUS_INDEX = 1u << 5             /* bounds-checking build: an index out of
                                           its array (the access was skipped) */
};

typedef struct hg_context hg_context;
typedef struct hg_mpm hg_mpm;
typedef struct hg_dem hg_dem;
typedef struct hg_hybrid hg_hybrid;

/* ---- context -------------------------------------------------------------- */

hg_status hg_context_create(int32_t device, hg_context **out);
hg_status hg_context_destroy(hg_context *ctx);
hg_status hg_context_synchronize(hg_context *ctx);
const char *hg_status_string(hg_status s);
const char *hg_last_error(void);
/* Number of kernels this library has launched in the process so far. */
int64_t hg_kernel_launch_count(void);
/* Host threads the library's host-side loops (zone update, resampling) may
 * use, process-wide: n >= 1, or 0 for the default (the hardware concurrency,
 * at most 16). Results do not depend on it. */
hg_status hg_set_host_threads(int32_t n);
/* Measurement hooks (no counterpart in the reference): CUDA events recorded
 * on the context's stream; _end synchronises and returns the elapsed time. */
hg_status hg_context_timer_begin(hg_context *ctx);
hg_status hg_context_timer_end(hg_context *ctx, double *ms);

/* Fences and page-locked memory, for callers that keep work queued while
 * they handle results (no counterpart in the reference, which steps
 * synchronously). A fence marks the point of the context's stream reached by
 * the calls made so far; it is done once the device has finished them.
 * Fence ids increase by one per call; only the latest 256 fences are
 * tracked exactly, and an older one may report "not done" until a later one
 * is done. */
hg_status hg_context_fence(hg_context *ctx, int64_t *fence);
hg_status hg_context_fence_done(hg_context *ctx, int64_t fence, int32_t *done);
hg_status hg_context_fence_wait(hg_context *ctx, int64_t fence);
/* Device bytes held by this process's objects (all contexts on the device). */
hg_status hg_context_device_bytes(hg_context *ctx, int64_t *bytes);
/* Page-locked host memory: asynchronous copies from and to it overlap with
 * queued work. */
hg_status hg_host_alloc(int64_t bytes, void **out);
hg_status hg_host_free(void *p);

/* ---- MPM (mpmgrains2d) ------------------------------------------------------ */

enum { HG_BASIS_LINEAR = 0, HG_BASIS_UGIMP = 1 };
enum { HG_PRECISION_FP64 = 0, HG_PRECISION_MIXED = 1 };
enum { HG_MAX_PLANES = 8 };

/* MPMStaticPlane (mpmgrains2d/StaticPlane.h:6-22). The normal is normalised
 * on creation, like the reference constructor (StaticPlane.cpp:6-12). */
typedef struct {
  double x[2];
  double n[2];
  int32_t sticking; /* 0 = SLIDING, 1 = STICKING */
  int32_t pad_;
  double lower_bound; /* -inf when absent */
} hg_mpm_plane;

/* Inputs of InitialSimulationState::generateSimulationState
 * (mpmgrains2d/InitialSimulationState.cpp:147-228) minus the particles. */
typedef struct {
  double grid_min[2];
  double grid_max[2];
  double cell_width;
  int32_t basis;     /* HG_BASIS_* (shape_function_category / order) */
  int32_t precision; /* HG_PRECISION_* */
  double shear_modulus;
  double bulk_modulus;
  double dp_alpha;   /* Drucker_Prager_alpha (<material alpha=...>) */
  double flip_alpha; /* PIC/FLIP blend (<integrator alpha=...>) */
  double gravity[2];
  int32_t num_planes;
  int32_t pad_;
  hg_mpm_plane planes[HG_MAX_PLANES];
  int64_t capacity; /* maximum number of material points */
} hg_mpm_desc;

/* Replaces SimulationState construction (PhysicsGrid::setDimensions,
 * mpmgrains2d/PhysicsGrid.cpp:14-55). */
hg_status hg_mpm_create(hg_context *ctx, const hg_mpm_desc *desc, hg_mpm **out);
hg_status hg_mpm_destroy(hg_mpm *m);
/* PhysicsGrid::min / max / cell_count after setDimensions. */
hg_status hg_mpm_grid_info(hg_mpm *m, double grid_min[2], double grid_max[2],
                           int32_t cell_count[2]);

/* InitialSimulationState rasterizeRectangle
 * (mpmgrains2d/InitialSimulationState.cpp:48-145) on the host: writes at most
 * cap points (q, v as 2 x N) and returns the generated count in *count. Pass
 * cap = 0 and NULL buffers to query the count. */
hg_status hg_mpm_seed_rectangle(hg_mpm *m, const double rmin[2],
                                const double rmax[2], double density,
                                int32_t samples_per_dim, const double vel[2],
                                double omega, int64_t cap, double *q, double *v,
                                double *mass, double *volume, double *hl,
                                int64_t *count);

/* hg_mpm_seed_rectangle followed by hg_mpm_upload_async of its points
 * (be_bar = I, J = 1), with the points generated on the device: bit-identical
 * to the host version and queued without host data or waiting. *count gets
 * the number of points; more than the capacity is HG_ERR_CAPACITY and
 * changes nothing. For scenes described by their geometry (many small
 * scenes admitted while others step); no counterpart in the reference. */
hg_status hg_mpm_seed_rectangle_device(hg_mpm *m, const double rmin[2],
                                       const double rmax[2], double density,
                                       int32_t samples_per_dim, const double vel[2],
                                       double omega, int64_t *count);

/* MaterialPoints::setPoints (mpmgrains2d/MaterialPoints.cpp). Optional
 * arrays may be NULL: be_bar = I, J = 1, just_homogenized = 0,
 * kinematic = 0. */
hg_status hg_mpm_upload(hg_mpm *m, int64_t n, const double *q, const double *v,
                        const double *mass, const double *volume,
                        const double *hl, const double *be_bar,
                        const double *J, const int32_t *just_homogenized,
                        const uint8_t *kinematic);
/* hg_mpm_upload without waiting: the copies are queued on the context's
 * stream, and the caller keeps the arrays unchanged until a fence taken
 * after this call is done. From page-locked memory (hg_host_alloc) the host
 * does not wait for queued steps. No counterpart in the reference. */
hg_status hg_mpm_upload_async(hg_mpm *m, int64_t n, const double *q, const double *v,
                              const double *mass, const double *volume,
                              const double *hl, const double *be_bar,
                              const double *J, const int32_t *just_homogenized,
                              const uint8_t *kinematic);
/* Positions and velocities (2 x N each, upload order; either may be NULL)
 * copied to host memory behind the steps queued so far, without waiting: the
 * arrays hold the frame once a fence taken after this call is done. Use
 * page-locked memory for the copy to overlap. A frame of the reference's
 * output loop (mpmgrains2d_cli.cpp) taken without stopping the device. */
hg_status hg_mpm_frame_async(hg_mpm *m, double *q, double *v);
/* Device bytes hg_mpm_create plus an upload and a download of capacity
 * points allocate for this description (admission control for many
 * resident scenes; no counterpart in the reference). */
hg_status hg_mpm_estimate_bytes(const hg_mpm_desc *desc, int64_t *bytes);
/* Material point state in upload order; any pointer may be NULL. */
hg_status hg_mpm_download(hg_mpm *m, double *q, double *v, double *be_bar,
                          double *J, int32_t *just_homogenized);
hg_status hg_mpm_num_particles(hg_mpm *m, int64_t *n);

/* ExplicitIntegrator::flow (mpmgrains2d/ExplicitIntegrator.cpp:63-67),
 * nsteps times. */
hg_status hg_mpm_step(hg_mpm *m, double dt, int32_t nsteps);
/* ExplicitIntegrator::flow_zero_phase / flow_first_phase /
 * flow_second_phase (ExplicitIntegrator.cpp:5-61); FP64 precision only.
 * The internal-force scatter is done in phase 0, which is equivalent because
 * the material points do not change between phase 0 and phase 1. */
hg_status hg_mpm_phase0(hg_mpm *m);
hg_status hg_mpm_phase1(hg_mpm *m, double dt);
hg_status hg_mpm_phase2(hg_mpm *m, double dt);

/* PhysicsGrid fields ((cell_count+1) node-major, 2 x nodes for vectors).
 * MIXED precision keeps mass, velocity and acceleration of the last grid
 * update only; requesting momentum, momentum_new or force from a MIXED
 * object returns HG_ERR_UNSUPPORTED. */
hg_status hg_mpm_download_grid(hg_mpm *m, double *mass, double *momentum,
                               double *momentum_new, double *force,
                               double *velocity, double *acceleration);
/* Cell of each material point, floor((x - grid_min) / cell_width) per axis
 * (2 ints per point, upload order): the first stencil index of the linear
 * basis (LinearBasisFunctions.cpp:49-62) and the key the MIXED path sorts
 * by. */
hg_status hg_mpm_cell_index(hg_mpm *m, int32_t *cells);
/* Synchronises and returns the device status word (HG_STATUS_* bits). */
hg_status hg_mpm_status(hg_mpm *m, uint32_t *word);
hg_status hg_mpm_clear_status(hg_mpm *m);
/* Number of particle re-sorts performed so far (MIXED precision). */
hg_status hg_mpm_rebin_count(hg_mpm *m, int64_t *count);
/* Measurement hooks (no counterpart in the reference), MIXED precision:
 * while enabled, every step records CUDA events around its grid-update and
 * fused G2P/P2G kernels; _read synchronises and returns the summed kernel
 * times since enabling and the number of steps recorded. */
hg_status hg_mpm_profile(hg_mpm *m, int32_t enable);
hg_status hg_mpm_profile_read(hg_mpm *m, double *g2p2g_ms,
                              double *grid_update_ms, int64_t *steps);

/* ---- batches of independent MIXED MPM scenes -------------------------------
 * No counterpart in the reference (it steps one scene per process). A batch
 * steps every member scene with one grid-update launch and one fused G2P/P2G
 * launch whose CTAs drain (scene, tile) work items, so many small scenes share
 * the GPU the way one large scene does. Members are MIXED MPM objects of the
 * batch's context; each keeps its own state, dt and parameters, and stepping
 * a member alone or in a batch gives the same result up to the order of FP32
 * atomic additions. Members may join and leave between steps; remove a
 * member before destroying it, and destroy a batch before its context. */
typedef struct hg_batch hg_batch;
enum { HG_MAX_BATCH = 1024 };
hg_status hg_batch_create(hg_context *ctx, int32_t max_members, hg_batch **out);
hg_status hg_batch_destroy(hg_batch *b);
hg_status hg_batch_add(hg_batch *b, hg_mpm *m, double dt);
hg_status hg_batch_remove(hg_batch *b, hg_mpm *m);
hg_status hg_batch_size(hg_batch *b, int32_t *n);
/* nsteps steps of every member (ExplicitIntegrator::flow per member). */
hg_status hg_batch_step(hg_batch *b, int32_t nsteps);
/* Counters since creation: member-steps queued, member re-sorts, batch
 * steps, host milliseconds spent inside hg_batch_step and, of those, the
 * milliseconds it waited for the device (argument tables in use). */
hg_status hg_batch_stats(hg_batch *b, int64_t *member_steps, int64_t *resorts,
                         int64_t *steps, double *host_ms, double *wait_ms);
/* Measurement hooks: CUDA events around each phase of every batch step
 * while enabled (enabling clears earlier records); _read synchronises and
 * returns the summed milliseconds of re-sorts, argument-table copies, grid
 * updates and fused launches, and the number of steps recorded. */
hg_status hg_batch_profile(hg_batch *b, int32_t enable);
hg_status hg_batch_profile_read(hg_batch *b, double *resort_ms, double *table_ms,
                                double *update_ms, double *fused_ms, int64_t *steps);

/* ---- launch-shape autotuning (no reference counterpart) -------------------
 * The MIXED kernels run as grids of CTAs that walk the active tiles (single
 * scene) or contiguous shares of the (scene, tile) items (batch). A launch
 * shape gives the CTAs per SM of the fused G2P/P2G kernel and of the grid
 * update; 0 keeps the built-in choice (3 and 8). The autotuner times
 * HG_TUNE_CANDIDATES shapes on the live object with CUDA events, each for
 * steps_per_candidate steps (the scene advances by all of them: a shape only
 * changes the order of FP32 atomic sums). A batch keeps the fastest shape for
 * each kernel. A single scene then times the whole step, replayed as graphs
 * in which the two kernels overlap, for every pair of a fused and an update
 * shape (48 more steps each) and keeps the fastest pair. The result is
 * recorded in a process-wide table under the object's size
 * class: the device's SM count, the tile count (single scenes) and the point
 * count, both rounded up to powers of two. MIXED objects and batches look up
 * their class before their first step. The table can be saved to and merged
 * from a text file. hg_mpm_autotune also records the object's step graphs
 * for dt with the chosen shape (for both particle buffers), so that the
 * steps after it replay them without capturing one on first use. */
enum { HG_TUNE_CANDIDATES = 4 };
typedef struct hg_launch_shape {
  int32_t fused_ctas_per_sm;
  int32_t update_ctas_per_sm;
} hg_launch_shape;
typedef struct hg_tune_report {
  int32_t candidates;
  hg_launch_shape tried[HG_TUNE_CANDIDATES];
  double fused_ms[HG_TUNE_CANDIDATES];  /* mean per step, per kernel */
  double update_ms[HG_TUNE_CANDIDATES]; /* mean per step, per kernel */
  hg_launch_shape chosen;
  /* single scenes: the whole step (graph replays, kernels overlapping as in
   * production) with fused shape i and update shape j, mean per step; the
   * chosen shape is the fastest pair. Batches: 0 (chosen per kernel). */
  double step_ms[HG_TUNE_CANDIDATES][HG_TUNE_CANDIDATES];
  int64_t steps; /* steps the object or every member advanced while tuning */
} hg_tune_report;
hg_status hg_mpm_autotune(hg_mpm *m, double dt, int32_t steps_per_candidate,
                          hg_tune_report *report);
hg_status hg_mpm_launch_shape(hg_mpm *m, hg_launch_shape *shape);
hg_status hg_mpm_set_launch_shape(hg_mpm *m, const hg_launch_shape *shape);
hg_status hg_batch_autotune(hg_batch *b, int32_t steps_per_candidate, hg_tune_report *report);
hg_status hg_batch_launch_shape(hg_batch *b, hg_launch_shape *shape);
/* ---- checkpoint / resume (no reference counterpart: the reference's
 * mpmgrains2d snapshot, mpmgrains2d_cli.cpp:154-247, holds host arrays, and
 * its hybrid and penalty-map serialization exit) --------------------------
 * An object's device state as one host blob in this library's own versioned
 * format ("HGSTATE" header, then tagged segments): for MIXED MPM the sorted
 * particle records, the next step's P2G accumulators and the sort tables; for
 * FP64 MPM the particle and grid arrays; for DEM the bodies and the live
 * contact history (keys and records); for a hybrid coupling the homogenised
 * stress and velocity accumulated in the current interval. A blob loads into
 * an object created with the same grid (MPM) and a capacity that holds it;
 * the loaded object continues as the saved one would. *_state_bytes gives the
 * size a save needs. */
hg_status hg_mpm_state_bytes(hg_mpm *m, int64_t *bytes);
hg_status hg_mpm_state_save(hg_mpm *m, void *dst, int64_t bytes);
hg_status hg_mpm_state_load(hg_mpm *m, const void *src, int64_t bytes);
hg_status hg_dem_state_bytes(hg_dem *d, int64_t *bytes);
hg_status hg_dem_state_save(hg_dem *d, void *dst, int64_t bytes);
hg_status hg_dem_state_load(hg_dem *d, const void *src, int64_t bytes);
hg_status hg_hybrid_state_bytes(hg_hybrid *h, int64_t *bytes);
hg_status hg_hybrid_state_save(hg_hybrid *h, void *dst, int64_t bytes);
hg_status hg_hybrid_state_load(hg_hybrid *h, const void *src, int64_t bytes);

/* One line per entry: "kind sms tiles points fused update" (kind 0: single
 * scene, 1: batch). */
hg_status hg_tune_save(const char *path);
hg_status hg_tune_load(const char *path);
hg_status hg_tune_clear(void);

/* ---- zone labels (hybridgrains2dnew ZoneTools), host code ----------------
 * Runs on the host at the resampling interval on positions copied from the
 * device (HybridGrains2DSim::updateHybridStates_poorman,
 * HybridGrains2DSim.cpp:301-326). Labels are bit-exact restatements of the
 * reference's FP64 arithmetic. */
enum { HG_ZONE_CONTINUUM = 0, HG_ZONE_DISCRETE = 1, HG_ZONE_HYBRID = 2 };
enum {
  HG_ZONES_RECONCILIATION = 0,    /* getRZones / getRZoneIndices */
  HG_ZONES_DIRECT_TRANSITION = 1, /* getDirectTransitionZonesFromDiscreteToContinuum */
  HG_ZONES_INNER_CONTINUUM = 2,   /* identifyInnerContinuumRegion */
  HG_ZONES_INNER_CONTINUUM_EXCLUDING_DIRECT = 3,
  HG_ZONES_LEVEL_SET_HYBRID = 4   /* hybrid cells of the level-set grid */
};
enum { HG_ZONES_MPM = 0, HG_ZONES_DEM = 1 };
typedef struct hg_zones hg_zones;
typedef struct {
  double mpm_grid_min[2];   /* PhysicsGrid::min after setDimensions */
  double mpm_cell_width;
  int32_t mpm_cells[2];     /* PhysicsGrid::cell_count */
  double level_set_cell_width;
  int32_t allow_direct_transitions;
  int32_t phi_samples_per_cell_side;
  double phi_window_size;
  double phi_threshold;
  double rzone_level_set;
  double rzone_half_thickness;
} hg_zones_desc;
/* ZoneTools::init (ZoneTools.cpp:6-64); a level-set cell wider than an MPM
 * cell is HG_ERR_INVALID_ARGUMENT (the reference exits). */
hg_status hg_zones_create(const hg_zones_desc *desc, hg_zones **out);
hg_status hg_zones_destroy(hg_zones *z);
/* updatePackingFraction + updateDistanceField + computeRZones
 * (ZoneTools.cpp:186-672). q: 3 x n_disks (x, y, theta), radius, fixed
 * (NULL: none fixed; fixed disks are ignored as in
 * getAllNonFixedCircleBodies); points: 2 x n_points MPM positions. */
hg_status hg_zones_update(hg_zones *z, int64_t n_disks, const double *q,
                          const double *radius, const uint8_t *fixed,
                          int64_t n_points, const double *points);
hg_status hg_zones_grid_info(hg_zones *z, int32_t level_set_cells[2],
                             int32_t mpm_cells[2]);
/* Packing fraction per level-set cell, signed distance per level-set grid
 * point ((nx+1) x (ny+1)), level-set cell labels, MPM cell labels; any
 * pointer may be NULL. */
hg_status hg_zones_fields(hg_zones *z, double *packing_fraction, double *distance,
                          int32_t *level_set_labels, int32_t *mpm_labels);
/* Replaces the MPM cell labels (the previous labels of the next update). */
hg_status hg_zones_set_labels(hg_zones *z, const int32_t *mpm_labels);
/* A zone list (HG_ZONES_*): boxes (x0, y0, x1, y1) and cell indices (i, j),
 * at most cap of each; *count gets the list's length. */
hg_status hg_zones_list(hg_zones *z, int32_t which, int64_t cap, double *boxes,
                        int32_t *cells, int64_t *count);
/* determineMPMParticlesToDelete (kind HG_ZONES_MPM) /
 * determineDEMGrainsToDelete (HG_ZONES_DEM) (ZoneTools.cpp:674-731): ids in
 * increasing order; x holds positions with the given stride in doubles (2
 * for MPM q, 3 for DEM q). */
hg_status hg_zones_to_delete(hg_zones *z, int32_t kind, int64_t n, const double *x,
                             int32_t stride, const uint8_t *fixed, int64_t cap,
                             int32_t *ids, int64_t *count);
/* demWeight / mpmWeight (ZoneTools.cpp:123-147) for n positions. */
hg_status hg_zones_weights(hg_zones *z, int32_t kind, int64_t n, const double *x,
                           int32_t stride, double *w);
/* Number of edge samples of the last distance field. */
hg_status hg_zones_boundary_samples(hg_zones *z, int64_t *count);
/* Area of the intersection of a disk with an axis-aligned box
 * (circleRectangleIntersectionArea, CircleRectangleIntersection.cpp:70-82). */
double hg_zones_disk_box_area(double x0, double x1, double y0, double y1,
                              double cx, double cy, double r);

/* ---- resampling (hybridgrains2dnew ResamplingTools), host code -----------
 * The resampling step of HybridGrains2DSim::updateHybridStates_poorman
 * (HybridGrains2DSim.cpp:327-536) after the zone labels are updated: grain
 * and point insertion in the reconciliation (and direct-transition) zones
 * and the inner continuum zones (CAvoidAVoid, AvoidAvoid.cpp:103-183), the
 * inserted bodies' quantities, deletion by zone, and mass weights. Runs on the
 * host on state copied from the device; bit-exact restatement of the
 * reference's FP64 arithmetic and random streams (MT19937 of random.c,
 * std::default_random_engine + std::normal_distribution for radii). */
typedef struct hg_resampler hg_resampler;
typedef struct {
  hg_zones_desc zones;              /* the MPM grid and zone settings */
  double mpm_grid_max[2];           /* PhysicsGrid::max after setDimensions */
  int32_t basis;                    /* HG_BASIS_* of the MPM scene */
  int32_t newly_inserted_continuum_stress_free;
  double initial_particle_size;     /* cell width / samples per dimension */
  double material_density;
  double dem_r_mean, dem_r_std;     /* demRMean, demRStd (mean < 0: unset) */
  double rho_dem;
  double kappa, mu;                 /* bulk and shear modulus */
  int32_t homogenize_stress, homogenize_velocity;
} hg_resampler_desc;
/* Counts of the last hg_resampler_run and its host time by phase (ms):
 * grain insertion, point insertion (transition, direct and inner regions),
 * the point search grids, the quantities of the inserted points and grains,
 * and deletion with the weight update. */
typedef struct {
  int64_t points_inserted, grains_inserted, points_deleted, grains_deleted;
  double ms_insert_grains, ms_insert_points, ms_point_grids, ms_quantities, ms_delete;
} hg_resampler_stats;
hg_status hg_resampler_create(const hg_resampler_desc *desc, hg_resampler **out);
hg_status hg_resampler_destroy(hg_resampler *r);
/* MaterialPoints arrays: q0, q, v 2 x n; m, volume, m0, volume0, hl, J n;
 * be_bar 4 per point (column-major); just_homogenized, kinematic may be
 * NULL (0). */
hg_status hg_resampler_set_points(hg_resampler *r, int64_t n, const double *q0,
                                  const double *q, const double *v, const double *m,
                                  const double *volume, const double *m0,
                                  const double *volume0, const double *hl,
                                  const double *be_bar, const double *J,
                                  const int32_t *just_homogenized,
                                  const uint8_t *kinematic);
/* RigidBody2DState: q0, q, v 3 x n; radius n; M0 3 x n (m, m, I); fixed
 * may be NULL. */
hg_status hg_resampler_set_grains(hg_resampler *r, int64_t n, const double *q0,
                                  const double *q, const double *v, const double *radius,
                                  const double *M0, const uint8_t *fixed);
/* Finalised homogenised stress (4 per node, column-major) and velocity (2
 * per node) of the MPM grid; NULL: zero. */
hg_status hg_resampler_set_homogenized(hg_resampler *r, const double *stress,
                                       const double *velocity);
/* The resampling step with the labels of z (updated by hg_zones_update). */
hg_status hg_resampler_run(hg_resampler *r, hg_zones *z);
hg_status hg_resampler_counts(hg_resampler *r, int64_t *points, int64_t *grains,
                              hg_resampler_stats *stats);
/* The state after the step, in the layouts of the setters; w: mass weights.
 * old_to_new maps the grains after insertion (before deletion) to their new
 * index or -1 (hg_resampler_dem_map_size entries), for the contact history. */
hg_status hg_resampler_get_points(hg_resampler *r, double *q0, double *q, double *v,
                                  double *m, double *volume, double *m0,
                                  double *volume0, double *w, double *hl,
                                  double *be_bar, double *J, int32_t *just_homogenized,
                                  uint8_t *kinematic);
hg_status hg_resampler_get_grains(hg_resampler *r, double *q0, double *q, double *v,
                                  double *radius, double *M0, double *w, uint8_t *fixed,
                                  int32_t *old_to_new);
hg_status hg_resampler_dem_map_size(hg_resampler *r, int64_t *n);
/* The resampler's random streams, advanced by one draw (for tests). */
uint32_t hg_resampler_random_u32(hg_resampler *r);
float hg_resampler_random_f32(hg_resampler *r);
double hg_resampler_random_radius(hg_resampler *r);
/* The random streams' state (the insertion MT19937, the radius engine and
 * its normal distribution, the next test id) as a host blob, for checkpoint
 * and resume of a hybrid simulation. */
hg_status hg_resampler_rng_bytes(hg_resampler *r, int64_t *bytes);
hg_status hg_resampler_rng_save(hg_resampler *r, void *dst, int64_t bytes);
hg_status hg_resampler_rng_load(hg_resampler *r, const void *src, int64_t bytes);

/* ---- DEM (rigidbody2d, penalty map) --------------------------------------- */

/* RigidBody2DStaticPlane, static (v = 0, omega = 0). */
typedef struct {
  double x[2];
  double n[2];
} hg_dem_plane;

/* RigidBody2DStaticDrum (rigidbody2d/RigidBody2DStaticDrum.h:6-33): a fixed
 * circular wall of radius r centred at x that holds the disks inside it
 * (StaticDrumCircleConstraint.cpp:7-13: a disk touches it once its centre is
 * r - r_disk or more from x). Scene files give only x and r; the drum does
 * not move. */
typedef struct {
  double x[2];
  double r;
} hg_dem_drum;
enum { HG_MAX_DRUMS = 8 };

/* PenaltyImpactFrictionMap parameters (rigidbody2d/PenaltyImpactFrictionMap.
 * cpp:15-26) plus NearEarthGravityForce, the static planes and drums and the
 * body/contact capacities. */
typedef struct {
  double gravity[2];
  double kn, kt, gamman, gammat, mu;
  double cell_scale; /* SpatialGrid cell scale (reporting only) */
  int32_t num_planes;
  int32_t pad_;
  hg_dem_plane planes[HG_MAX_PLANES];
  int64_t capacity;         /* bodies */
  int64_t contact_capacity; /* active contacts */
  /* HG_PRECISION_FP64: the reference's FP64 arithmetic, bit for bit.
   * HG_PRECISION_MIXED: contact law and integration in FP32; positions, the
   * pairwise position difference, contact points and the position update in
   * FP64 (velocities and records keep FP64 storage holding FP32 values). */
  int32_t precision;
  int32_t num_drums;
  hg_dem_drum drums[HG_MAX_DRUMS];
} hg_dem_desc;

hg_status hg_dem_create(hg_context *ctx, const hg_dem_desc *desc, hg_dem **out);
hg_status hg_dem_destroy(hg_dem *d);
/* RigidBody2DState::addBody for circles (rigidbody2d/RigidBody2DState.cpp:
 * 237-336): q, v as 3 x N; mass = rho pi r^2, inertia = m r^2 / 2. Resets the
 * contact history. */
hg_status hg_dem_upload(hg_dem *d, int64_t n, const double *q, const double *v,
                        const double *radius, const double *mass,
                        const double *inertia, const uint8_t *fixed);
/* hg_dem_upload after bodies were added and removed (the resampling step):
 * the contact history is kept, with the contacts of removed bodies dropped
 * and the others renumbered by old_to_new (n_old entries, -1: removed;
 * PenaltyImpactFrictionMap::deleteCacheEntries, PenaltyImpactFrictionMap.cpp:
 * 1199-1278). Added bodies start without contacts. */
hg_status hg_dem_upload_relabel(hg_dem *d, int64_t n, const double *q, const double *v,
                                const double *radius, const double *mass,
                                const double *inertia, const uint8_t *fixed,
                                int64_t n_old, const int32_t *old_to_new);
/* Removes and adds bodies on the device, without a round trip to the host:
 * body i of the current n_old moves to old_to_new[i] (-1: removed; kept
 * bodies keep their order and fill 0 .. kept-1), then n_add bodies from the
 * arrays (q, v 3 x n_add) are appended with weight 1; the contact history is
 * renumbered. Queued without waiting: the arrays stay valid and unchanged
 * until a fence taken after this call is done (page-locked for the copies to
 * overlap). For many independent scenes in one object; no counterpart in the
 * reference. */
hg_status hg_dem_edit_async(hg_dem *d, int64_t n_old, const int32_t *old_to_new,
                            int64_t n_add, const double *q, const double *v,
                            const double *radius, const double *mass,
                            const double *inertia, const uint8_t *fixed);
/* q, v (3 x N each; either may be NULL) copied to host memory behind the
 * queued steps, without waiting (valid once a later fence is done). */
hg_status hg_dem_frame_async(hg_dem *d, double *q, double *v);
hg_status hg_dem_num_bodies(hg_dem *d, int64_t *n);
/* Concurrent mode (no reference counterpart): on != 0 gives the DEM object a
 * stream of its own, so its steps overlap the work queued on the context's
 * stream; hg_dem_wait_context orders the DEM's later work after everything
 * the context's stream has queued, hg_dem_join orders the context's later
 * work (frames, fences) after everything the DEM has queued. Synchronous DEM
 * calls synchronise the DEM's stream. A DEM in a hybrid step stays on the
 * context's stream. */
hg_status hg_dem_set_concurrent(hg_dem *d, int32_t on);
hg_status hg_dem_wait_context(hg_dem *d);
hg_status hg_dem_join(hg_dem *d);
/* RigidBody2DState::updateCurrentMassUsingMassWeights
 * (RigidBody2DState.cpp:1182-1200). */
hg_status hg_dem_set_weights(hg_dem *d, const double *w);
hg_status hg_dem_set_state(hg_dem *d, const double *q, const double *v);
hg_status hg_dem_download(hg_dem *d, double *q, double *v);
/* PenaltyImpactFrictionMap::flow / flowWithWeights
 * (PenaltyImpactFrictionMap.cpp:1083-1149) through RigidBody2DSim::flow /
 * flowWithWeight (RigidBody2DSim.cpp:1013-1069), nsteps times. */
hg_status hg_dem_step(hg_dem *d, double dt, int32_t nsteps, int32_t weighted);
hg_status hg_dem_num_contacts(hg_dem *d, int64_t *n);
/* The collision cache (PenaltyImpactFrictionMap::getCollisionCache), one
 * record of HG_DEM_RECORD_WIDTH doubles per contact, ordered: contacts with
 * static objects (body-major; each body's plane contacts, then its drum
 * contacts), circle-circle (body-major), kinematic circle-circle
 * (body-major). Fields: kind (HG_DEM_KIND_*), first, second (the plane or
 * drum index for static objects), depth, n[2], delta_s[2], vrel[2], r0[2],
 * r1[2], weight, contact_point[2], normal_force[2], friction_force[2], 0. */
enum {
  HG_DEM_KIND_PLANE = 0,
  HG_DEM_KIND_CIRCLE = 1,
  HG_DEM_KIND_KINEMATIC = 2,
  HG_DEM_KIND_DRUM = 3
};
enum { HG_DEM_RECORD_WIDTH = 22 };
hg_status hg_dem_download_contacts(hg_dem *d, int64_t cap, double *records,
                                   int64_t *count);
hg_status hg_dem_status(hg_dem *d, uint32_t *word);
/* SpatialGrid::getPotentialOverlaps (rigidbody2d/SpatialGrid.cpp:90-118) on
 * explicit AABBs (2 x N min and max): the sorted set of (i, j), i < j, whose
 * boxes overlap. Writes at most cap pairs; *count is the full count. */
hg_status hg_dem_candidate_pairs(hg_context *ctx, int64_t n,
                                 const double *aabb_min, const double *aabb_max,
                                 int64_t cap, int32_t *pairs, int64_t *count);

/* Allocation-free variant of hg_dem_candidate_pairs. No counterpart in the
 * reference. For callers that cannot allocate device memory on the calling
 * path: cudaMalloc synchronises the device and may be forbidden by a
 * host application that sets a fixed device-memory budget at start-up, and
 * some callers run the broadphase from a loop whose timing must not include
 * allocation. All device temporaries live in one fixed array inside the
 * library (about 3.4 MB, held by every GPU that loads the library until the
 * process exits), so the call takes at most HG_STATIC_PAIRS_MAX_BOXES boxes
 * and returns at most HG_STATIC_PAIRS_MAX_PAIRS pairs; larger inputs are
 * rejected with HG_ERR_CAPACITY. It allocates nothing: no cudaMalloc, no
 * cudaFree. The first call on each device looks up the array's device
 * address; make that first call before any stream capture. The address is
 * kept until the process exits: a cudaDeviceReset ends every context of this
 * library on that device, and this entry point may not be called after one.
 * Calls share the array: calls that overlap on the GPU (from several threads
 * or contexts on one device) race, so serialise them. Same inputs, outputs
 * and results as hg_dem_candidate_pairs. */
enum { HG_STATIC_PAIRS_MAX_BOXES = 16384, HG_STATIC_PAIRS_MAX_PAIRS = 262144 };
hg_status hg_dem_candidate_pairs_static(hg_context *ctx, int64_t n,
                                        const double *aabb_min,
                                        const double *aabb_max, int64_t cap,
                                        int32_t *pairs, int64_t *count);

/* ---- hybrid node-node coupling (hybridgrains2dnew) ------------------------ */

enum {
  HG_HYBRID_HOMOGENIZE_STRESS = 1,
  HG_HYBRID_HOMOGENIZE_VELOCITY = 2
};

/* HybridGrains2DSim over an MPM object and a DEM object on the same context
 * (hybridgrains2dnew/HybridGrains2DSim.cpp:21-73). With an FP64 MPM object
 * the step follows the reference's arithmetic; with a MIXED one the MPM bulk
 * runs in FP32 (positions FP64) and the coupling exchange is formed in FP64
 * from the FP32 grid. */
hg_status hg_hybrid_create(hg_context *ctx, hg_mpm *m, hg_dem *d,
                           hg_hybrid **out);
hg_status hg_hybrid_destroy(hg_hybrid *h);
/* HybridGrains2DSim::stepSystem_constraintSetUp_prediction_correction_
 * advection_node_node (HybridGrains2DSim.cpp:116-220), nsteps times; flags
 * add the per-step ResamplingTools::homogenizeStress / homogenizeVelocity
 * accumulation (ResamplingTools.cpp:744-884). Resampling and zone
 * relabelling run on the host between calls. */
hg_status hg_hybrid_step(hg_hybrid *h, double dt, int32_t nsteps,
                         int32_t flags);
/* ResamplingTools::clearHomogenizedStress / clearHomogenizedVelocity. */
hg_status hg_hybrid_clear_homogenized(hg_hybrid *h);
hg_status hg_hybrid_num_packed(hg_hybrid *h, int64_t *num_grains,
                               int64_t *num_nodes);
/* Coupling buffers of the last step (Coupling.h:52-70): packed coupled
 * grain and node lists, DEM mass/momentum grids, v/a after coupling, grid
 * homog_factor, homogenized stress (4 per node) and velocity (2 per node).
 * Any pointer may be NULL. */
hg_status hg_hybrid_download(hg_hybrid *h, int32_t *packed_grains,
                             int32_t *packed_nodes, double *dem_mass_grid,
                             double *dem_momentum_grid, double *v_after,
                             double *a_after, double *homog_factor,
                             double *homog_stress, double *homog_velocity);

#ifdef __cplusplus
}
#endif

#endif /* HG_GPU_H */
