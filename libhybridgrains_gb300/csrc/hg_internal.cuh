// Internal declarations shared by the CUDA translation units of libhg_gpu.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <atomic>
#include <functional>
#include <thread>
#include <utility>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "hg_gpu.h"

namespace hg {

// ---- error handling --------------------------------------------------------

void set_error(const std::string &msg);
hg_status fail(hg_status s, const std::string &msg);
hg_status cuda_fail(cudaError_t e, const char *what);

#define HG_CUDA_TRY(call)                                                     \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess) return ::hg::cuda_fail(e_, #call);                 \
  } while (0)

// Launch bookkeeping: every kernel launch goes through HG_LAUNCH so that the
// number of library kernels launched is observable (hg_kernel_launch_count).
extern std::atomic<int64_t> g_launches;
extern std::atomic<int> g_host_threads; // hg_set_host_threads; 0: default
// An NVTX range over a C-ABI call, for timelines of profiling tools (a no-op
// when no tool is attached).
#ifdef HG_BOUNDS_CHECK
__device__ __forceinline__ bool index_ok(int64_t i, int64_t n, uint32_t *status) {
  if (i >= 0 && i < n) return true;
  atomicOr(status, (uint32_t)HG_STATUS_INDEX);
  return false;
}
#endif

struct TraceRange {
  explicit TraceRange(const char *name) { nvtxRangePushA(name); }
  ~TraceRange() { nvtxRangePop(); }
  TraceRange(const TraceRange &) = delete;
  TraceRange &operator=(const TraceRange &) = delete;
};

#define HG_TRACE(name) ::hg::TraceRange hg_trace_range_(name)

// Index checks of the bounds-checking build (compiled with HG_BOUNDS_CHECK,
// libhg_gpu_bounds.so): a computed index outside [0, n) sets HG_STATUS_INDEX
// in the object's status word and the caller skips the access. In the
// regular build the check is the constant true and compiles away.
#ifdef HG_BOUNDS_CHECK
#define HG_INDEX_OK(i, n, status) ::hg::index_ok((int64_t)(i), (int64_t)(n), (status))
#else
#define HG_INDEX_OK(i, n, status) true
#endif

#define HG_LAUNCH(kernel, grid, block, smem, stream, ...)                     \
  do {                                                                        \
    kernel<<<(grid), (block), (smem), (stream)>>>(__VA_ARGS__);               \
    ::hg::g_launches.fetch_add(1, std::memory_order_relaxed);                 \
  } while (0)

// Programmatic dependent launch: the kernel's CTAs may be scheduled while the
// previous kernel on the stream is finishing (in a captured graph the edge
// becomes programmatic). Such a kernel calls pdl_wait() before its first
// access to global memory, which returns once the previous kernel has
// completed and its writes are visible, and pdl_trigger() to let the next
// kernel be scheduled in turn. After a copy, a memset or an ordinary launch
// the wait returns at once and the ordering is the stream's.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                              cudaStream_t stream, Args &&...args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

#define HG_LAUNCH_PDL(kernel, grid, block, smem, stream, ...)                 \
  do {                                                                        \
    ::hg::launch_pdl(kernel, (grid), (block), (smem), (stream), __VA_ARGS__); \
    ::hg::g_launches.fetch_add(1, std::memory_order_relaxed);                 \
  } while (0)

__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

#define HG_CHECK_LAUNCH()                                                     \
  do {                                                                        \
    cudaError_t e_ = cudaGetLastError();                                      \
    if (e_ != cudaSuccess) return ::hg::cuda_fail(e_, "kernel launch");       \
  } while (0)

// ---- device buffers --------------------------------------------------------

// Stream-ordered allocation. While an AllocScope is active on the calling
// thread, DevBuf allocates with cudaMallocAsync on the scope's stream and
// frees with cudaFreeAsync on the same stream, so creating and destroying
// objects neither waits for queued work nor lets a buffer be reused while a
// queued kernel still reads it. Without a scope it uses cudaMalloc/cudaFree.
extern thread_local cudaStream_t t_alloc_stream;

struct AllocScope {
  cudaStream_t prev;
  explicit AllocScope(cudaStream_t s) : prev(t_alloc_stream) { t_alloc_stream = s; }
  ~AllocScope() { t_alloc_stream = prev; }
};

template <typename T> struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  cudaStream_t s = nullptr; // stream of a stream-ordered allocation
  hg_status alloc(size_t count) {
    free();
    if (count == 0) count = 1;
    cudaError_t e;
    if (t_alloc_stream) {
      e = cudaMallocAsync(reinterpret_cast<void **>(&p), count * sizeof(T), t_alloc_stream);
      s = t_alloc_stream;
    } else {
      e = cudaMalloc(&p, count * sizeof(T));
      s = nullptr;
    }
    if (e != cudaSuccess) {
      p = nullptr;
      return cuda_fail(e, "device allocation");
    }
    n = count;
    return HG_OK;
  }
  void free() {
    if (p) {
      if (s) cudaFreeAsync(p, s);
      else cudaFree(p);
    }
    p = nullptr;
    n = 0;
    s = nullptr;
  }
  ~DevBuf() { free(); }
};

} // namespace hg

// Reference-counted: every MPM/DEM/hybrid object holds a reference, so
// destroying the context before its objects only drops the caller's reference.
struct hg_context {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  int refs = 1;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  // fences: a ring of events recorded on the stream (hg_context_fence)
  std::vector<cudaEvent_t> fences;
  int64_t next_fence = 0;
  // page-locked 8-byte slots for small asynchronous read-backs; a slot is
  // reused only by later work on the same stream, after the earlier copy
  std::vector<uint32_t *> pinned_chunks;
  std::vector<uint32_t *> pinned_free;
};

namespace hg {
// Runs task(0) .. task(ntasks - 1) on the calling thread and the process's
// pool of host worker threads (created on first use, kept for the life of
// the process); returns when all are done. Calls from several host threads
// take turns.
void host_pool_run(size_t ntasks, const std::function<void(size_t)> &task);

// Host loop over [0, n) split into contiguous ranges over the host threads
// (hg_set_host_threads, by default the hardware concurrency up to 16), at
// least min_per_worker items each; f(begin, end) must only write what its
// range owns.
// The host threads the loops below use: hg_set_host_threads, by default the
// hardware concurrency up to 16.
inline size_t host_workers() {
  const int set = g_host_threads.load();
  return set > 0 ? (size_t)set : std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
}

template <typename F>
void host_parallel(size_t n, size_t min_per_worker, F f) {
  const size_t hw = host_workers();
  const size_t workers = std::min(hw, std::max<size_t>(1, n / std::max<size_t>(min_per_worker, 1)));
  if (workers <= 1) {
    f((size_t)0, n);
    return;
  }
  host_pool_run(workers, [&](size_t t) { f(n * t / workers, n * (t + 1) / workers); });
}

// Host loop over [0, n) in ranges of `chunk` items that the host threads
// take in turn as they finish (for loops whose cost per item varies, such as
// rows of a grid with material in a band of it); f(begin, end) must only
// write what its range owns.
template <typename F>
void host_parallel_dynamic(size_t n, size_t chunk, F f) {
  chunk = std::max<size_t>(chunk, 1);
  const size_t hw = host_workers();
  const size_t chunks = (n + chunk - 1) / chunk;
  const size_t workers = std::min(hw, chunks);
  if (workers <= 1) {
    if (n) f((size_t)0, n);
    return;
  }
  std::atomic<size_t> next{0};
  host_pool_run(workers, [&](size_t) {
    for (size_t c = next.fetch_add(1); c < chunks; c = next.fetch_add(1))
      f(c * chunk, std::min(n, (c + 1) * chunk));
  });
}

void context_retain(hg_context *c);
void context_release(hg_context *c);
// two page-locked uint32 words; NULL when page-locked memory is exhausted
uint32_t *context_pinned_pair(hg_context *c);
void context_return_pair(hg_context *c, uint32_t *p);
} // namespace hg

namespace hg {

// ---- MPM -------------------------------------------------------------------

struct MpmPlaneDev {
  double x[2], n[2];
  double lower_bound;
  int sticking;
  // The same plane in grid units: u = (x - grid_min) / h.
  double ux[2];
  double ulb;
  float fux[2], fulb;
  float fn[2]; // the normal in FP32 for the mixed-precision kernels
};

struct MpmParams {
  double gmin[2], gmax[2], h, inv_h;
  int nx, ny; // cell counts; nodes are (nx+1) x (ny+1)
  int basis;
  int precision;
  double mu, kappa, dp_alpha, flip_alpha;
  double g[2];
  int nplanes;
  MpmPlaneDev planes[HG_MAX_PLANES];
};

// Bin (tile) geometry of the MIXED path: a tile is BIN x BIN cells; particles
// are kept sorted by (tile, cell within tile). Tiles also partition the nodes
// for the grid update: node (i, j) belongs to tile (i / BIN, j / BIN).
constexpr int BIN = 16;
constexpr int BIN_CELLS = BIN * BIN;
// Particles may drift this many cells out of their tile before their next
// re-sort and still use the tile's shared-memory windows.
constexpr int DRIFT = 2;
constexpr int VA_W = BIN + 2 * DRIFT + 1;  // G2P node window width
constexpr int ACC_W = BIN + 2 * DRIFT + 3; // P2G node window width

struct MixedParticles {
  double2 *u;     // position in grid units, (x - grid_min) / h
  float2 *v;      // velocity
  float2 *mv;     // mass, volume
  float4 *strain; // (J - 1, be_bar - I: xx, xy, yy)
  uint8_t *flags; // bit0 just_homogenized, bit1 kinematically scripted
  int32_t *id;    // upload index
  float *hl;      // uGIMP half-width in cells (nullptr for the linear basis)
};

} // namespace hg

struct hg_mpm {
  hg_context *ctx = nullptr;
  hg::MpmParams p{};
  int64_t cap = 0, n = 0;
  hg::DevBuf<uint32_t> status;
  // ---- FP64 state (reference layouts: q, v interleaved; be 4 per point) ----
  hg::DevBuf<double> q, v, m, vol, hl, be, J, sigma;
  hg::DevBuf<int32_t> jh;
  hg::DevBuf<uint8_t> kin;
  hg::DevBuf<double> g_mass, g_mom, g_mom_new, g_force, g_vel, g_acc, g_cforce,
      g_homog;
  hg::DevBuf<int32_t> g_hyb;
  // ---- MIXED state ----
  hg::DevBuf<double2> mu_[2];
  hg::DevBuf<float2> mv_[2], mmv_[2];
  hg::DevBuf<float4> mstrain_[2];
  hg::DevBuf<uint8_t> mflags_[2];
  hg::DevBuf<int32_t> mid_[2];
  hg::DevBuf<float> mhl_[2]; // uGIMP only
  int cur = 0; // which buffer of the pairs above is live
  // uGIMP: the half-width of the first uploaded point in cells (the grains'
  // stencil half-width of the hybrid coupling, points.hl(0))
  float hl_cells = 0.f;
  hg::DevBuf<float4> acc4; // (px, py, fx, fy) accumulated for the next update
  hg::DevBuf<float> accm;  // mass accumulated for the next update
  hg::DevBuf<float4> va;   // (vx, vy, ax, ay) of the last update
  hg::DevBuf<float> gm;    // mass of the last update
  int ntx = 0, nty = 0;    // tiles in x, y
  hg::DevBuf<int32_t> keys, counts, offsets, cursor, scan_tmp;
  hg::DevBuf<int32_t> active_bins, active_tiles, nactive; // nactive[2]
  hg::DevBuf<uint32_t> outside; // particles outside their window last step
  uint32_t *h_outside = nullptr; // pinned mirror
  cudaEvent_t outside_ev = nullptr;
  bool outside_pending = false;
  int64_t steps_since_rebin = 0;
  int64_t rebins = 0;
  bool primed = false;
  // launch shape of the MIXED kernels (0: built-in); set explicitly or by
  // the autotuner, else looked up in the tuning table at priming
  hg_launch_shape shape{0, 0};
  bool shape_set = false;
  // CHUNK_STEPS steps captured as a CUDA graph, one per live buffer; rebuilt
  // when dt, the point count or the launch shape changes
  cudaGraphExec_t chunk_exec[2] = {nullptr, nullptr};
  double chunk_dt[2] = {0.0, 0.0};
  int64_t chunk_n[2] = {-1, -1};
  hg_launch_shape chunk_shape[2] = {{-1, -1}, {-1, -1}};
  int64_t chunk_launches = 0;
  // per-kernel event timing (hg_mpm_profile)
  bool profile = false;
  std::vector<cudaEvent_t> prof_events; // 3 per recorded step
  size_t prof_used = 0;
  // host-side staging for upload/download conversion
  hg::DevBuf<double> stage_d;
  hg::DevBuf<int32_t> stage_i;
  hg::DevBuf<uint8_t> stage_u8;
  // MIXED: the live buffer's order as the last single-object re-sort left
  // it: inv[i] is the slot of upload index i, skey[slot] the cell key the
  // slot was sorted under; order_valid while they describe the live buffer
  hg::DevBuf<int32_t> inv, skey;
  bool order_valid = false;
  int64_t order_n = 0; // the point count they were written for
  hg::DevBuf<uint32_t> d_flag; // points outside their slot's window at upload
  uint32_t *h_flag = nullptr;  // pinned mirror (a pair slot of the context)
};

namespace hg {

hg_status mpm64_phase0(hg_mpm *m);
hg_status mpm64_phase1(hg_mpm *m, double dt);
hg_status mpm64_phase2(hg_mpm *m, double dt);

hg_status mixed_alloc(hg_mpm *m);
// hl: device array of half-widths (world units) for the uGIMP basis, else
// nullptr
hg_status mixed_upload(hg_mpm *m, const double *q, const double *v,
                       const double *mass, const double *vol, const double *hl,
                       const double *be, const double *J, const int32_t *jh,
                       const uint8_t *kin);
hg_status mixed_download(hg_mpm *m, double *q, double *v, double *be,
                         double *J, int32_t *jh);
// Transfers of the MIXED state straight between the caller's arrays (in the
// reference's layouts, page-locked host or device memory) and the particle
// buffers, by kernels that read or write them over the host link.
// mixed_upload_direct: when the live buffer's order is still known (same
// point count, nothing re-sorted it since) the points go to their slots and
// the re-sort is skipped unless a point left its slot's tile window.
// Absent be, J, jh, kin take the identity, 1, 0, 0. Synchronises.
hg_status mixed_upload_direct(hg_mpm *m, const double *q, const double *v, const double *mass,
                              const double *vol, const double *hl, const double *be,
                              const double *J, const int32_t *jh, const uint8_t *kin);
// mixed_download_direct: every output index from its slot; false in *done
// when the order is unknown (the caller then takes mixed_download). Absent
// outputs are skipped. Queued on the context's stream.
hg_status mixed_download_direct(hg_mpm *m, double *q, double *v, double *be, double *J,
                                int32_t *jh, bool *done);
hg_status mixed_step(hg_mpm *m, double dt, int nsteps);
hg_status mixed_download_grid(hg_mpm *m, double *mass, double *vel,
                              double *acc);
// device bytes mixed_alloc plus the staging of an upload allocate
int64_t mixed_device_bytes(int nx, int ny, int64_t cap);
hg_status mixed_autotune(hg_mpm *m, double dt, int steps, hg_tune_report *report);
hg_status batch_autotune(hg_batch *b, int steps, hg_tune_report *report);
hg_status mpm_state_bytes(hg_mpm *m, int64_t *bytes);
hg_status mpm_state_save(hg_mpm *m, void *dst, int64_t bytes);
hg_status mpm_state_load(hg_mpm *m, const void *src, int64_t bytes);
hg_status dem_state_bytes(hg_dem *d, int64_t *bytes);
hg_status dem_state_save(hg_dem *d, void *dst, int64_t bytes);
hg_status dem_state_load(hg_dem *d, const void *src, int64_t bytes);
hg_status hybrid_state_bytes(hg_hybrid *h, int64_t *bytes);
hg_status hybrid_state_save(hg_hybrid *h, void *dst, int64_t bytes);
hg_status hybrid_state_load(hg_hybrid *h, const void *src, int64_t bytes);
hg_status tune_save(const char *path);
hg_status tune_load(const char *path);
void tune_clear();
hg_status mixed_profile_read(hg_mpm *m, double *g2p2g_ms, double *update_ms,
                             int64_t *steps);

} // namespace hg

struct hg_batch {
  static constexpr int NBUF = 4;        // page-locked argument tables in flight
  static constexpr int PROF_PHASES = 4; // re-sorts, table copy, grid update, fused
  struct Sig { // what an argument-table entry depends on
    hg_mpm *m = nullptr;
    int cur = -1;
    int64_t n = -1;
    double dt = 0.0;
    bool operator==(const Sig &o) const {
      return m == o.m && cur == o.cur && n == o.n && dt == o.dt;
    }
  };
  hg_context *ctx = nullptr;
  int max_members = 0;
  std::vector<hg_mpm *> members;
  std::vector<double> dts;
  std::vector<Sig> sigs;
  std::vector<unsigned char> args; // host copy of the argument table
  bool dirty = true;
  hg::DevBuf<unsigned char> table; // [update args | fused args] per member
  unsigned char *h_table[NBUF] = {};
  cudaEvent_t table_ev[NBUF] = {};
  int tb = 0;
  // batched re-sort: members due this step and their argument tables
  std::vector<hg_mpm *> due;
  hg::DevBuf<unsigned char> rtable;
  unsigned char *h_rtable[NBUF] = {};
  cudaEvent_t rtable_ev[NBUF] = {};
  int rb = 0;
  hg::DevBuf<uint32_t> outside; // 2 counters per member
  // work queues of the batched kernels: [fused cursor, fused done, update
  // cursor, update done], zero between launches
  hg::DevBuf<int32_t> queue;
  uint32_t *h_outside = nullptr;
  cudaEvent_t out_ev = nullptr;
  bool out_pending = false;
  std::vector<hg_mpm *> out_members; // members whose counters are in flight
  // CHUNK_STEPS steps of all members captured as a CUDA graph (kernels read
  // the argument table through a fixed pointer, so only the member count
  // keys it)
  cudaGraphExec_t chunk_exec = nullptr;
  int chunk_members = -1;
  hg_launch_shape chunk_shape{-1, -1};
  int64_t chunk_launches = 0;
  // launch shape of the batched kernels and the size class it was looked
  // up for (the total point count changes as members come and go)
  hg_launch_shape shape{0, 0};
  bool shape_set = false;
  int64_t shape_class = -1;
  int64_t member_steps = 0, resorts = 0, steps = 0;
  double host_ms = 0.0, wait_ms = 0.0; // wait: host blocked on the device
  bool profile = false;
  std::vector<cudaEvent_t> prof_events; // PROF_PHASES + 1 per step
  size_t prof_used = 0;
};

namespace hg {
hg_status batch_alloc(hg_batch *b);
void batch_free(hg_batch *b);
hg_status batch_step(hg_batch *b, int nsteps);
// per-phase milliseconds [re-sorts, table copy, grid update, fused] summed
// over the profiled steps
hg_status batch_profile_read(hg_batch *b, double *ms, int64_t *steps);

// ---- DEM ---------------------------------------------------------------------

struct DemParams {
  double g[2];
  double kn, kt, gn, gt, mu;
  double cell_scale;
  int precision; // HG_PRECISION_FP64 (bit-exact) or HG_PRECISION_MIXED
  int nplanes;
  double px[HG_MAX_PLANES][2], pn[HG_MAX_PLANES][2];
  // static drums; their contacts share the plane contacts' list as static
  // objects nplanes .. nplanes + ndrums - 1
  int ndrums;
  double dx[HG_MAX_DRUMS][2], dr[HG_MAX_DRUMS];
};

} // namespace hg

struct hg_dem {
  hg_context *ctx = nullptr;
  // concurrent mode (hg_dem_set_concurrent): the DEM runs on a stream of its
  // own, ordered against the context's stream only at explicit joins
  cudaStream_t own = nullptr;
  cudaEvent_t own_ev = nullptr, ctx_ev = nullptr;
  hg::DemParams p{};
  int64_t cap = 0, ccap = 0, n = 0;
  hg::DevBuf<uint32_t> status;
  // bodies
  hg::DevBuf<double> q, v, r, m0, I0, w;
  // per body (as double4): gravity force x, y; dt / M; dt / Mi
  hg::DevBuf<double> minv;
  bool inv_valid = false;  // minv matches m0, I0, w and terms_dt
  double terms_dt = 0.0;
  hg::DevBuf<uint8_t> fixed;
  // broadphase: hash grid of cell width H over the AABB minima
  double cell_h = 0.0;
  uint32_t mask = 0; // hash table size - 1 at the capacity
  // per body, 32 bytes: FP32 offset from the home cell, radius, flags; home cell
  hg::DevBuf<float4> brec;
  hg::DevBuf<uint32_t> plist;  // partners kept by the counting pass
  hg::DevBuf<int32_t> pfill;   // partners credited per body in the counting pass
  hg::DevBuf<int32_t> bcount, bstart, items; // bstart holds bucket ends after the fill
  hg::DevBuf<int32_t> scan_tmp;
  // contacts: current and previous, sorted by (kind, first, second)
  hg::DevBuf<int32_t> c_count; // contacts in ckey[0], ckey[1] (device)
  hg::DevBuf<int32_t> overflow; // set when this step's contacts exceed ccap
  hg::DevBuf<int32_t> per_body, per_body_off; // emission counts / offsets
  hg::DevBuf<int64_t> ckey[2];                 // kind << 60 | first << 30 | second
  hg::DevBuf<double> crec[2];                  // HG_DEM_RECORD_WIDTH per contact
  int cc = 0;                                  // live contact buffer
  int64_t ncontacts_host = 0;                  // count after the last step
  bool history_valid = false;
  int contact_grid = 0; // blocks of the contact law's grid-stride launch
  // body gather lists for deterministic force accumulation
  hg::DevBuf<int32_t> in_count, in_off, in_list, in_cursor;
  hg::DevBuf<int32_t> out_off; // first contact index of each body
  // two steps captured as a CUDA graph (the contact buffers alternate, so a
  // pair of steps returns to the same pointers); rebuilt when n, dt, the
  // weighting, the live buffer or the broadphase cell change
  cudaGraphExec_t pair_exec = nullptr;
  int64_t pair_n = -1, pair_launches = 0;
  double pair_dt = 0.0, pair_cell = 0.0;
  int pair_weighted = -1, pair_cc = -1;
};

namespace hg {
// the stream a DEM object's work runs on
inline cudaStream_t dem_stream(const hg_dem *d) { return d->own ? d->own : d->ctx->stream; }
hg_status dem_alloc(hg_dem *d);
hg_status dem_reset_history(hg_dem *d);
// renumber the contact history by old_to_new (-1: removed) of nmap bodies
hg_status dem_relabel(hg_dem *d, const int32_t *old_to_new, int64_t nmap);
hg_status dem_relabel_device(hg_dem *d, const int32_t *old_to_new, int64_t nmap);
// remove bodies by old_to_new and append n_add bodies, on the device, queued
hg_status dem_edit(hg_dem *d, int64_t n_old, const int32_t *old_to_new, int64_t n_keep,
                   int64_t n_add, const double *q, const double *v, const double *r,
                   const double *m, const double *I, const uint8_t *fixed);
hg_status dem_step(hg_dem *d, double dt, int weighted);
void dem_set_launch_shapes(hg_dem *d);
// per-body terms that dem_step needs and that only change with the bodies
// or the time step; called before a step is captured into a graph
hg_status dem_prepare(hg_dem *d, double dt);
hg_status dem_download_contacts(hg_dem *d, int64_t cap, double *rec,
                                int64_t *count);
hg_status dem_candidate_pairs(hg_context *ctx, int64_t n, const double *mn,
                              const double *mx, int64_t cap, int32_t *pairs,
                              int64_t *count);
hg_status exclusive_scan_i32(const int32_t *in, int32_t *out, int64_t n,
                             int32_t *tmp, cudaStream_t s);
// Elements per tile of exclusive_scan_i32 (256 threads x 8 elements).
constexpr int SCAN_TILE_ELEMS = 2048;
// Ints of temporary storage exclusive_scan_i32 needs for n elements: two per
// tile at every level of the recursive scan of tile sums, plus two.
constexpr int64_t scan_tmp_size(int64_t n) {
  int64_t total = 0;
  while (n > SCAN_TILE_ELEMS) {
    const int64_t tiles = (n + SCAN_TILE_ELEMS - 1) / SCAN_TILE_ELEMS;
    total += 2 * tiles;
    n = tiles;
  }
  return total + 2;
}
// A capacity limit checked by the scan that produces the offsets: when the
// total exceeds limit (>= 0), *overflow is set, status_bit raised in
// *status and every count and offset written as zero; *total (when given)
// receives the total, or 0 when the limit is exceeded.
struct ScanLimit {
  int64_t limit = -1;
  int32_t *overflow = nullptr;
  uint32_t *status = nullptr;
  uint32_t status_bit = 0;
  int32_t *total = nullptr;
};
// The largest n exclusive_scan_i32_limited takes (one CTA, one launch).
int64_t small_scan_max();
hg_status exclusive_scan_i32_limited(int32_t *in, int32_t *out, int64_t n, const ScanLimit &lim,
                                     cudaStream_t s);
} // namespace hg

struct hg_hybrid {
  hg_context *ctx = nullptr;
  hg_mpm *m = nullptr;
  hg_dem *d = nullptr;
  hg::DevBuf<double> dem_mass, dem_mom, v_after, a_after, pos_before,
      hstress, hvel, hmom, hmass;
  hg::DevBuf<int32_t> coupled, packed_dem, packed_mpm, flag_tmp, scan_tmp,
      node_flag, node_pos, counts; // counts[2]: packed sizes
  int64_t n_packed_dem = 0, n_packed_mpm = 0;
  // the packed lists (and counts) describe the last step; built on demand
  bool packed_valid = false;
  int64_t step_bodies = 0; // DEM bodies at the last step
  // with a MIXED MPM object: the node homogenisation factors (an FP64 object
  // keeps them in its grid) and the points' half-width hl(0) in world units
  hg::DevBuf<double> homog, hl0;
  double hl0_value = -1.0;
};

namespace hg {
// The MIXED step in the three parts the hybrid step interleaves with the
// coupling: re-sort if due (this step's P2G sums are then in accm/acc4), the
// grid update (gm, va), and G2P of this step fused with P2G of the next.
hg_status mixed_step_begin(hg_mpm *m);
hg_status mixed_grid_update(hg_mpm *m, double dt);
hg_status mixed_particles(hg_mpm *m, double dt);
hg_status hybrid_alloc(hg_hybrid *h);
hg_status hybrid_step(hg_hybrid *h, double dt, int flags);
hg_status hybrid_clear_homogenized(hg_hybrid *h);
// The last step's coupled grains and nodes as packed index lists in the
// reference's stable-partition order, for callers that read them.
hg_status hybrid_pack_lists(hg_hybrid *h);
} // namespace hg
