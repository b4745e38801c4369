// extern "C" entry points of libhg_gpu (declared in include/hg_gpu.h):
// argument validation, host<->device staging and dispatch to the kernels.
#include "hg_internal.cuh"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>
#include <new>
#include <string>
#include <condition_variable>
#include <mutex>
#include <vector>

namespace hg {

std::atomic<int64_t> g_launches{0};
std::atomic<int> g_host_threads{0};
thread_local cudaStream_t t_alloc_stream = nullptr;

namespace {
thread_local std::string t_last_error;
}

void set_error(const std::string &msg) { t_last_error = msg; }

hg_status fail(hg_status s, const std::string &msg) {
  set_error(msg);
  return s;
}

hg_status cuda_fail(cudaError_t e, const char *what) {
  set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? HG_ERR_OUT_OF_MEMORY : HG_ERR_CUDA;
}

const char *last_error_cstr() { return t_last_error.c_str(); }

void context_retain(hg_context *c) { ++c->refs; }

void context_release(hg_context *c) {
  if (--c->refs > 0) return;
  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != c->device) cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  cudaStreamDestroy(c->stream);
  if (c->t0) cudaEventDestroy(c->t0);
  if (c->t1) cudaEventDestroy(c->t1);
  for (cudaEvent_t e : c->fences)
    if (e) cudaEventDestroy(e);
  for (uint32_t *p : c->pinned_chunks) cudaFreeHost(p);
  if (prev >= 0 && prev != c->device) cudaSetDevice(prev);
  delete c;
}

uint32_t *context_pinned_pair(hg_context *c) {
  constexpr int PAIRS_PER_CHUNK = 4096;
  if (c->pinned_free.empty()) {
    uint32_t *chunk = nullptr;
    if (cudaMallocHost(&chunk, 2 * sizeof(uint32_t) * PAIRS_PER_CHUNK) != cudaSuccess)
      return nullptr;
    c->pinned_chunks.push_back(chunk);
    for (int k = PAIRS_PER_CHUNK - 1; k >= 0; --k) c->pinned_free.push_back(chunk + 2 * k);
  }
  uint32_t *p = c->pinned_free.back();
  c->pinned_free.pop_back();
  return p;
}

void context_return_pair(hg_context *c, uint32_t *p) {
  if (p) c->pinned_free.push_back(p);
}

} // namespace hg

using namespace hg;

namespace capi_impl {

// Selects the context's device and makes device buffers allocated in the
// scope stream-ordered on the context's stream.
struct DeviceGuard {
  int prev = -1;
  AllocScope scope;
  explicit DeviceGuard(int dev) : scope(nullptr) { select(dev); }
  explicit DeviceGuard(const hg_context *c) : scope(c->stream) { select(c->device); }
  void select(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
};

bool finite_all(const double *a, int k) {
  for (int i = 0; i < k; ++i)
    if (!std::isfinite(a[i])) return false;
  return true;
}

template <typename T>
hg_status h2d(cudaStream_t s, T *dst, const T *src, size_t n) {
  if (n == 0) return HG_OK;
  // cudaMemcpyDefault: the source may be host or device memory
  HG_CUDA_TRY(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyDefault, s));
  return HG_OK;
}

// The address at which kernels reach p: p itself for device (or managed)
// memory, the mapped address for page-locked host memory; nullptr for
// pageable host memory (and for nullptr), which is copied instead.
template <typename T> T *device_view(T *p) {
  if (!p) return nullptr;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError(); // (clears the error of an unknown pointer)
    return nullptr;
  }
  if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return p;
  if (a.type == cudaMemoryTypeHost && a.devicePointer) return static_cast<T *>(a.devicePointer);
  return nullptr;
}

inline bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

template <typename T>
hg_status d2h(cudaStream_t s, T *dst, const T *src, size_t n) {
  if (n == 0 || dst == nullptr) return HG_OK;
  HG_CUDA_TRY(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyDeviceToHost, s));
  return HG_OK;
}

__global__ void k_fill_d(double *a, int64_t n, double v, int stride, int comp) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) a[(int64_t)stride * i + comp] = v;
}

hg_status fill(cudaStream_t s, double *a, int64_t n, double v, int stride = 1, int comp = 0) {
  if (n <= 0) return HG_OK;
  HG_LAUNCH(k_fill_d, (int)((n + 255) / 256), 256, 0, s, a, n, v, stride, comp);
  HG_CHECK_LAUNCH();
  return HG_OK;
}

__global__ void k_cells_fp64(int64_t n, const double *__restrict__ q, double gx, double gy,
                             double h, int32_t *cells) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= n) return;
  cells[2 * p] = (int32_t)floor((q[2 * p] - gx) / h);
  cells[2 * p + 1] = (int32_t)floor((q[2 * p + 1] - gy) / h);
}

__global__ void k_cells_mixed(int64_t n, const double2 *__restrict__ u,
                              const int32_t *__restrict__ id, int32_t *cells) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int64_t o = id[k];
  const double2 uu = u[k];
  cells[2 * o] = (int32_t)floor(uu.x);
  cells[2 * o + 1] = (int32_t)floor(uu.y);
}

// PhysicsGrid::setDimensions (mpmgrains2d/PhysicsGrid.cpp:14-55).
// Device version of the rasterizeRectangle lattice (InitialSimulationState.
// cpp:48-145): lattice point k = ((gy * nbx + gx) * npd + cy) * npd + cx in
// the host loop order, with the same FP64 expressions (this file is compiled
// without FMA contraction, like the host code), so positions are
// bit-identical to hg_mpm_seed_rectangle.
struct SeedLattice {
  double rmin[2], rmax[2], vel[2], omega, ctr[2], pmass, pvol, half;
  unsigned bx0, by0, nbx, nby;
  int npd;
};

__device__ __forceinline__ bool seed_point(const MpmParams &P, const SeedLattice &L, int64_t k,
                                           double &px, double &py) {
  const int npd = L.npd;
  const int cx = (int)(k % npd), cy = (int)((k / npd) % npd);
  const int64_t cell = k / ((int64_t)npd * npd);
  const unsigned gx = L.bx0 + (unsigned)(cell % L.nbx), gy = L.by0 + (unsigned)(cell / L.nbx);
  px = P.gmin[0] + P.h * ((double)gx + ((double)cx + 0.5) / (double)npd);
  py = P.gmin[1] + P.h * ((double)gy + ((double)cy + 0.5) / (double)npd);
  if (px < L.rmin[0] || py < L.rmin[1] || px > L.rmax[0] || py > L.rmax[1]) return false;
  for (int i = 0; i < P.nplanes; ++i) { // pointInsidePlane
    const MpmPlaneDev &pl = P.planes[i];
    if (py < pl.lower_bound) break;
    if (pl.n[0] * (px - pl.x[0]) + pl.n[1] * (py - pl.x[1]) < 0.0) return false;
  }
  return true;
}

__global__ void k_seed_keep(MpmParams P, SeedLattice L, int64_t total, int32_t *keep) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k > total) return;
  double px, py;
  keep[k] = k < total && seed_point(P, L, k, px, py) ? 1 : 0;
}

__global__ void k_seed_write(MpmParams P, SeedLattice L, int64_t total, int64_t count,
                             const int32_t *__restrict__ keep, const int32_t *__restrict__ off,
                             double *q, double *v, double *mass, double *vol, double *hl) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= total || !keep[k]) return;
  const int64_t o = off[k];
  if (o >= count) return;
  double px, py;
  seed_point(P, L, k, px, py);
  const double ax = px - L.ctr[0], ay = py - L.ctr[1];
  q[2 * o] = px;
  q[2 * o + 1] = py;
  v[2 * o] = L.vel[0] + L.omega * (-ay);
  v[2 * o + 1] = L.vel[1] + L.omega * ax;
  mass[o] = L.pmass;
  vol[o] = L.pvol;
  hl[o] = L.half;
}

void set_dimensions(MpmParams &P, const double gmin[2], const double gmax[2], double h) {
  const double cx = 0.5 * (gmin[0] + gmax[0]), cy = 0.5 * (gmin[1] + gmax[1]);
  double wx = gmax[0] - gmin[0], wy = gmax[1] - gmin[1];
  P.nx = (int)std::ceil(wx / h);
  P.ny = (int)std::ceil(wy / h);
  wx = (double)P.nx * h;
  wy = (double)P.ny * h;
  P.gmin[0] = cx - 0.5 * wx;
  P.gmin[1] = cy - 0.5 * wy;
  P.gmax[0] = cx + 0.5 * wx;
  P.gmax[1] = cy + 0.5 * wy;
  P.h = h;
  P.inv_h = 1.0 / h;
}

} // namespace capi_impl

using namespace capi_impl;

namespace hg {
namespace {

// Worker threads of host_pool_run. A dispatch publishes the task and its
// count under the lock and bumps the generation; workers and the caller
// claim task indices from an atomic counter; the caller waits until every
// claimed task has finished.
struct HostPool {
  std::mutex dispatch;                // one dispatch at a time
  std::mutex m;
  std::condition_variable wake, idle;
  // written under m before next is reset (sequentially consistent), so a
  // worker that claims an index below ntasks sees that dispatch's task
  std::atomic<const std::function<void(size_t)> *> task{nullptr};
  std::atomic<size_t> ntasks{0};
  std::atomic<size_t> next{0};
  size_t running = 0;                 // workers inside the current dispatch
  uint64_t gen = 0;
  size_t nthreads = 0;

  void claim_all() {
    for (size_t i; (i = next.fetch_add(1)) < ntasks.load();) (*task.load())(i);
  }
  void worker() {
    uint64_t seen = 0;
    std::unique_lock<std::mutex> lk(m);
    for (;;) {
      wake.wait(lk, [&] { return gen != seen; });
      seen = gen;
      ++running;
      lk.unlock();
      claim_all();
      lk.lock();
      if (--running == 0) idle.notify_all();
    }
  }
  void run(size_t n, const std::function<void(size_t)> &f) {
    std::lock_guard<std::mutex> d(dispatch);
    {
      std::lock_guard<std::mutex> lk(m);
      const size_t want = std::min<size_t>(n - 1, 15);
      while (nthreads < want) { // the pool lives as long as the process
        std::thread(&HostPool::worker, this).detach();
        ++nthreads;
      }
      task.store(&f);
      ntasks.store(n);
      next.store(0);
      ++gen;
    }
    wake.notify_all();
    claim_all();
    std::unique_lock<std::mutex> lk(m);
    idle.wait(lk, [&] { return running == 0 && next.load() >= ntasks.load(); });
    task.store(nullptr);
  }
};

} // namespace

void host_pool_run(size_t ntasks, const std::function<void(size_t)> &task) {
  static HostPool *pool = new HostPool(); // never destroyed: its threads outlive exit
  if (ntasks == 0) return;
  if (ntasks == 1) {
    task(0);
    return;
  }
  pool->run(ntasks, task);
}

} // namespace hg

extern "C" {

const char *hg_status_string(hg_status s) {
  switch (s) {
  case HG_OK: return "ok";
  case HG_ERR_INVALID_ARGUMENT: return "invalid argument";
  case HG_ERR_CUDA: return "CUDA error";
  case HG_ERR_OUT_OF_MEMORY: return "out of device memory";
  case HG_ERR_CAPACITY: return "capacity exceeded";
  case HG_ERR_UNSUPPORTED: return "unsupported";
  case HG_ERR_DEVICE_STATUS: return "device status word set";
  default: return "unknown status";
  }
}

const char *hg_last_error(void) { return hg::last_error_cstr(); }

int64_t hg_kernel_launch_count(void) { return g_launches.load(); }

hg_status hg_set_host_threads(int32_t n) {
  if (n < 0 || n > 1024) return fail(HG_ERR_INVALID_ARGUMENT, "host threads must be 0 .. 1024");
  g_host_threads.store(n);
  return HG_OK;
}

// ---- context --------------------------------------------------------------

hg_status hg_context_create(int32_t device, hg_context **out) {
  if (!out) return fail(HG_ERR_INVALID_ARGUMENT, "out is NULL");
  *out = nullptr;
  int count = 0;
  HG_CUDA_TRY(cudaGetDeviceCount(&count));
  if (device < 0 || device >= count)
    return fail(HG_ERR_INVALID_ARGUMENT, "device index out of range");
  DeviceGuard g(device);
  hg_context *c = new (std::nothrow) hg_context();
  if (!c) return fail(HG_ERR_OUT_OF_MEMORY, "host allocation failed");
  c->device = device;
  cudaError_t e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    return cuda_fail(e, "context creation");
  }
  // Objects allocate stream-ordered from the device's default pool; keep
  // freed blocks in the pool (this process only) so that scenes created and
  // destroyed while others run reuse memory without returning it to the
  // driver at every synchronisation.
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  *out = c;
  return HG_OK;
}

hg_status hg_context_destroy(hg_context *ctx) {
  if (!ctx) return HG_OK;
  context_release(ctx);
  return HG_OK;
}

hg_status hg_context_timer_begin(hg_context *ctx) {
  if (!ctx) return fail(HG_ERR_INVALID_ARGUMENT, "ctx is NULL");
  DeviceGuard g(ctx);
  if (!ctx->t0) HG_CUDA_TRY(cudaEventCreate(&ctx->t0));
  if (!ctx->t1) HG_CUDA_TRY(cudaEventCreate(&ctx->t1));
  HG_CUDA_TRY(cudaEventRecord(ctx->t0, ctx->stream));
  return HG_OK;
}

hg_status hg_context_timer_end(hg_context *ctx, double *ms) {
  if (!ctx || !ms) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  if (!ctx->t0) return fail(HG_ERR_INVALID_ARGUMENT, "timer not started");
  DeviceGuard g(ctx);
  HG_CUDA_TRY(cudaEventRecord(ctx->t1, ctx->stream));
  HG_CUDA_TRY(cudaEventSynchronize(ctx->t1));
  float f = 0.f;
  HG_CUDA_TRY(cudaEventElapsedTime(&f, ctx->t0, ctx->t1));
  *ms = f;
  return HG_OK;
}

hg_status hg_context_synchronize(hg_context *ctx) {
  if (!ctx) return fail(HG_ERR_INVALID_ARGUMENT, "ctx is NULL");
  DeviceGuard g(ctx);
  HG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return HG_OK;
}

static constexpr int FENCE_RING = 256;

hg_status hg_context_fence(hg_context *ctx, int64_t *fence) {
  if (!ctx || !fence) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  DeviceGuard g(ctx);
  if (ctx->fences.empty()) ctx->fences.assign(FENCE_RING, nullptr);
  const int64_t id = ctx->next_fence;
  cudaEvent_t &e = ctx->fences[id % FENCE_RING];
  if (!e) HG_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  HG_CUDA_TRY(cudaEventRecord(e, ctx->stream));
  ctx->next_fence = id + 1;
  *fence = id;
  return HG_OK;
}

hg_status hg_context_fence_done(hg_context *ctx, int64_t fence, int32_t *done) {
  if (!ctx || !done) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  if (fence < 0 || fence >= ctx->next_fence) return fail(HG_ERR_INVALID_ARGUMENT, "unknown fence");
  DeviceGuard g(ctx);
  // a slot reused by a later fence answers for that one: done then implies
  // done for this one (same stream), not-done is conservative
  const cudaError_t q = cudaEventQuery(ctx->fences[fence % FENCE_RING]);
  if (q != cudaSuccess && q != cudaErrorNotReady) return cuda_fail(q, "fence query");
  *done = q == cudaSuccess ? 1 : 0;
  return HG_OK;
}

hg_status hg_context_fence_wait(hg_context *ctx, int64_t fence) {
  if (!ctx) return fail(HG_ERR_INVALID_ARGUMENT, "ctx is NULL");
  if (fence < 0 || fence >= ctx->next_fence) return fail(HG_ERR_INVALID_ARGUMENT, "unknown fence");
  DeviceGuard g(ctx);
  HG_CUDA_TRY(cudaEventSynchronize(ctx->fences[fence % FENCE_RING]));
  return HG_OK;
}

hg_status hg_context_device_bytes(hg_context *ctx, int64_t *bytes) {
  if (!ctx || !bytes) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  DeviceGuard g(ctx);
  cudaMemPool_t pool;
  HG_CUDA_TRY(cudaDeviceGetDefaultMemPool(&pool, ctx->device));
  uint64_t used = 0;
  HG_CUDA_TRY(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used));
  *bytes = (int64_t)used;
  return HG_OK;
}

hg_status hg_host_alloc(int64_t bytes, void **out) {
  if (!out) return fail(HG_ERR_INVALID_ARGUMENT, "out is NULL");
  *out = nullptr;
  if (bytes <= 0) return fail(HG_ERR_INVALID_ARGUMENT, "bytes must be positive");
  HG_CUDA_TRY(cudaMallocHost(out, (size_t)bytes));
  return HG_OK;
}

hg_status hg_host_free(void *p) {
  if (p) HG_CUDA_TRY(cudaFreeHost(p));
  return HG_OK;
}

// ---- MPM --------------------------------------------------------------------

static hg_status validate_desc(const hg_mpm_desc *d) {
  if (!(d->cell_width > 0.0) || !std::isfinite(d->cell_width))
    return fail(HG_ERR_INVALID_ARGUMENT, "cell_width must be positive and finite");
  if (!finite_all(d->grid_min, 2) || !finite_all(d->grid_max, 2) ||
      !(d->grid_max[0] > d->grid_min[0]) || !(d->grid_max[1] > d->grid_min[1]))
    return fail(HG_ERR_INVALID_ARGUMENT, "grid_max must exceed grid_min");
  if (d->basis != HG_BASIS_LINEAR && d->basis != HG_BASIS_UGIMP)
    return fail(HG_ERR_INVALID_ARGUMENT, "unknown basis");
  if (d->precision != HG_PRECISION_FP64 && d->precision != HG_PRECISION_MIXED)
    return fail(HG_ERR_INVALID_ARGUMENT, "unknown precision");
  if (d->num_planes < 0 || d->num_planes > HG_MAX_PLANES)
    return fail(HG_ERR_INVALID_ARGUMENT, "num_planes out of range");
  if (d->capacity < 0 || d->capacity > (int64_t)INT32_MAX)
    return fail(HG_ERR_INVALID_ARGUMENT, "capacity out of range");
  if (!finite_all(d->gravity, 2)) return fail(HG_ERR_INVALID_ARGUMENT, "gravity not finite");
  const double cw = (d->grid_max[0] - d->grid_min[0]) / d->cell_width;
  const double ch = (d->grid_max[1] - d->grid_min[1]) / d->cell_width;
  if (cw > 1.0e6 || ch > 1.0e6) return fail(HG_ERR_INVALID_ARGUMENT, "grid too large");
  return HG_OK;
}

hg_status hg_mpm_create(hg_context *ctx, const hg_mpm_desc *d, hg_mpm **out) {
  if (!ctx || !d || !out) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  *out = nullptr;
  hg_status vst = validate_desc(d);
  if (vst != HG_OK) return vst;
  DeviceGuard g(ctx);
  hg_mpm *m = new (std::nothrow) hg_mpm();
  if (!m) return fail(HG_ERR_OUT_OF_MEMORY, "host allocation failed");
  m->ctx = ctx;
  context_retain(ctx);
  MpmParams &P = m->p;
  set_dimensions(P, d->grid_min, d->grid_max, d->cell_width);
  P.basis = d->basis;
  P.precision = d->precision;
  P.mu = d->shear_modulus;
  P.kappa = d->bulk_modulus;
  P.dp_alpha = d->dp_alpha;
  P.flip_alpha = d->flip_alpha;
  P.g[0] = d->gravity[0];
  P.g[1] = d->gravity[1];
  P.nplanes = d->num_planes;
  for (int k = 0; k < d->num_planes; ++k) {
    const hg_mpm_plane &pl = d->planes[k];
    const double nn = std::sqrt(pl.n[0] * pl.n[0] + pl.n[1] * pl.n[1]);
    if (!(nn > 0.0) || !finite_all(pl.x, 2) || std::isnan(pl.lower_bound)) {
      hg_mpm_destroy(m);
      return fail(HG_ERR_INVALID_ARGUMENT, "invalid plane");
    }
    MpmPlaneDev &q = P.planes[k];
    q.x[0] = pl.x[0];
    q.x[1] = pl.x[1];
    q.n[0] = pl.n[0] / nn; // StaticPlane.cpp:6-12 normalises the normal
    q.n[1] = pl.n[1] / nn;
    q.sticking = pl.sticking ? 1 : 0;
    q.lower_bound = pl.lower_bound;
    q.ux[0] = (pl.x[0] - P.gmin[0]) / P.h;
    q.ux[1] = (pl.x[1] - P.gmin[1]) / P.h;
    q.ulb = (pl.lower_bound - P.gmin[1]) / P.h;
    q.fn[0] = (float)q.n[0];
    q.fn[1] = (float)q.n[1];
    q.fux[0] = (float)q.ux[0];
    q.fux[1] = (float)q.ux[1];
    q.fulb = (float)q.ulb;
  }
  m->cap = d->capacity;
  hg_status st = m->status.alloc(1);
  if (st == HG_OK) {
    cudaError_t e = cudaMemsetAsync(m->status.p, 0, sizeof(uint32_t), ctx->stream);
    if (e != cudaSuccess) st = cuda_fail(e, "cudaMemsetAsync");
  }
  const int64_t nn = (int64_t)(P.nx + 1) * (P.ny + 1);
  if (st == HG_OK && P.precision == HG_PRECISION_FP64) {
    if ((st = m->q.alloc(2 * m->cap)) || (st = m->v.alloc(2 * m->cap)) ||
        (st = m->m.alloc(m->cap)) || (st = m->vol.alloc(m->cap)) ||
        (st = m->hl.alloc(m->cap)) || (st = m->be.alloc(4 * m->cap)) ||
        (st = m->J.alloc(m->cap)) || (st = m->sigma.alloc(4 * m->cap)) ||
        (st = m->jh.alloc(m->cap)) || (st = m->kin.alloc(m->cap)) ||
        (st = m->g_mass.alloc(nn)) || (st = m->g_mom.alloc(2 * nn)) ||
        (st = m->g_mom_new.alloc(2 * nn)) || (st = m->g_force.alloc(2 * nn)) ||
        (st = m->g_vel.alloc(2 * nn)) || (st = m->g_acc.alloc(2 * nn)) ||
        (st = m->g_cforce.alloc(2 * nn)) || (st = m->g_homog.alloc(nn)) ||
        (st = m->g_hyb.alloc(nn))) {
    } else {
      cudaStream_t s = ctx->stream;
      cudaMemsetAsync(m->g_cforce.p, 0, sizeof(double) * 2 * nn, s);
      cudaMemsetAsync(m->g_hyb.p, 0, sizeof(int32_t) * nn, s);
      cudaMemsetAsync(m->g_mass.p, 0, sizeof(double) * nn, s);
      cudaMemsetAsync(m->g_mom.p, 0, sizeof(double) * 2 * nn, s);
      cudaMemsetAsync(m->g_mom_new.p, 0, sizeof(double) * 2 * nn, s);
      cudaMemsetAsync(m->g_force.p, 0, sizeof(double) * 2 * nn, s);
      cudaMemsetAsync(m->g_vel.p, 0, sizeof(double) * 2 * nn, s);
      cudaMemsetAsync(m->g_acc.p, 0, sizeof(double) * 2 * nn, s);
      st = fill(s, m->g_homog.p, nn, 1.0);
    }
  } else if (st == HG_OK) {
    st = mixed_alloc(m);
  }
  if (st == HG_OK) {
    // no wait for the queued memsets: creating a scene while others step
    // must not drain the stream; errors surface at the next synchronising call
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) st = cuda_fail(e, "hg_mpm_create");
  }
  if (st != HG_OK) {
    hg_mpm_destroy(m);
    return st;
  }
  *out = m;
  return HG_OK;
}

hg_status hg_mpm_destroy(hg_mpm *m) {
  if (!m) return HG_OK;
  hg_context *ctx = m->ctx;
  {
    DeviceGuard g(ctx);
    // buffers are released stream-ordered behind the queued work; the
    // read-back slot goes back to the context's pool for later work
    context_return_pair(ctx, m->h_outside);
    context_return_pair(ctx, m->h_flag);
    if (m->outside_ev) cudaEventDestroy(m->outside_ev);
    for (cudaGraphExec_t &e : m->chunk_exec)
      if (e) cudaGraphExecDestroy(e);
    for (cudaEvent_t e : m->prof_events) cudaEventDestroy(e);
    delete m;
  }
  context_release(ctx);
  return HG_OK;
}

hg_status hg_mpm_grid_info(hg_mpm *m, double gmin[2], double gmax[2], int32_t cc[2]) {
  if (!m) return fail(HG_ERR_INVALID_ARGUMENT, "m is NULL");
  if (gmin) {
    gmin[0] = m->p.gmin[0];
    gmin[1] = m->p.gmin[1];
  }
  if (gmax) {
    gmax[0] = m->p.gmax[0];
    gmax[1] = m->p.gmax[1];
  }
  if (cc) {
    cc[0] = m->p.nx;
    cc[1] = m->p.ny;
  }
  return HG_OK;
}

// InitialSimulationState.cpp:48-145
hg_status hg_mpm_seed_rectangle(hg_mpm *m, const double rmin[2], const double rmax[2],
                                double rho, int32_t npd, const double vel[2], double omega,
                                int64_t cap, double *q, double *v, double *mass,
                                double *volume, double *hl, int64_t *count) {
  if (!m || !rmin || !rmax || !count) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  if (npd <= 0 || !(rho > 0.0)) return fail(HG_ERR_INVALID_ARGUMENT, "bad density or samples");
  if (cap > 0 && (!q || !v || !mass || !volume || !hl))
    return fail(HG_ERR_INVALID_ARGUMENT, "NULL output buffer");
  const MpmParams &P = m->p;
  if (rmin[0] < P.gmin[0] || rmin[1] < P.gmin[1])
    return fail(HG_ERR_INVALID_ARGUMENT,
                "initial rectangle region is below the simulation grid");
  if (rmax[0] > P.gmax[0] || rmax[1] > P.gmax[1])
    return fail(HG_ERR_INVALID_ARGUMENT,
                "initial rectangle region is above the simulation grid");
  const double v0x = vel ? vel[0] : 0.0, v0y = vel ? vel[1] : 0.0;
  const unsigned bx0 = (unsigned)std::floor((rmin[0] - P.gmin[0]) / P.h);
  const unsigned by0 = (unsigned)std::floor((rmin[1] - P.gmin[1]) / P.h);
  const unsigned bx1 = (unsigned)std::ceil((rmax[0] - P.gmin[0]) / P.h);
  const unsigned by1 = (unsigned)std::ceil((rmax[1] - P.gmin[1]) / P.h);
  const double ctrx = 0.5 * (rmin[0] + rmax[0]), ctry = 0.5 * (rmin[1] + rmax[1]);
  const double half = 0.5 * P.h / (double)npd;
  const double pvol = half * half * 4.0;
  const double pmass = rho * pvol;
  int64_t k = 0;
  for (unsigned gy = by0; gy < by1; ++gy)
    for (unsigned gx = bx0; gx < bx1; ++gx)
      for (int cy = 0; cy < npd; ++cy)
        for (int cx = 0; cx < npd; ++cx) {
          const double px = P.gmin[0] + P.h * ((double)gx + ((double)cx + 0.5) / (double)npd);
          const double py = P.gmin[1] + P.h * ((double)gy + ((double)cy + 0.5) / (double)npd);
          if (px < rmin[0] || py < rmin[1] || px > rmax[0] || py > rmax[1]) continue;
          bool inside = false; // pointInsidePlane (InitialSimulationState.cpp:33-43)
          for (int i = 0; i < P.nplanes; ++i) {
            const MpmPlaneDev &pl = P.planes[i];
            if (py < pl.lower_bound) break;
            if (pl.n[0] * (px - pl.x[0]) + pl.n[1] * (py - pl.x[1]) < 0.0) {
              inside = true;
              break;
            }
          }
          if (inside) continue;
          if (k < cap) {
            const double ax = px - ctrx, ay = py - ctry;
            q[2 * k] = px;
            q[2 * k + 1] = py;
            v[2 * k] = v0x + omega * (-ay);
            v[2 * k + 1] = v0y + omega * ax;
            mass[k] = pmass;
            volume[k] = pvol;
            hl[k] = half;
          }
          ++k;
        }
  *count = k;
  return HG_OK;
}

static hg_status upload_impl(hg_mpm *m, int64_t n, const double *q, const double *v,
                             const double *mass, const double *volume, const double *hl,
                             const double *be, const double *J, const int32_t *jh,
                             const uint8_t *kin, bool wait);

hg_status hg_mpm_seed_rectangle_device(hg_mpm *m, const double rmin[2], const double rmax[2],
                                       double rho, int32_t npd, const double vel[2],
                                       double omega, int64_t *count) {
  if (!m || !rmin || !rmax || !count) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  // the count, and the argument checks, of the host version
  hg_status st = hg_mpm_seed_rectangle(m, rmin, rmax, rho, npd, vel, omega, 0, nullptr,
                                       nullptr, nullptr, nullptr, nullptr, count);
  if (st != HG_OK) return st;
  const int64_t n = *count;
  if (n > m->cap) return fail(HG_ERR_CAPACITY, "seeded points exceed the capacity");
  const MpmParams &P = m->p;
  SeedLattice L{};
  L.rmin[0] = rmin[0];
  L.rmin[1] = rmin[1];
  L.rmax[0] = rmax[0];
  L.rmax[1] = rmax[1];
  L.vel[0] = vel ? vel[0] : 0.0;
  L.vel[1] = vel ? vel[1] : 0.0;
  L.omega = omega;
  L.ctr[0] = 0.5 * (rmin[0] + rmax[0]);
  L.ctr[1] = 0.5 * (rmin[1] + rmax[1]);
  L.half = 0.5 * P.h / (double)npd;
  L.pvol = L.half * L.half * 4.0;
  L.pmass = rho * L.pvol;
  L.bx0 = (unsigned)std::floor((rmin[0] - P.gmin[0]) / P.h);
  L.by0 = (unsigned)std::floor((rmin[1] - P.gmin[1]) / P.h);
  const unsigned bx1 = (unsigned)std::ceil((rmax[0] - P.gmin[0]) / P.h);
  const unsigned by1 = (unsigned)std::ceil((rmax[1] - P.gmin[1]) / P.h);
  L.nbx = bx1 > L.bx0 ? bx1 - L.bx0 : 0;
  L.nby = by1 > L.by0 ? by1 - L.by0 : 0;
  L.npd = npd;
  const int64_t total = (int64_t)L.nbx * L.nby * npd * npd;
  if (total + 1 > (int64_t)INT32_MAX) return fail(HG_ERR_INVALID_ARGUMENT, "rectangle too large");
  DeviceGuard g(m->ctx);
  cudaStream_t s = m->ctx->stream;
  DevBuf<int32_t> keep, off, tmp;
  DevBuf<double> pts;
  if ((st = keep.alloc(total + 1)) || (st = off.alloc(total + 1)) ||
      (st = tmp.alloc(scan_tmp_size(total + 1))) || (st = pts.alloc(7 * std::max<int64_t>(n, 1))))
    return st;
  HG_LAUNCH(k_seed_keep, (int)((total + 256) / 256), 256, 0, s, P, L, total, keep.p);
  HG_CHECK_LAUNCH();
  if ((st = exclusive_scan_i32(keep.p, off.p, total + 1, tmp.p, s))) return st;
  double *q = pts.p, *v = q + 2 * n, *ms = v + 2 * n, *vol = ms + n, *hl = vol + n;
  if (total > 0) {
    HG_LAUNCH(k_seed_write, (int)((total + 255) / 256), 256, 0, s, P, L, total, n, keep.p,
              off.p, q, v, ms, vol, hl);
    HG_CHECK_LAUNCH();
  }
  // scratch is released stream-ordered after the upload's copies
  return upload_impl(m, n, q, v, ms, vol, hl, nullptr, nullptr, nullptr, nullptr, false);
}

static hg_status upload_impl(hg_mpm *m, int64_t n, const double *q, const double *v,
                             const double *mass, const double *volume, const double *hl,
                             const double *be, const double *J, const int32_t *jh,
                             const uint8_t *kin, bool wait) {
  if (!m) return fail(HG_ERR_INVALID_ARGUMENT, "m is NULL");
  if (n < 0) return fail(HG_ERR_INVALID_ARGUMENT, "negative particle count");
  if (n > m->cap) return fail(HG_ERR_CAPACITY, "particle count exceeds capacity");
  if (n > 0 && (!q || !v || !mass || !volume))
    return fail(HG_ERR_INVALID_ARGUMENT, "q, v, mass and volume are required");
  if (n > 0 && m->p.basis == HG_BASIS_UGIMP && !hl)
    return fail(HG_ERR_INVALID_ARGUMENT, "hl is required for the uGIMP basis");
  DeviceGuard g(m->ctx);
  cudaStream_t s = m->ctx->stream;
  m->n = n;
  hg_status st = HG_OK;
  if (m->p.precision == HG_PRECISION_FP64) {
    if ((st = h2d(s, m->q.p, q, 2 * n)) || (st = h2d(s, m->v.p, v, 2 * n)) ||
        (st = h2d(s, m->m.p, mass, n)) || (st = h2d(s, m->vol.p, volume, n)))
      return st;
    if (hl) {
      if ((st = h2d(s, m->hl.p, hl, n))) return st;
    } else if ((st = fill(s, m->hl.p, n, 0.0))) {
      return st;
    }
    if (be) {
      if ((st = h2d(s, m->be.p, be, 4 * n))) return st;
    } else {
      HG_CUDA_TRY(cudaMemsetAsync(m->be.p, 0, sizeof(double) * 4 * n, s));
      if ((st = fill(s, m->be.p, n, 1.0, 4, 0)) || (st = fill(s, m->be.p, n, 1.0, 4, 3))) return st;
    }
    if (J) {
      if ((st = h2d(s, m->J.p, J, n))) return st;
    } else if ((st = fill(s, m->J.p, n, 1.0))) {
      return st;
    }
    if (jh) {
      if ((st = h2d(s, m->jh.p, jh, n))) return st;
    } else {
      HG_CUDA_TRY(cudaMemsetAsync(m->jh.p, 0, sizeof(int32_t) * n, s));
    }
    if (kin) {
      if ((st = h2d(s, m->kin.p, kin, n))) return st;
    } else {
      HG_CUDA_TRY(cudaMemsetAsync(m->kin.p, 0, n, s));
    }
    HG_CUDA_TRY(cudaMemsetAsync(m->sigma.p, 0, sizeof(double) * 4 * n, s));
  } else {
    // stage in upload order, then convert and sort on the device (the
    // half-widths only with the uGIMP basis)
    const int64_t nd = (m->p.basis == HG_BASIS_UGIMP ? 12 : 11) * n;
    if (m->stage_d.n < (size_t)nd && (st = m->stage_d.alloc(nd))) return st;
    if (m->stage_i.n < (size_t)n && (st = m->stage_i.alloc(n))) return st;
    if (m->stage_u8.n < (size_t)n && (st = m->stage_u8.alloc(n))) return st;
    double *sq = m->stage_d.p, *sv = sq + 2 * n, *sm = sv + 2 * n, *svol = sm + n,
           *sbe = svol + n, *sJ = sbe + 4 * n, *shl = sJ + n;
    const bool ugimp = m->p.basis == HG_BASIS_UGIMP;
    if (ugimp && n > 0) {
      // per-point half-widths; the FP32 weights of the MIXED kernel take
      // 0 < hl <= h / 2 (the stencil of nodes c-1 .. c+2)
      std::vector<double> h(n);
      HG_CUDA_TRY(cudaMemcpy(h.data(), hl, sizeof(double) * n, cudaMemcpyDefault));
      for (int64_t i = 0; i < n; ++i) {
        const double cells = h[i] / m->p.h;
        if (!(cells > 0.0 && cells <= 0.5))
          return fail(HG_ERR_UNSUPPORTED, "MIXED uGIMP needs 0 < hl <= h / 2");
      }
      m->hl_cells = (float)(h[0] / m->p.h);
    }
    // defaults of the arrays the caller leaves out, ahead of every chunk
    if (!be) {
      HG_CUDA_TRY(cudaMemsetAsync(sbe, 0, sizeof(double) * 4 * n, s));
      if ((st = fill(s, sbe, n, 1.0, 4, 0)) || (st = fill(s, sbe, n, 1.0, 4, 3))) return st;
    }
    if (!J && (st = fill(s, sJ, n, 1.0))) return st;
    if (!jh) HG_CUDA_TRY(cudaMemsetAsync(m->stage_i.p, 0, sizeof(int32_t) * n, s));
    if (!kin) HG_CUDA_TRY(cudaMemsetAsync(m->stage_u8.p, 0, n, s));
    // the copies of upload indices [i0, i1) into the staging arrays
    auto copy = [&](int64_t i0, int64_t i1) -> hg_status {
      const int64_t k = i1 - i0;
      hg_status r;
      if ((r = h2d(s, sq + 2 * i0, q + 2 * i0, 2 * k)) ||
          (r = h2d(s, sv + 2 * i0, v + 2 * i0, 2 * k)) ||
          (r = h2d(s, sm + i0, mass + i0, k)) || (r = h2d(s, svol + i0, volume + i0, k)))
        return r;
      if (be && (r = h2d(s, sbe + 4 * i0, be + 4 * i0, 4 * k))) return r;
      if (J && (r = h2d(s, sJ + i0, J + i0, k))) return r;
      if (jh && (r = h2d(s, m->stage_i.p + i0, jh + i0, k))) return r;
      if (kin && (r = h2d(s, m->stage_u8.p + i0, kin + i0, k))) return r;
      if (ugimp && (r = h2d(s, shl + i0, hl + i0, k))) return r;
      return HG_OK;
    };
    m->primed = false;
    if (wait && n > 0) {
      // arrays the GPU can reach (page-locked host or device memory) are
      // read in place by the conversion kernel, without staging copies
      const double *dq = device_view(q), *dv = device_view(v), *dm = device_view(mass),
                   *dvol = device_view(volume), *dhl = device_view(hl),
                   *dbe = device_view(be), *dJ = device_view(J);
      const int32_t *djh = device_view(jh);
      const uint8_t *dkin = device_view(kin);
      if (dq && dv && dm && dvol && (!ugimp || dhl) && (!be || dbe) && (!J || dJ) &&
          (!jh || djh) && (!kin || dkin))
        return mixed_upload_direct(m, dq, dv, dm, dvol, ugimp ? dhl : nullptr, dbe, dJ, djh,
                                   dkin);
    }
    if ((st = copy(0, n))) return st;
    if (wait) // (synchronises)
      return mixed_upload_direct(m, sq, sv, sm, svol, ugimp ? shl : nullptr, sbe, sJ,
                                 m->stage_i.p, m->stage_u8.p);
    if ((st = mixed_upload(m, sq, sv, sm, svol, ugimp ? shl : nullptr, sbe, sJ, m->stage_i.p,
                           m->stage_u8.p)))
      return st;
  }
  // the caller may reuse its buffers as soon as this returns
  if (wait) HG_CUDA_TRY(cudaStreamSynchronize(s));
  return HG_OK;
}

hg_status hg_mpm_upload(hg_mpm *m, int64_t n, const double *q, const double *v,
                        const double *mass, const double *volume, const double *hl,
                        const double *be, const double *J, const int32_t *jh,
                        const uint8_t *kin) {
  HG_TRACE("hg_mpm_upload");
  return upload_impl(m, n, q, v, mass, volume, hl, be, J, jh, kin, true);
}

hg_status hg_mpm_upload_async(hg_mpm *m, int64_t n, const double *q, const double *v,
                              const double *mass, const double *volume, const double *hl,
                              const double *be, const double *J, const int32_t *jh,
                              const uint8_t *kin) {
  return upload_impl(m, n, q, v, mass, volume, hl, be, J, jh, kin, false);
}

hg_status hg_mpm_frame_async(hg_mpm *m, double *q, double *v) {
  if (!m) return fail(HG_ERR_INVALID_ARGUMENT, "m is NULL");
  DeviceGuard g(m->ctx);
  cudaStream_t s = m->ctx->stream;
  const int64_t n = m->n;
  if (n == 0 || (!q && !v)) return HG_OK;
  hg_status st;
  if (m->p.precision == HG_PRECISION_FP64) {
    if ((st = d2h(s, q, m->q.p, 2 * n)) || (st = d2h(s, v, m->v.p, 2 * n))) return st;
    return HG_OK;
  }
  if (m->stage_d.n < (size_t)(4 * n) && (st = m->stage_d.alloc(4 * n))) return st;
  double *sq = m->stage_d.p, *sv = sq + 2 * n;
  if ((st = mixed_download(m, sq, sv, nullptr, nullptr, nullptr))) return st;
  if ((st = d2h(s, q, sq, 2 * n)) || (st = d2h(s, v, sv, 2 * n))) return st;
  return HG_OK;
}

hg_status hg_mpm_estimate_bytes(const hg_mpm_desc *d, int64_t *bytes) {
  if (!d || !bytes) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  hg_status st = validate_desc(d);
  if (st != HG_OK) return st;
  MpmParams P{};
  set_dimensions(P, d->grid_min, d->grid_max, d->cell_width);
  const int64_t nn = (int64_t)(P.nx + 1) * (P.ny + 1), cap = d->capacity;
  int64_t b = 4; // status word
  if (d->precision == HG_PRECISION_FP64) {
    b += cap * (2 * 16 + 3 * 8 + 32 + 8 + 32 + 4 + 1); // q v | m vol hl | be | J | sigma | jh | kin
    b += nn * (8 + 6 * 16 + 8 + 4);                    // grid fields
  } else {
    const bool ugimp = d->basis == HG_BASIS_UGIMP;
    b += mixed_device_bytes(P.nx, P.ny, cap);
    if (ugimp) b += 2 * 4 * cap; // per-point half-widths, both buffers
    b += 8 * std::max<int64_t>((ugimp ? 12 : 11) * cap, 5 * nn) + cap; // upload / download staging
  }
  b += 4 * 2 * cap; // int staging (upload, cell index)
  *bytes = b;
  return HG_OK;
}

hg_status hg_mpm_download(hg_mpm *m, double *q, double *v, double *be, double *J,
                          int32_t *jh) {
  HG_TRACE("hg_mpm_download");
  if (!m) return fail(HG_ERR_INVALID_ARGUMENT, "m is NULL");
  DeviceGuard g(m->ctx);
  cudaStream_t s = m->ctx->stream;
  const int64_t n = m->n;
  hg_status st;
  if (m->p.precision == HG_PRECISION_FP64) {
    if ((st = d2h(s, q, m->q.p, 2 * n)) || (st = d2h(s, v, m->v.p, 2 * n)) ||
        (st = d2h(s, be, m->be.p, 4 * n)) || (st = d2h(s, J, m->J.p, n)) ||
        (st = d2h(s, jh, m->jh.p, n)))
      return st;
  } else {
    const int64_t nd = 11 * n;
    if (m->stage_d.n < (size_t)nd && (st = m->stage_d.alloc(nd))) return st;
    if (m->stage_i.n < (size_t)n && (st = m->stage_i.alloc(n))) return st;
    double *sq = m->stage_d.p, *sv = sq + 2 * n, *sbe = sv + 2 * n, *sJ = sbe + 4 * n;
    int32_t *sjh = m->stage_i.p;
    // the copies of output indices [i0, i1) out of the staging arrays
    auto copy = [&](int64_t i0, int64_t i1) -> hg_status {
      const int64_t k = i1 - i0;
      hg_status r;
      if ((q && (r = d2h(s, q + 2 * i0, sq + 2 * i0, 2 * k))) ||
          (v && (r = d2h(s, v + 2 * i0, sv + 2 * i0, 2 * k))) ||
          (be && (r = d2h(s, be + 4 * i0, sbe + 4 * i0, 4 * k))) ||
          (J && (r = d2h(s, J + i0, sJ + i0, k))) || (jh && (r = d2h(s, jh + i0, sjh + i0, k))))
        return r;
      return HG_OK;
    };
    // outputs the GPU can reach are written in place by the conversion kernel
    double *dq = device_view(q), *dv = device_view(v), *dbe = device_view(be),
           *dJ = device_view(J);
    int32_t *djh = device_view(jh);
    bool done = false;
    if ((!q || dq) && (!v || dv) && (!be || dbe) && (!J || dJ) && (!jh || djh) &&
        aligned16(dq) && aligned16(dv) && aligned16(dbe) && aligned16(dJ) && aligned16(djh) &&
        (st = mixed_download_direct(m, dq, dv, dbe, dJ, djh, &done)))
      return st;
    if (!done) {
      if ((st = mixed_download(m, sq, sv, sbe, sJ, sjh)) || (st = copy(0, n))) return st;
    }
  }
  HG_CUDA_TRY(cudaStreamSynchronize(s));
  return HG_OK;
}

hg_status hg_mpm_num_particles(hg_mpm *m, int64_t *n) {
  if (!m || !n) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  *n = m->n;
  return HG_OK;
}

hg_status hg_mpm_step(hg_mpm *m, double dt, int32_t nsteps) {
  HG_TRACE("hg_mpm_step");
  if (!m) return fail(HG_ERR_INVALID_ARGUMENT, "m is NULL");
  if (!(dt > 0.0) || !std::isfinite(dt)) return fail(HG_ERR_INVALID_ARGUMENT, "dt must be positive");
  if (nsteps < 0) return fail(HG_ERR_INVALID_ARGUMENT, "negative step count");
  DeviceGuard g(m->ctx);
  if (m->p.precision == HG_PRECISION_MIXED) return mixed_step(m, dt, nsteps);
  for (int k = 0; k < nsteps; ++k) {
    hg_status st;
    if ((st = mpm64_phase0(m)) || (st = mpm64_phase1(m, dt)) || (st = mpm64_phase2(m, dt)))
      return st;
  }
  return HG_OK;
}

hg_status hg_mpm_phase0(hg_mpm *m) {
  if (!m) return fail(HG_ERR_INVALID_ARGUMENT, "m is NULL");
  if (m->p.precision != HG_PRECISION_FP64)
    return fail(HG_ERR_UNSUPPORTED, "phase calls need FP64 precision");
  DeviceGuard g(m->ctx);
  return mpm64_phase0(m);
}

hg_status hg_mpm_phase1(hg_mpm *m, double dt) {
  if (!m) return fail(HG_ERR_INVALID_ARGUMENT, "m is NULL");
  if (m->p.precision != HG_PRECISION_FP64)
    return fail(HG_ERR_UNSUPPORTED, "phase calls need FP64 precision");
  if (!(dt > 0.0)) return fail(HG_ERR_INVALID_ARGUMENT, "dt must be positive");
  DeviceGuard g(m->ctx);
  return mpm64_phase1(m, dt);
}

hg_status hg_mpm_phase2(hg_mpm *m, double dt) {
  if (!m) return fail(HG_ERR_INVALID_ARGUMENT, "m is NULL");
  if (m->p.precision != HG_PRECISION_FP64)
    return fail(HG_ERR_UNSUPPORTED, "phase calls need FP64 precision");
  if (!(dt > 0.0)) return fail(HG_ERR_INVALID_ARGUMENT, "dt must be positive");
  DeviceGuard g(m->ctx);
  return mpm64_phase2(m, dt);
}

hg_status hg_mpm_download_grid(hg_mpm *m, double *mass, double *mom, double *mom_new,
                               double *force, double *vel, double *acc) {
  if (!m) return fail(HG_ERR_INVALID_ARGUMENT, "m is NULL");
  DeviceGuard g(m->ctx);
  cudaStream_t s = m->ctx->stream;
  const int64_t nn = (int64_t)(m->p.nx + 1) * (m->p.ny + 1);
  hg_status st;
  if (m->p.precision == HG_PRECISION_FP64) {
    if ((st = d2h(s, mass, m->g_mass.p, nn)) || (st = d2h(s, mom, m->g_mom.p, 2 * nn)) ||
        (st = d2h(s, mom_new, m->g_mom_new.p, 2 * nn)) ||
        (st = d2h(s, force, m->g_force.p, 2 * nn)) || (st = d2h(s, vel, m->g_vel.p, 2 * nn)) ||
        (st = d2h(s, acc, m->g_acc.p, 2 * nn)))
      return st;
  } else {
    if (mom || mom_new || force)
      return fail(HG_ERR_UNSUPPORTED, "MIXED keeps mass, velocity and acceleration only");
    if (m->stage_d.n < (size_t)(5 * nn) && (st = m->stage_d.alloc(5 * nn))) return st;
    double *sm = m->stage_d.p, *sv = sm + nn, *sa = sv + 2 * nn;
    if ((st = mixed_download_grid(m, sm, sv, sa))) return st;
    if ((st = d2h(s, mass, sm, nn)) || (st = d2h(s, vel, sv, 2 * nn)) ||
        (st = d2h(s, acc, sa, 2 * nn)))
      return st;
  }
  HG_CUDA_TRY(cudaStreamSynchronize(s));
  return HG_OK;
}

hg_status hg_mpm_cell_index(hg_mpm *m, int32_t *cells) {
  if (!m || !cells) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  DeviceGuard g(m->ctx);
  cudaStream_t s = m->ctx->stream;
  const int64_t n = m->n;
  if (n == 0) return HG_OK;
  hg_status st;
  if (m->stage_i.n < (size_t)(2 * n) && (st = m->stage_i.alloc(2 * n))) return st;
  if (m->p.precision == HG_PRECISION_FP64) {
    HG_LAUNCH(k_cells_fp64, (int)((n + 255) / 256), 256, 0, s, n, m->q.p, m->p.gmin[0],
              m->p.gmin[1], m->p.h, m->stage_i.p);
  } else {
    HG_LAUNCH(k_cells_mixed, (int)((n + 255) / 256), 256, 0, s, n, m->mu_[m->cur].p,
              m->mid_[m->cur].p, m->stage_i.p);
  }
  HG_CHECK_LAUNCH();
  if ((st = d2h(s, cells, m->stage_i.p, 2 * n))) return st;
  HG_CUDA_TRY(cudaStreamSynchronize(s));
  return HG_OK;
}

hg_status hg_mpm_status(hg_mpm *m, uint32_t *word) {
  if (!m || !word) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  DeviceGuard g(m->ctx);
  HG_CUDA_TRY(cudaMemcpyAsync(word, m->status.p, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                              m->ctx->stream));
  HG_CUDA_TRY(cudaStreamSynchronize(m->ctx->stream));
  return HG_OK;
}

hg_status hg_mpm_clear_status(hg_mpm *m) {
  if (!m) return fail(HG_ERR_INVALID_ARGUMENT, "m is NULL");
  DeviceGuard g(m->ctx);
  HG_CUDA_TRY(cudaMemsetAsync(m->status.p, 0, sizeof(uint32_t), m->ctx->stream));
  return HG_OK;
}

hg_status hg_mpm_profile(hg_mpm *m, int32_t enable) {
  if (!m) return fail(HG_ERR_INVALID_ARGUMENT, "m is NULL");
  if (m->p.precision != HG_PRECISION_MIXED)
    return fail(HG_ERR_UNSUPPORTED, "kernel profiling covers the MIXED path");
  DeviceGuard g(m->ctx);
  HG_CUDA_TRY(cudaStreamSynchronize(m->ctx->stream));
  m->profile = enable != 0;
  m->prof_used = 0;
  return HG_OK;
}

hg_status hg_mpm_profile_read(hg_mpm *m, double *a, double *b, int64_t *steps) {
  if (!m) return fail(HG_ERR_INVALID_ARGUMENT, "m is NULL");
  DeviceGuard g(m->ctx);
  return mixed_profile_read(m, a, b, steps);
}

hg_status hg_mpm_autotune(hg_mpm *m, double dt, int32_t steps_per_candidate,
                          hg_tune_report *report) {
  HG_TRACE("hg_mpm_autotune");
  if (!m) return fail(HG_ERR_INVALID_ARGUMENT, "m is NULL");
  if (m->p.precision != HG_PRECISION_MIXED)
    return fail(HG_ERR_UNSUPPORTED, "launch shapes apply to the MIXED path");
  if (!(dt > 0.0) || !std::isfinite(dt)) return fail(HG_ERR_INVALID_ARGUMENT, "dt must be positive");
  if (steps_per_candidate < 1 || steps_per_candidate > 100000)
    return fail(HG_ERR_INVALID_ARGUMENT, "steps_per_candidate must lie in [1, 100000]");
  DeviceGuard g(m->ctx);
  return mixed_autotune(m, dt, steps_per_candidate, report);
}

static bool valid_shape(const hg_launch_shape &s) {
  return s.fused_ctas_per_sm >= 0 && s.fused_ctas_per_sm <= 64 && s.update_ctas_per_sm >= 0 &&
         s.update_ctas_per_sm <= 64;
}

hg_status hg_mpm_launch_shape(hg_mpm *m, hg_launch_shape *shape) {
  if (!m || !shape) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  *shape = m->shape;
  return HG_OK;
}

hg_status hg_mpm_set_launch_shape(hg_mpm *m, const hg_launch_shape *shape) {
  if (!m || !shape) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  if (!valid_shape(*shape)) return fail(HG_ERR_INVALID_ARGUMENT, "CTAs per SM must lie in [0, 64]");
  m->shape = *shape;
  m->shape_set = true;
  return HG_OK;
}

// ---- checkpoint / resume ------------------------------------------------------------

#define HG_STATE_API(T, obj, name)                                                          \
  hg_status hg_##name##_state_bytes(T *o, int64_t *bytes) {                                 \
    if (!o || !bytes) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");                \
    DeviceGuard g(o->ctx);                                                                  \
    return name##_state_bytes(o, bytes);                                                    \
  }                                                                                         \
  hg_status hg_##name##_state_save(T *o, void *dst, int64_t bytes) {                        \
    if (!o || !dst) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");                  \
    HG_TRACE("hg_" #name "_state_save");                                                    \
    DeviceGuard g(o->ctx);                                                                  \
    return name##_state_save(o, dst, bytes);                                                \
  }                                                                                         \
  hg_status hg_##name##_state_load(T *o, const void *src, int64_t bytes) {                  \
    if (!o || !src) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");                  \
    HG_TRACE("hg_" #name "_state_load");                                                    \
    DeviceGuard g(o->ctx);                                                                  \
    return name##_state_load(o, src, bytes);                                                \
  }

HG_STATE_API(hg_mpm, m, mpm)
HG_STATE_API(hg_dem, d, dem)
HG_STATE_API(hg_hybrid, h, hybrid)

hg_status hg_tune_save(const char *path) {
  if (!path) return fail(HG_ERR_INVALID_ARGUMENT, "path is NULL");
  return tune_save(path);
}

hg_status hg_tune_load(const char *path) {
  if (!path) return fail(HG_ERR_INVALID_ARGUMENT, "path is NULL");
  return tune_load(path);
}

hg_status hg_tune_clear(void) {
  tune_clear();
  return HG_OK;
}

hg_status hg_mpm_rebin_count(hg_mpm *m, int64_t *count) {
  if (!m || !count) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  *count = m->rebins;
  return HG_OK;
}

// ---- batches ------------------------------------------------------------------------

hg_status hg_batch_create(hg_context *ctx, int32_t max_members, hg_batch **out) {
  if (!ctx || !out) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  *out = nullptr;
  if (max_members < 1 || max_members > HG_MAX_BATCH)
    return fail(HG_ERR_INVALID_ARGUMENT, "max_members must lie in [1, HG_MAX_BATCH]");
  DeviceGuard g(ctx);
  hg_batch *b = new (std::nothrow) hg_batch();
  if (!b) return fail(HG_ERR_OUT_OF_MEMORY, "host allocation failed");
  b->ctx = ctx;
  b->max_members = max_members;
  context_retain(ctx);
  hg_status st = batch_alloc(b);
  if (st != HG_OK) {
    hg_batch_destroy(b);
    return st;
  }
  *out = b;
  return HG_OK;
}

hg_status hg_batch_destroy(hg_batch *b) {
  if (!b) return HG_OK;
  hg_context *ctx = b->ctx;
  {
    DeviceGuard g(ctx);
    cudaStreamSynchronize(ctx->stream);
    batch_free(b);
    delete b;
  }
  context_release(ctx);
  return HG_OK;
}

hg_status hg_batch_add(hg_batch *b, hg_mpm *m, double dt) {
  if (!b || !m) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  if (m->ctx != b->ctx) return fail(HG_ERR_INVALID_ARGUMENT, "member of another context");
  if (m->p.precision != HG_PRECISION_MIXED)
    return fail(HG_ERR_UNSUPPORTED, "batches hold MIXED precision MPM objects");
  if (m->p.basis != HG_BASIS_LINEAR)
    return fail(HG_ERR_UNSUPPORTED, "batches hold MPM objects with the linear basis");
  if (!(dt > 0.0) || !std::isfinite(dt)) return fail(HG_ERR_INVALID_ARGUMENT, "dt must be positive");
  for (hg_mpm *x : b->members)
    if (x == m) return fail(HG_ERR_INVALID_ARGUMENT, "already a member");
  if ((int)b->members.size() >= b->max_members) return fail(HG_ERR_CAPACITY, "batch is full");
  b->members.push_back(m);
  b->dts.push_back(dt);
  b->dirty = true;
  return HG_OK;
}

hg_status hg_batch_remove(hg_batch *b, hg_mpm *m) {
  if (!b || !m) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  for (size_t i = 0; i < b->members.size(); ++i)
    if (b->members[i] == m) {
      b->members.erase(b->members.begin() + i);
      b->dts.erase(b->dts.begin() + i);
      b->dirty = true;
      // its counters may still be in flight: forget the object, keep the slot
      for (hg_mpm *&x : b->out_members)
        if (x == m) x = nullptr;
      return HG_OK;
    }
  return fail(HG_ERR_INVALID_ARGUMENT, "not a member");
}

hg_status hg_batch_size(hg_batch *b, int32_t *n) {
  if (!b || !n) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  *n = (int32_t)b->members.size();
  return HG_OK;
}

hg_status hg_batch_step(hg_batch *b, int32_t nsteps) {
  HG_TRACE("hg_batch_step");
  if (!b) return fail(HG_ERR_INVALID_ARGUMENT, "b is NULL");
  if (nsteps < 0) return fail(HG_ERR_INVALID_ARGUMENT, "negative step count");
  DeviceGuard g(b->ctx);
  const auto t0 = std::chrono::steady_clock::now();
  const hg_status st = batch_step(b, nsteps);
  b->host_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return st;
}

hg_status hg_batch_autotune(hg_batch *b, int32_t steps_per_candidate, hg_tune_report *report) {
  HG_TRACE("hg_batch_autotune");
  if (!b) return fail(HG_ERR_INVALID_ARGUMENT, "b is NULL");
  if (steps_per_candidate < 1 || steps_per_candidate > 100000)
    return fail(HG_ERR_INVALID_ARGUMENT, "steps_per_candidate must lie in [1, 100000]");
  if (b->members.empty()) return fail(HG_ERR_INVALID_ARGUMENT, "the batch has no members");
  DeviceGuard g(b->ctx);
  return batch_autotune(b, steps_per_candidate, report);
}

hg_status hg_batch_launch_shape(hg_batch *b, hg_launch_shape *shape) {
  if (!b || !shape) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  *shape = b->shape;
  return HG_OK;
}

hg_status hg_batch_profile(hg_batch *b, int32_t enable) {
  if (!b) return fail(HG_ERR_INVALID_ARGUMENT, "b is NULL");
  b->profile = enable != 0;
  if (b->profile) b->prof_used = 0;
  return HG_OK;
}

hg_status hg_batch_profile_read(hg_batch *b, double *resort_ms, double *table_ms,
                                double *update_ms, double *fused_ms, int64_t *steps) {
  if (!b) return fail(HG_ERR_INVALID_ARGUMENT, "b is NULL");
  DeviceGuard g(b->ctx);
  double ms[hg_batch::PROF_PHASES];
  hg_status st = batch_profile_read(b, ms, steps);
  if (st != HG_OK) return st;
  if (resort_ms) *resort_ms = ms[0];
  if (table_ms) *table_ms = ms[1];
  if (update_ms) *update_ms = ms[2];
  if (fused_ms) *fused_ms = ms[3];
  return HG_OK;
}

hg_status hg_batch_stats(hg_batch *b, int64_t *member_steps, int64_t *resorts, int64_t *steps,
                         double *host_ms, double *wait_ms) {
  if (!b) return fail(HG_ERR_INVALID_ARGUMENT, "b is NULL");
  if (member_steps) *member_steps = b->member_steps;
  if (resorts) *resorts = b->resorts;
  if (steps) *steps = b->steps;
  if (host_ms) *host_ms = b->host_ms;
  if (wait_ms) *wait_ms = b->wait_ms;
  return HG_OK;
}

// ---- DEM ------------------------------------------------------------------------

hg_status hg_dem_create(hg_context *ctx, const hg_dem_desc *d, hg_dem **out) {
  if (!ctx || !d || !out) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  *out = nullptr;
  if (d->num_planes < 0 || d->num_planes > HG_MAX_PLANES)
    return fail(HG_ERR_INVALID_ARGUMENT, "num_planes out of range");
  if (d->num_drums < 0 || d->num_drums > HG_MAX_DRUMS)
    return fail(HG_ERR_INVALID_ARGUMENT, "num_drums out of range");
  for (int k = 0; k < d->num_drums; ++k)
    if (!finite_all(d->drums[k].x, 2) || !(d->drums[k].r > 0.0) || !std::isfinite(d->drums[k].r))
      return fail(HG_ERR_INVALID_ARGUMENT, "invalid drum");
  if (d->capacity < 0 || d->capacity > (int64_t)(1 << 30) || d->contact_capacity < 0 ||
      d->contact_capacity > (int64_t)INT32_MAX)
    return fail(HG_ERR_INVALID_ARGUMENT, "capacity out of range");
  const double params[7] = {d->gravity[0], d->gravity[1], d->kn, d->kt, d->gamman,
                            d->gammat, d->mu};
  if (!finite_all(params, 7) || d->kn < 0 || d->kt < 0 || d->gamman < 0 || d->gammat < 0 ||
      d->mu < 0)
    return fail(HG_ERR_INVALID_ARGUMENT, "penalty parameters must be finite and >= 0");
  DeviceGuard g(ctx);
  hg_dem *dm = new (std::nothrow) hg_dem();
  if (!dm) return fail(HG_ERR_OUT_OF_MEMORY, "host allocation failed");
  dm->ctx = ctx;
  context_retain(ctx);
  DemParams &P = dm->p;
  P.g[0] = d->gravity[0];
  P.g[1] = d->gravity[1];
  P.kn = d->kn;
  P.kt = d->kt;
  P.gn = d->gamman;
  P.gt = d->gammat;
  P.mu = d->mu;
  P.cell_scale = d->cell_scale;
  if (d->precision != HG_PRECISION_FP64 && d->precision != HG_PRECISION_MIXED) {
    hg_dem_destroy(dm);
    return fail(HG_ERR_INVALID_ARGUMENT, "precision must be HG_PRECISION_FP64 or HG_PRECISION_MIXED");
  }
  P.precision = d->precision;
  dem_set_launch_shapes(dm);
  P.nplanes = d->num_planes;
  for (int k = 0; k < d->num_planes; ++k) {
    const hg_dem_plane &pl = d->planes[k];
    // RigidBody2DSceneParser.cpp:264: planes are built with n.normalized()
    const double n2 = pl.n[0] * pl.n[0] + pl.n[1] * pl.n[1];
    if (!(n2 > 0.0) || !finite_all(pl.x, 2)) {
      hg_dem_destroy(dm);
      return fail(HG_ERR_INVALID_ARGUMENT, "invalid plane");
    }
    const double nn = std::sqrt(n2);
    P.px[k][0] = pl.x[0];
    P.px[k][1] = pl.x[1];
    P.pn[k][0] = pl.n[0] / nn;
    P.pn[k][1] = pl.n[1] / nn;
  }
  P.ndrums = d->num_drums;
  for (int k = 0; k < d->num_drums; ++k) {
    P.dx[k][0] = d->drums[k].x[0];
    P.dx[k][1] = d->drums[k].x[1];
    P.dr[k] = d->drums[k].r;
  }
  dm->cap = d->capacity;
  dm->ccap = d->contact_capacity;
  hg_status st = dem_alloc(dm);
  if (st != HG_OK) {
    hg_dem_destroy(dm);
    return st;
  }
  *out = dm;
  return HG_OK;
}

hg_status hg_dem_destroy(hg_dem *d) {
  if (!d) return HG_OK;
  hg_context *ctx = d->ctx;
  {
    DeviceGuard g(ctx);
    if (d->own) cudaStreamSynchronize(d->own);
    cudaStreamSynchronize(ctx->stream);
    if (d->pair_exec) cudaGraphExecDestroy(d->pair_exec);
    if (d->own) cudaStreamDestroy(d->own);
    if (d->own_ev) cudaEventDestroy(d->own_ev);
    if (d->ctx_ev) cudaEventDestroy(d->ctx_ev);
    delete d;
  }
  context_release(ctx);
  return HG_OK;
}

// Concurrent mode: the DEM's work runs on a stream of its own, so that its
// steps overlap work queued on the context's stream (the MPM steps of a
// serving batch). The two streams meet only at hg_dem_wait_context (the DEM
// waits for what the context's stream has queued) and hg_dem_join (the
// context's stream waits for what the DEM has queued).
hg_status hg_dem_set_concurrent(hg_dem *d, int32_t on) {
  if (!d) return fail(HG_ERR_INVALID_ARGUMENT, "d is NULL");
  DeviceGuard g(d->ctx);
  if (on && !d->own) {
    HG_CUDA_TRY(cudaStreamCreateWithFlags(&d->own, cudaStreamNonBlocking));
    HG_CUDA_TRY(cudaEventCreateWithFlags(&d->own_ev, cudaEventDisableTiming));
    HG_CUDA_TRY(cudaEventCreateWithFlags(&d->ctx_ev, cudaEventDisableTiming));
    // everything queued so far (allocation, uploads) comes first
    HG_CUDA_TRY(cudaEventRecord(d->ctx_ev, d->ctx->stream));
    HG_CUDA_TRY(cudaStreamWaitEvent(d->own, d->ctx_ev, 0));
  } else if (!on && d->own) {
    HG_CUDA_TRY(cudaStreamSynchronize(d->own));
    if (d->pair_exec) { // captured on the own stream; rebuilt on the next step
      cudaGraphExecDestroy(d->pair_exec);
      d->pair_exec = nullptr;
    }
    cudaStreamDestroy(d->own);
    cudaEventDestroy(d->own_ev);
    cudaEventDestroy(d->ctx_ev);
    d->own = nullptr;
    d->own_ev = d->ctx_ev = nullptr;
  }
  return HG_OK;
}

hg_status hg_dem_wait_context(hg_dem *d) {
  if (!d) return fail(HG_ERR_INVALID_ARGUMENT, "d is NULL");
  if (!d->own) return HG_OK;
  DeviceGuard g(d->ctx);
  HG_CUDA_TRY(cudaEventRecord(d->ctx_ev, d->ctx->stream));
  HG_CUDA_TRY(cudaStreamWaitEvent(d->own, d->ctx_ev, 0));
  return HG_OK;
}

hg_status hg_dem_join(hg_dem *d) {
  if (!d) return fail(HG_ERR_INVALID_ARGUMENT, "d is NULL");
  if (!d->own) return HG_OK;
  DeviceGuard g(d->ctx);
  HG_CUDA_TRY(cudaEventRecord(d->own_ev, d->own));
  HG_CUDA_TRY(cudaStreamWaitEvent(d->ctx->stream, d->own_ev, 0));
  return HG_OK;
}

static hg_status dem_upload_impl(hg_dem *d, int64_t n, const double *q, const double *v,
                                 const double *r, const double *mass, const double *inertia,
                                 const uint8_t *fixed, int64_t nmap, const int32_t *old_to_new);

hg_status hg_dem_upload(hg_dem *d, int64_t n, const double *q, const double *v,
                        const double *r, const double *mass, const double *inertia,
                        const uint8_t *fixed) {
  return dem_upload_impl(d, n, q, v, r, mass, inertia, fixed, -1, nullptr);
}

hg_status hg_dem_upload_relabel(hg_dem *d, int64_t n, const double *q, const double *v,
                                const double *r, const double *mass, const double *inertia,
                                const uint8_t *fixed, int64_t n_old, const int32_t *old_to_new) {
  if (n_old < 0 || (n_old > 0 && !old_to_new))
    return fail(HG_ERR_INVALID_ARGUMENT, "invalid body map");
  for (int64_t i = 0; i < n_old; ++i)
    if (old_to_new[i] >= n) return fail(HG_ERR_INVALID_ARGUMENT, "body map points past n");
  return dem_upload_impl(d, n, q, v, r, mass, inertia, fixed, n_old, old_to_new);
}

static hg_status dem_upload_impl(hg_dem *d, int64_t n, const double *q, const double *v,
                                 const double *r, const double *mass, const double *inertia,
                                 const uint8_t *fixed, int64_t nmap, const int32_t *old_to_new) {
  if (!d) return fail(HG_ERR_INVALID_ARGUMENT, "d is NULL");
  if (n < 0) return fail(HG_ERR_INVALID_ARGUMENT, "negative body count");
  if (n > d->cap) return fail(HG_ERR_CAPACITY, "body count exceeds capacity");
  if (n > 0 && (!q || !v || !r || !mass || !inertia))
    return fail(HG_ERR_INVALID_ARGUMENT, "q, v, radius, mass and inertia are required");
  double rmax = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    if (!(r[i] > 0.0) || !(mass[i] > 0.0) || !(inertia[i] > 0.0) || !std::isfinite(r[i]))
      return fail(HG_ERR_INVALID_ARGUMENT, "radius, mass and inertia must be positive");
    rmax = std::max(rmax, r[i]);
  }
  DeviceGuard g(d->ctx);
  AllocScope dem_scope(dem_stream(d)); // temporaries on the DEM's stream
  // Broadphase cell width: the widest disk AABB plus a relative margin, so a
  // disk's partners lie in the 3x3 cells around the cell of its AABB minimum.
  d->cell_h = 2.0 * rmax * (1.0 + 1.0e-6);
  cudaStream_t s = dem_stream(d);
  d->n = n;
  d->inv_valid = false;
  hg_status st;
  if ((st = h2d(s, d->q.p, q, 3 * n)) || (st = h2d(s, d->v.p, v, 3 * n)) ||
      (st = h2d(s, d->r.p, r, n)) || (st = h2d(s, d->m0.p, mass, n)) ||
      (st = h2d(s, d->I0.p, inertia, n)))
    return st;
  if (fixed) {
    if ((st = h2d(s, d->fixed.p, fixed, n))) return st;
  } else {
    HG_CUDA_TRY(cudaMemsetAsync(d->fixed.p, 0, n, s));
  }
  if ((st = fill(s, d->w.p, n, 1.0))) return st;
  if (nmap < 0) {
    if ((st = dem_reset_history(d))) return st;
  } else if ((st = dem_relabel(d, old_to_new, nmap))) {
    return st;
  }
  d->ncontacts_host = 0;
  HG_CUDA_TRY(cudaStreamSynchronize(s));
  return HG_OK;
}

hg_status hg_dem_edit_async(hg_dem *d, int64_t n_old, const int32_t *old_to_new, int64_t n_add,
                            const double *q, const double *v, const double *r,
                            const double *mass, const double *inertia, const uint8_t *fixed) {
  HG_TRACE("hg_dem_edit_async");
  if (!d) return fail(HG_ERR_INVALID_ARGUMENT, "d is NULL");
  if (n_old != d->n) return fail(HG_ERR_INVALID_ARGUMENT, "n_old must be the current body count");
  if (n_add < 0 || (n_old > 0 && !old_to_new)) return fail(HG_ERR_INVALID_ARGUMENT, "invalid edit");
  if (n_add > 0 && (!q || !v || !r || !mass || !inertia))
    return fail(HG_ERR_INVALID_ARGUMENT, "q, v, radius, mass and inertia are required");
  int64_t keep = 0;
  for (int64_t i = 0; i < n_old; ++i) {
    if (old_to_new[i] < 0) continue;
    if (old_to_new[i] != keep) return fail(HG_ERR_INVALID_ARGUMENT, "kept bodies must keep their order");
    ++keep;
  }
  if (keep + n_add > d->cap) return fail(HG_ERR_CAPACITY, "body count exceeds capacity");
  double rmax = 0.0;
  for (int64_t i = 0; i < n_add; ++i) {
    if (!(r[i] > 0.0) || !(mass[i] > 0.0) || !(inertia[i] > 0.0) || !std::isfinite(r[i]))
      return fail(HG_ERR_INVALID_ARGUMENT, "radius, mass and inertia must be positive");
    rmax = std::max(rmax, r[i]);
  }
  DeviceGuard g(d->ctx);
  AllocScope dem_scope(dem_stream(d)); // temporaries on the DEM's stream
  // the broadphase cell only grows: the candidate set does not depend on it
  d->cell_h = std::max(d->cell_h, 2.0 * rmax * (1.0 + 1.0e-6));
  return dem_edit(d, n_old, old_to_new, keep, n_add, q, v, r, mass, inertia, fixed);
}

hg_status hg_dem_frame_async(hg_dem *d, double *q, double *v) {
  if (!d) return fail(HG_ERR_INVALID_ARGUMENT, "d is NULL");
  DeviceGuard g(d->ctx);
  AllocScope dem_scope(dem_stream(d)); // temporaries on the DEM's stream
  hg_status st;
  if ((st = d2h(dem_stream(d), q, d->q.p, 3 * d->n)) || (st = d2h(dem_stream(d), v, d->v.p, 3 * d->n)))
    return st;
  return HG_OK;
}

hg_status hg_dem_num_bodies(hg_dem *d, int64_t *n) {
  if (!d || !n) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  *n = d->n;
  return HG_OK;
}

hg_status hg_dem_set_weights(hg_dem *d, const double *w) {
  if (!d || (!w && d->n > 0)) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  for (int64_t i = 0; i < d->n; ++i)
    if (!(w[i] >= 0.0 && w[i] <= 1.0)) return fail(HG_ERR_INVALID_ARGUMENT, "weights must lie in [0, 1]");
  DeviceGuard g(d->ctx);
  AllocScope dem_scope(dem_stream(d)); // temporaries on the DEM's stream
  hg_status st = h2d(dem_stream(d), d->w.p, w, d->n);
  if (st) return st;
  d->inv_valid = false;
  HG_CUDA_TRY(cudaStreamSynchronize(dem_stream(d)));
  return HG_OK;
}

hg_status hg_dem_set_state(hg_dem *d, const double *q, const double *v) {
  if (!d) return fail(HG_ERR_INVALID_ARGUMENT, "d is NULL");
  DeviceGuard g(d->ctx);
  AllocScope dem_scope(dem_stream(d)); // temporaries on the DEM's stream
  hg_status st;
  if (q && (st = h2d(dem_stream(d), d->q.p, q, 3 * d->n))) return st;
  if (v && (st = h2d(dem_stream(d), d->v.p, v, 3 * d->n))) return st;
  HG_CUDA_TRY(cudaStreamSynchronize(dem_stream(d)));
  return HG_OK;
}

hg_status hg_dem_download(hg_dem *d, double *q, double *v) {
  if (!d) return fail(HG_ERR_INVALID_ARGUMENT, "d is NULL");
  DeviceGuard g(d->ctx);
  AllocScope dem_scope(dem_stream(d)); // temporaries on the DEM's stream
  hg_status st;
  if ((st = d2h(dem_stream(d), q, d->q.p, 3 * d->n)) ||
      (st = d2h(dem_stream(d), v, d->v.p, 3 * d->n)))
    return st;
  HG_CUDA_TRY(cudaStreamSynchronize(dem_stream(d)));
  return HG_OK;
}

// Captures two consecutive DEM steps on the context's stream into a graph
// (once per state: n, dt, weighting, live contact buffer, broadphase cell).
static hg_status dem_pair_graph(hg_dem *d, double dt, int weighted) {
  if (d->pair_exec && d->pair_n == d->n && d->pair_dt == dt && d->pair_weighted == weighted &&
      d->pair_cc == d->cc && d->pair_cell == d->cell_h)
    return HG_OK;
  if (d->pair_exec) {
    cudaGraphExecDestroy(d->pair_exec);
    d->pair_exec = nullptr;
  }
  cudaStream_t s = dem_stream(d);
  const int cc0 = d->cc;
  const bool hv0 = d->history_valid;
  const int64_t l0 = g_launches.load();
  HG_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  hg_status st = dem_step(d, dt, weighted);
  if (st == HG_OK) st = dem_step(d, dt, weighted);
  cudaGraph_t graph = nullptr;
  const cudaError_t e = cudaStreamEndCapture(s, &graph);
  // capturing ran no step: restore the host-side bookkeeping it advanced
  d->cc = cc0;
  d->history_valid = hv0;
  const int64_t launches = g_launches.load() - l0;
  g_launches.fetch_sub(launches, std::memory_order_relaxed);
  if (st != HG_OK) {
    if (graph) cudaGraphDestroy(graph);
    return st;
  }
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
  const cudaError_t ei = cudaGraphInstantiate(&d->pair_exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ei != cudaSuccess) {
    d->pair_exec = nullptr;
    return cuda_fail(ei, "cudaGraphInstantiate");
  }
  d->pair_n = d->n;
  d->pair_dt = dt;
  d->pair_weighted = weighted;
  d->pair_cc = cc0;
  d->pair_cell = d->cell_h;
  d->pair_launches = launches;
  // a pair of replays leaves the live buffer where it started
  d->history_valid = true;
  return HG_OK;
}

hg_status hg_dem_step(hg_dem *d, double dt, int32_t nsteps, int32_t weighted) {
  HG_TRACE("hg_dem_step");
  if (!d) return fail(HG_ERR_INVALID_ARGUMENT, "d is NULL");
  if (!(dt > 0.0) || !std::isfinite(dt)) return fail(HG_ERR_INVALID_ARGUMENT, "dt must be positive");
  if (nsteps < 0) return fail(HG_ERR_INVALID_ARGUMENT, "negative step count");
  DeviceGuard g(d->ctx);
  AllocScope dem_scope(dem_stream(d)); // temporaries on the DEM's stream
  int k = 0;
  if (nsteps >= 4 && d->n > 0) {
    // Repeated steps replay a captured pair of steps: one graph launch in
    // place of about 40 kernel launches and memsets.
    hg_status st = dem_prepare(d, dt);
    if (st == HG_OK) st = dem_pair_graph(d, dt, weighted);
    if (st != HG_OK) return st;
    for (; k + 2 <= nsteps; k += 2) {
      HG_CUDA_TRY(cudaGraphLaunch(d->pair_exec, dem_stream(d)));
      g_launches.fetch_add(d->pair_launches, std::memory_order_relaxed);
    }
  }
  for (; k < nsteps; ++k) {
    hg_status st = dem_step(d, dt, weighted);
    if (st != HG_OK) return st;
  }
  return HG_OK;
}

hg_status hg_dem_num_contacts(hg_dem *d, int64_t *n) {
  if (!d || !n) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  DeviceGuard g(d->ctx);
  AllocScope dem_scope(dem_stream(d)); // temporaries on the DEM's stream
  int32_t c = 0;
  if (d->history_valid) {
    HG_CUDA_TRY(cudaMemcpyAsync(&c, d->c_count.p + d->cc, sizeof(int32_t),
                                cudaMemcpyDeviceToHost, dem_stream(d)));
    HG_CUDA_TRY(cudaStreamSynchronize(dem_stream(d)));
  }
  *n = c;
  return HG_OK;
}

hg_status hg_dem_download_contacts(hg_dem *d, int64_t cap, double *rec, int64_t *count) {
  if (!d || !count || (cap > 0 && !rec)) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  DeviceGuard g(d->ctx);
  AllocScope dem_scope(dem_stream(d)); // temporaries on the DEM's stream
  return dem_download_contacts(d, cap, rec, count);
}

hg_status hg_dem_status(hg_dem *d, uint32_t *word) {
  if (!d || !word) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  DeviceGuard g(d->ctx);
  AllocScope dem_scope(dem_stream(d)); // temporaries on the DEM's stream
  HG_CUDA_TRY(cudaMemcpyAsync(word, d->status.p, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                              dem_stream(d)));
  HG_CUDA_TRY(cudaStreamSynchronize(dem_stream(d)));
  return HG_OK;
}

hg_status hg_dem_candidate_pairs(hg_context *ctx, int64_t n, const double *mn,
                                 const double *mx, int64_t cap, int32_t *pairs,
                                 int64_t *count) {
  if (!ctx || !count || n < 0 || (n > 0 && (!mn || !mx)) || (cap > 0 && !pairs))
    return fail(HG_ERR_INVALID_ARGUMENT, "bad argument");
  if (n > (int64_t)(1 << 30)) return fail(HG_ERR_INVALID_ARGUMENT, "too many boxes");
  for (int64_t i = 0; i < 2 * n; ++i)
    if (!std::isfinite(mn[i]) || !std::isfinite(mx[i]) || !(mn[i] < mx[i]))
      return fail(HG_ERR_INVALID_ARGUMENT, "boxes must be finite with min < max");
  DeviceGuard g(ctx);
  return dem_candidate_pairs(ctx, n, mn, mx, cap, pairs, count);
}

// ---- hybrid ---------------------------------------------------------------------

hg_status hg_hybrid_create(hg_context *ctx, hg_mpm *m, hg_dem *d, hg_hybrid **out) {
  if (!ctx || !m || !d || !out) return fail(HG_ERR_INVALID_ARGUMENT, "NULL argument");
  *out = nullptr;
  if (m->ctx != ctx || d->ctx != ctx)
    return fail(HG_ERR_INVALID_ARGUMENT, "objects belong to another context");
  if (d->own)
    return fail(HG_ERR_UNSUPPORTED, "the hybrid step runs the DEM on the context's stream");
  DeviceGuard g(ctx);
  hg_hybrid *h = new (std::nothrow) hg_hybrid();
  if (!h) return fail(HG_ERR_OUT_OF_MEMORY, "host allocation failed");
  h->ctx = ctx;
  h->m = m;
  h->d = d;
  context_retain(ctx);
  hg_status st = hybrid_alloc(h);
  if (st != HG_OK) {
    hg_hybrid_destroy(h);
    return st;
  }
  *out = h;
  return HG_OK;
}

hg_status hg_hybrid_destroy(hg_hybrid *h) {
  if (!h) return HG_OK;
  hg_context *ctx = h->ctx;
  {
    DeviceGuard g(ctx);
    cudaStreamSynchronize(ctx->stream);
    delete h;
  }
  context_release(ctx);
  return HG_OK;
}

hg_status hg_hybrid_step(hg_hybrid *h, double dt, int32_t nsteps, int32_t flags) {
  if (h && h->d && h->d->own)
    return fail(HG_ERR_UNSUPPORTED, "the hybrid step runs the DEM on the context's stream");
  HG_TRACE("hg_hybrid_step");
  if (!h) return fail(HG_ERR_INVALID_ARGUMENT, "h is NULL");
  if (!(dt > 0.0) || !std::isfinite(dt)) return fail(HG_ERR_INVALID_ARGUMENT, "dt must be positive");
  if (nsteps < 0) return fail(HG_ERR_INVALID_ARGUMENT, "negative step count");
  if (h->m->n > 0 && h->m->cap < 1) return fail(HG_ERR_INVALID_ARGUMENT, "empty MPM object");
  if (h->m->n == 0)
    return fail(HG_ERR_INVALID_ARGUMENT, "the coupling needs at least one material point");
  DeviceGuard g(h->ctx);
  for (int k = 0; k < nsteps; ++k) {
    hg_status st = hybrid_step(h, dt, flags);
    if (st != HG_OK) return st;
  }
  return HG_OK;
}

hg_status hg_hybrid_clear_homogenized(hg_hybrid *h) {
  if (!h) return fail(HG_ERR_INVALID_ARGUMENT, "h is NULL");
  DeviceGuard g(h->ctx);
  return hybrid_clear_homogenized(h);
}

hg_status hg_hybrid_num_packed(hg_hybrid *h, int64_t *ng, int64_t *nn) {
  if (!h) return fail(HG_ERR_INVALID_ARGUMENT, "h is NULL");
  DeviceGuard g(h->ctx);
  hg_status st = hybrid_pack_lists(h);
  if (st != HG_OK) return st;
  int32_t c[2] = {0, 0};
  HG_CUDA_TRY(cudaMemcpyAsync(c, h->counts.p, sizeof(c), cudaMemcpyDeviceToHost, h->ctx->stream));
  HG_CUDA_TRY(cudaStreamSynchronize(h->ctx->stream));
  if (ng) *ng = c[0];
  if (nn) *nn = c[1];
  return HG_OK;
}

hg_status hg_hybrid_download(hg_hybrid *h, int32_t *pg, int32_t *pn, double *dm, double *dp,
                             double *va, double *aa, double *hf, double *hs, double *hv) {
  if (!h) return fail(HG_ERR_INVALID_ARGUMENT, "h is NULL");
  DeviceGuard g(h->ctx);
  cudaStream_t s = h->ctx->stream;
  hg_status st = hybrid_pack_lists(h);
  if (st != HG_OK) return st;
  int32_t c[2] = {0, 0};
  HG_CUDA_TRY(cudaMemcpyAsync(c, h->counts.p, sizeof(c), cudaMemcpyDeviceToHost, s));
  HG_CUDA_TRY(cudaStreamSynchronize(s));
  const int64_t nn = (int64_t)(h->m->p.nx + 1) * (h->m->p.ny + 1);
  if ((st = d2h(s, pg, h->packed_dem.p, c[0])) || (st = d2h(s, pn, h->packed_mpm.p, c[1])) ||
      (st = d2h(s, dm, h->dem_mass.p, nn)) || (st = d2h(s, dp, h->dem_mom.p, 2 * nn)) ||
      (st = d2h(s, va, h->v_after.p, 2 * nn)) || (st = d2h(s, aa, h->a_after.p, 2 * nn)) ||
      (st = d2h(s, hf, h->m->p.precision == HG_PRECISION_MIXED ? h->homog.p : h->m->g_homog.p,
                nn)) ||
      (st = d2h(s, hs, h->hstress.p, 4 * nn)) ||
      (st = d2h(s, hv, h->hvel.p, 2 * nn)))
    return st;
  HG_CUDA_TRY(cudaStreamSynchronize(s));
  return HG_OK;
}

} // extern "C"
