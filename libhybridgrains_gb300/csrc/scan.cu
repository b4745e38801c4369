// Device-wide exclusive prefix sum of int32 counts (counting-sort offsets for
// the particle re-sort and the DEM contact lists).
//
// Three phases over tiles of SCAN_TILE elements: per-tile sums, a recursive
// scan of the tile sums, and a per-tile scan that adds the tile offset. Tiles
// are read with coalesced 32-bit loads; the whole pass streams the counts
// twice, which is the floor for a scan that does not fuse into its producer.
#include "hg_internal.cuh"
#include "scan_block.cuh"

namespace hg {

namespace {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;
static_assert(SCAN_TILE == SCAN_TILE_ELEMS, "scan_tmp_size assumes this tile size");

__global__ void k_tile_sums(const int32_t *__restrict__ in, int64_t n,
                            int32_t *__restrict__ sums) {
  // (launched with programmatic dependence on the kernel before it)
  pdl_wait();
  pdl_trigger();
  const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
  int s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    const int64_t i = base + k * SCAN_THREADS + threadIdx.x;
    if (i < n) s += in[i];
  }
  int total;
  block_excl_scan<SCAN_THREADS>(s, &total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void k_tile_scan(const int32_t *__restrict__ in, int64_t n,
                            const int32_t *__restrict__ tile_off,
                            int32_t *__restrict__ out) {
  // (launched with programmatic dependence on the kernel before it)
  pdl_wait();
  pdl_trigger();
  const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
  // Each thread owns SCAN_ITEMS consecutive elements.
  int v[SCAN_ITEMS];
  int s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    const int64_t i = base + (int64_t)threadIdx.x * SCAN_ITEMS + k;
    v[k] = i < n ? in[i] : 0;
    s += v[k];
  }
  int total;
  int run = block_excl_scan<SCAN_THREADS>(s, &total) + (tile_off ? tile_off[blockIdx.x] : 0);
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    const int64_t i = base + (int64_t)threadIdx.x * SCAN_ITEMS + k;
    if (i < n) out[i] = run;
    run += v[k];
  }
}

// The per-tile scan of a device-wide scan with few tiles: each CTA forms its
// tile's offset itself, summing the sums of the tiles before it (at most
// FUSED_TILES of them, a few loads per thread), so that the scan of the tile
// sums needs no launch of its own.
constexpr int64_t FUSED_TILES = 2048;

__global__ void k_tile_scan_summed(const int32_t *__restrict__ in, int64_t n,
                                   const int32_t *__restrict__ sums,
                                   int32_t *__restrict__ out) {
  // (launched with programmatic dependence on the kernel before it)
  pdl_wait();
  pdl_trigger();
  int before = 0;
  for (int k = threadIdx.x; k < (int)blockIdx.x; k += SCAN_THREADS) before += sums[k];
  int tile_off;
  block_excl_scan<SCAN_THREADS>(before, &tile_off);
  const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
  int v[SCAN_ITEMS];
  int s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    const int64_t i = base + (int64_t)threadIdx.x * SCAN_ITEMS + k;
    v[k] = i < n ? in[i] : 0;
    s += v[k];
  }
  int total;
  int run = block_excl_scan<SCAN_THREADS>(s, &total) + tile_off;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    const int64_t i = base + (int64_t)threadIdx.x * SCAN_ITEMS + k;
    if (i < n) out[i] = run;
    run += v[k];
  }
}

// Up to small_scan_max() elements: one CTA and one launch in place of three
// (in a captured step the launches, not the bytes, are the cost at these
// sizes). Thread t owns the SMALL_ITEMS consecutive elements from
// t * SMALL_ITEMS: it reads them as 16-byte vectors (all loads in flight at
// once), scans them sequentially in registers, and one block scan of the
// 1,024 thread totals gives each run its offset. The chain of dependent steps
// is one pass over 32 registers and one block scan, instead of 32 warp scans.
// No large shared-memory staging, so the launch needs no change of the
// shared-memory carve-out.
constexpr int SMALL_THREADS = 1024;
constexpr int SMALL_ITEMS = 32;
constexpr int SMALL_N = SMALL_THREADS * SMALL_ITEMS;
static_assert(SMALL_ITEMS % 4 == 0, "runs are read as int4");

__global__ void __launch_bounds__(SMALL_THREADS)
    k_small_scan(int32_t *__restrict__ in, int64_t n64, int32_t *__restrict__ out, ScanLimit lim) {
  // (launched with programmatic dependence on the kernel before it)
  pdl_wait();
  pdl_trigger();
  const int n = (int)n64; // <= SMALL_N
  // Each warp owns 32 x SMALL_ITEMS consecutive counts, read and written in
  // rows of 128 (4 per lane: one coalesced 512-byte access per row); each
  // row is scanned across the warp, the rows one after another.
  constexpr int ROWS = SMALL_ITEMS / 4;
  const int lane = threadIdx.x & 31;
  const int wbase = (threadIdx.x >> 5) * (32 * SMALL_ITEMS);
  const bool vec =
      ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15u) == 0 &&
      wbase + 32 * SMALL_ITEMS <= n;
  int v[ROWS][4];
#pragma unroll
  for (int r = 0; r < ROWS; ++r) {
    const int i = wbase + 128 * r + 4 * lane;
    if (vec) {
      const int4 q = *reinterpret_cast<const int4 *>(in + i);
      v[r][0] = q.x;
      v[r][1] = q.y;
      v[r][2] = q.z;
      v[r][3] = q.w;
    } else {
#pragma unroll
      for (int j = 0; j < 4; ++j) v[r][j] = i + j < n ? in[i + j] : 0;
    }
  }
  // pre[r]: the offset of the lane's first count of row r in the warp's run
  int pre[ROWS];
  int carry = 0;
#pragma unroll
  for (int r = 0; r < ROWS; ++r) {
    const int x = v[r][0] + v[r][1] + v[r][2] + v[r][3];
    const int inc = warp_incl_scan(x);
    pre[r] = carry + inc - x;
    carry += __shfl_sync(0xffffffffu, inc, 31);
  }
  // the warps' runs: lane 31 carries its warp's total, so every lane's
  // exclusive prefix is the sum of the warps before its own
  int total;
  const int off = block_excl_scan<SMALL_THREADS>(lane == 31 ? carry : 0, &total);
  // the same decision in every thread: the total is block-wide
  const bool over = lim.limit >= 0 && (int64_t)total > lim.limit;
  if (threadIdx.x == 0) {
    if (lim.overflow) *lim.overflow = over ? 1 : 0;
    if (over && lim.status) atomicOr(lim.status, lim.status_bit);
    if (lim.total) *lim.total = over ? 0 : total;
  }
#pragma unroll
  for (int r = 0; r < ROWS; ++r) {
    const int i = wbase + 128 * r + 4 * lane;
    int o[4];
    o[0] = off + pre[r];
    o[1] = o[0] + v[r][0];
    o[2] = o[1] + v[r][1];
    o[3] = o[2] + v[r][2];
    if (vec) {
      *reinterpret_cast<int4 *>(out + i) =
          over ? make_int4(0, 0, 0, 0) : make_int4(o[0], o[1], o[2], o[3]);
      if (over) // every count and offset dropped
        *reinterpret_cast<int4 *>(in + i) = make_int4(0, 0, 0, 0);
    } else {
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (i + j < n) {
          out[i + j] = over ? 0 : o[j];
          if (over) in[i + j] = 0;
        }
    }
  }
}

hg_status launch_small_scan(int32_t *in, int64_t n, int32_t *out, const ScanLimit &lim,
                            cudaStream_t s) {
  HG_LAUNCH_PDL(k_small_scan, 1, SMALL_THREADS, 0, s, in, n, out, lim);
  HG_CHECK_LAUNCH();
  return HG_OK;
}

} // namespace

int64_t small_scan_max() { return SMALL_N; }

hg_status exclusive_scan_i32_limited(int32_t *in, int32_t *out, int64_t n, const ScanLimit &lim,
                                     cudaStream_t s) {
  if (n <= 0 || n > small_scan_max())
    return fail(HG_ERR_INVALID_ARGUMENT, "limited scan: size out of range");
  return launch_small_scan(in, n, out, lim, s);
}

// out[i] = sum(in[0..i)); in and out may not alias. tmp must hold
// scan_tmp_size(n) ints.
hg_status exclusive_scan_i32(const int32_t *in, int32_t *out, int64_t n,
                             int32_t *tmp, cudaStream_t s) {
  if (n <= 0) return HG_OK;
  if (n <= SCAN_TILE) {
    HG_LAUNCH_PDL(k_tile_scan, 1, SCAN_THREADS, 0, s, in, n, nullptr, out);
    HG_CHECK_LAUNCH();
    return HG_OK;
  }
  if (n <= small_scan_max()) // (writes to its input only when a limit is exceeded)
    return launch_small_scan(const_cast<int32_t *>(in), n, out, ScanLimit{}, s);
  const int64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  int32_t *sums = tmp;
  int32_t *sums_scanned = tmp + tiles;
  HG_LAUNCH_PDL(k_tile_sums, (int)tiles, SCAN_THREADS, 0, s, in, n, sums);
  HG_CHECK_LAUNCH();
  if (tiles <= FUSED_TILES) { // two launches in place of three
    HG_LAUNCH_PDL(k_tile_scan_summed, (int)tiles, SCAN_THREADS, 0, s, in, n, sums, out);
    HG_CHECK_LAUNCH();
    return HG_OK;
  }
  hg_status st = exclusive_scan_i32(sums, sums_scanned, tiles, tmp + 2 * tiles, s);
  if (st != HG_OK) return st;
  HG_LAUNCH_PDL(k_tile_scan, (int)tiles, SCAN_THREADS, 0, s, in, n, sums_scanned, out);
  HG_CHECK_LAUNCH();
  return HG_OK;
}

} // namespace hg
