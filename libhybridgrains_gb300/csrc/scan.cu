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

__global__ void k_tile_sums(const int32_t *__restrict__ in, int64_t n,
                            int32_t *__restrict__ sums) {
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

} // namespace

int64_t scan_tmp_size(int64_t n) {
  int64_t total = 0;
  while (n > SCAN_TILE) {
    const int64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    total += 2 * tiles;
    n = tiles;
  }
  return total + 2;
}

// out[i] = sum(in[0..i)); in and out may not alias. tmp must hold
// scan_tmp_size(n) ints.
hg_status exclusive_scan_i32(const int32_t *in, int32_t *out, int64_t n,
                             int32_t *tmp, cudaStream_t s) {
  if (n <= 0) return HG_OK;
  if (n <= SCAN_TILE) {
    HG_LAUNCH(k_tile_scan, 1, SCAN_THREADS, 0, s, in, n, nullptr, out);
    HG_CHECK_LAUNCH();
    return HG_OK;
  }
  const int64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  int32_t *sums = tmp;
  int32_t *sums_scanned = tmp + tiles;
  HG_LAUNCH(k_tile_sums, (int)tiles, SCAN_THREADS, 0, s, in, n, sums);
  HG_CHECK_LAUNCH();
  hg_status st = exclusive_scan_i32(sums, sums_scanned, tiles, tmp + 2 * tiles, s);
  if (st != HG_OK) return st;
  HG_LAUNCH(k_tile_scan, (int)tiles, SCAN_THREADS, 0, s, in, n, sums_scanned, out);
  HG_CHECK_LAUNCH();
  return HG_OK;
}

} // namespace hg
