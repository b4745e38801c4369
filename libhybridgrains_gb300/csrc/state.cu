// Checkpoint/resume: the device state of an MPM, DEM or hybrid object as one
// host blob in this library's own versioned format.
//
// The reference snapshots host arrays (mpmgrains2d_cli.cpp:154-247 through
// SimulationState::serialize, SimulationState.cpp:119-129) and its hybrid and
// penalty-map serialization exit (HybridIntegratorState.cpp:67-85,
// PenaltyImpactFrictionMap.cpp:1155-1158). Here an object's state lives on
// the device in layouts of its own (sorted FP32 particle records with FP64
// positions in grid units, the next step's P2G accumulators, the DEM contact
// history), so the blob carries those buffers as they are: an object loaded
// from it continues as the saved one would, step for step.
//
// Layout: a header (magic "HGSTATE", version, kind, 16 int64 fields) and
// segments, each a (tag, byte count) pair followed by the bytes, padded to
// 8 bytes. Loading checks the kind, the grid or capacity and every segment's
// size before it copies anything.
#include "hg_internal.cuh"

#include <cstring>
#include <vector>

namespace hg {

namespace {

constexpr char MAGIC[8] = {'H', 'G', 'S', 'T', 'A', 'T', 'E', '\0'};
constexpr uint32_t VERSION = 1;
enum : uint32_t { KIND_MPM = 0, KIND_DEM = 1, KIND_HYBRID = 2 };

struct Header {
  char magic[8];
  uint32_t version;
  uint32_t kind;
  int64_t meta[16];
  uint32_t nseg;
  uint32_t pad;
};

struct SegHeader {
  uint32_t tag;
  uint32_t pad;
  uint64_t bytes;
};

struct Seg {
  uint32_t tag;
  void *dev;   // device address (save: source, load: destination)
  uint64_t bytes;
};

int64_t pad8(uint64_t b) { return (int64_t)((b + 7) & ~(uint64_t)7); }

int64_t blob_bytes(const std::vector<Seg> &segs) {
  int64_t t = sizeof(Header);
  for (const Seg &s : segs) t += sizeof(SegHeader) + pad8(s.bytes);
  return t;
}

template <class T> Seg seg(uint32_t tag, const DevBuf<T> &b, int64_t count) {
  return Seg{tag, (void *)b.p, (uint64_t)count * sizeof(T)};
}
template <class T> Seg whole(uint32_t tag, const DevBuf<T> &b) {
  return Seg{tag, (void *)b.p, (uint64_t)b.n * sizeof(T)};
}

hg_status write_blob(cudaStream_t s, uint32_t kind, const int64_t meta[16],
                     const std::vector<Seg> &segs, void *dst, int64_t bytes) {
  if (bytes < blob_bytes(segs)) return fail(HG_ERR_CAPACITY, "state buffer too small");
  unsigned char *o = static_cast<unsigned char *>(dst);
  Header h{};
  std::memcpy(h.magic, MAGIC, 8);
  h.version = VERSION;
  h.kind = kind;
  for (int k = 0; k < 16; ++k) h.meta[k] = meta[k];
  h.nseg = (uint32_t)segs.size();
  std::memcpy(o, &h, sizeof h);
  o += sizeof h;
  for (const Seg &sg : segs) {
    SegHeader sh{sg.tag, 0, sg.bytes};
    std::memcpy(o, &sh, sizeof sh);
    o += sizeof sh;
    if (sg.bytes) HG_CUDA_TRY(cudaMemcpyAsync(o, sg.dev, sg.bytes, cudaMemcpyDeviceToHost, s));
    const int64_t p = pad8(sg.bytes);
    if (p > (int64_t)sg.bytes) std::memset(o + sg.bytes, 0, p - sg.bytes);
    o += p;
  }
  HG_CUDA_TRY(cudaStreamSynchronize(s));
  return HG_OK;
}

// Parses a blob of the given kind: header fields and the host address of
// each segment, checked against the expected tags and sizes.
hg_status read_header(const void *src, int64_t bytes, uint32_t kind, Header *h) {
  if (bytes < (int64_t)sizeof(Header)) return fail(HG_ERR_INVALID_ARGUMENT, "state blob too short");
  std::memcpy(h, src, sizeof *h);
  if (std::memcmp(h->magic, MAGIC, 8) != 0) return fail(HG_ERR_INVALID_ARGUMENT, "not a state blob");
  if (h->version != VERSION) return fail(HG_ERR_UNSUPPORTED, "state blob of another version");
  if (h->kind != kind) return fail(HG_ERR_INVALID_ARGUMENT, "state blob of another object kind");
  return HG_OK;
}

hg_status read_segments(cudaStream_t s, const void *src, int64_t bytes, const Header &h,
                        const std::vector<Seg> &expect) {
  if (h.nseg != expect.size()) return fail(HG_ERR_INVALID_ARGUMENT, "state blob segment count");
  const unsigned char *base = static_cast<const unsigned char *>(src);
  // check everything first, then copy
  std::vector<const unsigned char *> at(expect.size());
  int64_t o = sizeof(Header);
  for (size_t k = 0; k < expect.size(); ++k) {
    if (o + (int64_t)sizeof(SegHeader) > bytes) return fail(HG_ERR_INVALID_ARGUMENT, "state blob truncated");
    SegHeader sh;
    std::memcpy(&sh, base + o, sizeof sh);
    o += sizeof sh;
    if (sh.tag != expect[k].tag || sh.bytes != expect[k].bytes)
      return fail(HG_ERR_INVALID_ARGUMENT, "state blob does not match the object");
    if (o + pad8(sh.bytes) > bytes) return fail(HG_ERR_INVALID_ARGUMENT, "state blob truncated");
    at[k] = base + o;
    o += pad8(sh.bytes);
  }
  for (size_t k = 0; k < expect.size(); ++k)
    if (expect[k].bytes)
      HG_CUDA_TRY(cudaMemcpyAsync(expect[k].dev, at[k], expect[k].bytes, cudaMemcpyHostToDevice, s));
  HG_CUDA_TRY(cudaStreamSynchronize(s));
  return HG_OK;
}

// ---- MPM ----------------------------------------------------------------------

void mpm_meta(const hg_mpm *m, int64_t meta[16]) {
  for (int k = 0; k < 16; ++k) meta[k] = 0;
  meta[0] = m->p.precision;
  meta[1] = m->p.nx;
  meta[2] = m->p.ny;
  meta[3] = m->p.basis;
  meta[4] = m->n;
  meta[5] = m->primed ? 1 : 0;
  meta[6] = m->steps_since_rebin;
  meta[7] = m->rebins;
  int32_t hb;
  std::memcpy(&hb, &m->hl_cells, sizeof hb);
  meta[8] = hb; // uGIMP half-width of the first uploaded point in cells (MIXED)
}

// Segments of the live state; buf selects the particle buffer of the pair.
std::vector<Seg> mpm_segments(hg_mpm *m, int64_t n, int buf) {
  std::vector<Seg> v;
  if (m->p.precision == HG_PRECISION_MIXED) {
    v.push_back(seg(1, m->mu_[buf], n));
    v.push_back(seg(2, m->mv_[buf], n));
    v.push_back(seg(3, m->mmv_[buf], n));
    v.push_back(seg(4, m->mstrain_[buf], n));
    v.push_back(seg(5, m->mflags_[buf], n));
    v.push_back(seg(6, m->mid_[buf], n));
    v.push_back(whole(7, m->acc4));
    v.push_back(whole(8, m->accm));
    v.push_back(whole(9, m->va));
    v.push_back(whole(10, m->gm));
    v.push_back(whole(11, m->offsets));
    v.push_back(whole(12, m->active_bins));
    v.push_back(whole(13, m->active_tiles));
    v.push_back(whole(14, m->nactive));
    v.push_back(whole(15, m->outside));
    if (m->p.basis == HG_BASIS_UGIMP) v.push_back(seg(16, m->mhl_[buf], n));
  } else {
    v.push_back(seg(1, m->q, 2 * n));
    v.push_back(seg(2, m->v, 2 * n));
    v.push_back(seg(3, m->m, n));
    v.push_back(seg(4, m->vol, n));
    v.push_back(seg(5, m->hl, n));
    v.push_back(seg(6, m->be, 4 * n));
    v.push_back(seg(7, m->J, n));
    v.push_back(seg(8, m->jh, n));
    v.push_back(seg(9, m->kin, n));
    v.push_back(whole(10, m->g_mass));
    v.push_back(whole(11, m->g_mom));
    v.push_back(whole(12, m->g_mom_new));
    v.push_back(whole(13, m->g_force));
    v.push_back(whole(14, m->g_vel));
    v.push_back(whole(15, m->g_acc));
    v.push_back(whole(16, m->g_cforce));
    v.push_back(whole(17, m->g_homog));
    v.push_back(whole(18, m->g_hyb));
  }
  v.push_back(whole(31, m->status));
  return v;
}

// ---- DEM -------------------------------------------------------------------------

hg_status dem_live_count(hg_dem *d, int32_t *count) {
  *count = 0;
  if (!d->history_valid) return HG_OK;
  HG_CUDA_TRY(cudaMemcpyAsync(count, d->c_count.p + d->cc, sizeof(int32_t), cudaMemcpyDeviceToHost,
                              dem_stream(d)));
  HG_CUDA_TRY(cudaStreamSynchronize(dem_stream(d)));
  *count = (int32_t)std::min<int64_t>(*count, d->ccap);
  return HG_OK;
}

std::vector<Seg> dem_segments(hg_dem *d, int64_t n, int64_t contacts, int buf) {
  std::vector<Seg> v;
  v.push_back(seg(1, d->q, 3 * n));
  v.push_back(seg(2, d->v, 3 * n));
  v.push_back(seg(3, d->r, n));
  v.push_back(seg(4, d->m0, n));
  v.push_back(seg(5, d->I0, n));
  v.push_back(seg(6, d->w, n));
  v.push_back(seg(7, d->fixed, n));
  v.push_back(seg(8, d->ckey[buf], contacts));
  v.push_back(seg(9, d->crec[buf], contacts * HG_DEM_RECORD_WIDTH));
  v.push_back(whole(31, d->status));
  return v;
}

} // namespace

hg_status mpm_state_bytes(hg_mpm *m, int64_t *bytes) {
  *bytes = blob_bytes(mpm_segments(m, m->n, m->cur));
  return HG_OK;
}

hg_status mpm_state_save(hg_mpm *m, void *dst, int64_t bytes) {
  int64_t meta[16];
  mpm_meta(m, meta);
  return write_blob(m->ctx->stream, KIND_MPM, meta, mpm_segments(m, m->n, m->cur), dst, bytes);
}

hg_status mpm_state_load(hg_mpm *m, const void *src, int64_t bytes) {
  Header h;
  hg_status st = read_header(src, bytes, KIND_MPM, &h);
  if (st != HG_OK) return st;
  if (h.meta[0] != m->p.precision || h.meta[1] != m->p.nx || h.meta[2] != m->p.ny ||
      h.meta[3] != m->p.basis)
    return fail(HG_ERR_INVALID_ARGUMENT, "state blob of another precision, grid or basis");
  const int64_t n = h.meta[4];
  if (n < 0 || n > m->cap) return fail(HG_ERR_CAPACITY, "state blob holds more points than the capacity");
  // the live particle buffer becomes the first of the pair
  if ((st = read_segments(m->ctx->stream, src, bytes, h, mpm_segments(m, n, 0)))) return st;
  m->n = n;
  m->cur = 0;
  m->order_valid = false; // the blob keeps no order tables
  m->primed = h.meta[5] != 0;
  m->steps_since_rebin = h.meta[6];
  m->rebins = h.meta[7];
  const int32_t hb = (int32_t)h.meta[8];
  std::memcpy(&m->hl_cells, &hb, sizeof hb);
  m->outside_pending = false;
  return HG_OK;
}

hg_status dem_state_bytes(hg_dem *d, int64_t *bytes) {
  int32_t c = 0;
  hg_status st = dem_live_count(d, &c);
  if (st != HG_OK) return st;
  *bytes = blob_bytes(dem_segments(d, d->n, c, d->cc));
  return HG_OK;
}

hg_status dem_state_save(hg_dem *d, void *dst, int64_t bytes) {
  int32_t c = 0;
  hg_status st = dem_live_count(d, &c);
  if (st != HG_OK) return st;
  int64_t meta[16] = {0};
  meta[0] = d->n;
  meta[1] = c;
  meta[2] = d->history_valid ? 1 : 0;
  std::memcpy(&meta[3], &d->cell_h, sizeof(double));
  meta[4] = d->ncontacts_host;
  return write_blob(dem_stream(d), KIND_DEM, meta, dem_segments(d, d->n, c, d->cc), dst, bytes);
}

hg_status dem_state_load(hg_dem *d, const void *src, int64_t bytes) {
  Header h;
  hg_status st = read_header(src, bytes, KIND_DEM, &h);
  if (st != HG_OK) return st;
  const int64_t n = h.meta[0], c = h.meta[1];
  if (n < 0 || n > d->cap) return fail(HG_ERR_CAPACITY, "state blob holds more bodies than the capacity");
  if (c < 0 || c > d->ccap) return fail(HG_ERR_CAPACITY, "state blob holds more contacts than the capacity");
  // the live contact history becomes buffer 0
  if ((st = read_segments(dem_stream(d), src, bytes, h, dem_segments(d, n, c, 0)))) return st;
  const int32_t c32 = (int32_t)c;
  HG_CUDA_TRY(cudaMemcpyAsync(d->c_count.p, &c32, sizeof(int32_t), cudaMemcpyHostToDevice,
                              dem_stream(d)));
  HG_CUDA_TRY(cudaStreamSynchronize(dem_stream(d)));
  d->n = n;
  d->cc = 0;
  d->history_valid = h.meta[2] != 0;
  std::memcpy(&d->cell_h, &h.meta[3], sizeof(double));
  d->ncontacts_host = h.meta[4];
  d->inv_valid = false;
  return HG_OK;
}

hg_status hybrid_state_bytes(hg_hybrid *hy, int64_t *bytes) {
  *bytes = blob_bytes({whole(1, hy->hstress), whole(2, hy->hvel)});
  return HG_OK;
}

hg_status hybrid_state_save(hg_hybrid *hy, void *dst, int64_t bytes) {
  int64_t meta[16] = {0};
  return write_blob(hy->ctx->stream, KIND_HYBRID, meta, {whole(1, hy->hstress), whole(2, hy->hvel)},
                    dst, bytes);
}

hg_status hybrid_state_load(hg_hybrid *hy, const void *src, int64_t bytes) {
  Header h;
  hg_status st = read_header(src, bytes, KIND_HYBRID, &h);
  if (st != HG_OK) return st;
  return read_segments(hy->ctx->stream, src, bytes, h, {whole(1, hy->hstress), whole(2, hy->hvel)});
}

} // namespace hg
