// ela3d_engine.cu -- host engine: device layout, C-PML slab sizing, tensor
// maps, work schedule and the time-step loop.
#include "ela3d_engine.h"

#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <numeric>

namespace ela3d {

static thread_local std::string g_last_error;
void set_last_error(const std::string &m) { g_last_error = m; }
const char *last_error() { return g_last_error.c_str(); }

ela3d_status status_from_cuda(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return ELA3D_OK;
  set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
  if (e == cudaErrorMemoryAllocation) return ELA3D_ERR_OOM;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return ELA3D_ERR_NO_DEVICE;
  return ELA3D_ERR_CUDA;
}

#define CK(call)                                              \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return status_from_cuda(e_, #call); \
  } while (0)

#define BAD(msg)                  \
  do {                            \
    set_last_error(msg);          \
    return ELA3D_ERR_INVALID_ARG; \
  } while (0)

ela3d_status validate_params(const ela3d_params &p) {
  if (p.nx < 3 || p.ny < 3 || p.nz < 3) BAD("grid must be at least 3 cells on each axis");
  if ((long long)p.nx * p.ny * p.nz > (1ll << 34)) BAD("grid too large");
  if (!(p.dx > 0 && p.dy > 0 && p.dz > 0 && p.dt > 0)) BAD("spacing and time step must be positive");
  if (p.nstep < 0 || p.sampgat < 1) BAD("nstep must be >= 0 and sampgat >= 1");
  if (p.npml < 0) BAD("npml must be >= 0");
  if (p.npml > 0 && !(p.rcoef > 0 && p.rcoef < 1)) BAD("rcoef must lie in (0, 1)");
  if (p.precision != ELA3D_FP32 && p.precision != ELA3D_FP64) BAD("precision must be FP32 or FP64");
  if (p.pml_mode != ELA3D_PML_COMPAT && p.pml_mode != ELA3D_PML_CLEAN) BAD("unknown pml_mode");
  if (p.stf < 0 || p.stf > 2) BAD("unknown stf");
  if (p.src_kind != ELA3D_SRC_FORCE && p.src_kind != ELA3D_SRC_EXPLOSIVE) BAD("unknown src_kind");
  if (p.src_i < 0 || p.src_i >= p.nx || p.src_j < 0 || p.src_j >= p.ny || p.src_k < 0 || p.src_k >= p.nz)
    BAD("source outside the grid");
  if (p.nrec < 0 || (p.nrec > 0 && !p.rec)) BAD("receiver list missing");
  for (int r = 0; r < p.nrec; ++r) {
    const int32_t *q = p.rec + 3 * r;
    if (q[0] < 0 || q[0] >= p.nx || q[1] < 0 || q[1] >= p.ny || q[2] < 0 || q[2] >= p.nz)
      BAD("receiver " + std::to_string(r) + " outside the grid");
  }
  return ELA3D_OK;
}

void slab_extent(const double *a_full, const double *a_half, int n, int *lo, int *hi) {
  int l = 0, h = n;
  for (int i = 0; i < n; ++i) {
    const bool act = a_full[i] != 0.0 || a_half[i] != 0.0;
    if (!act) continue;
    if (2 * i < n) l = std::max(l, i + 1);
    else h = std::min(h, i);
  }
  bool clean = l <= h;
  for (int i = l; clean && i < h; ++i)
    if (a_full[i] != 0.0 || a_half[i] != 0.0) clean = false;
  if (!clean || l >= h) { l = n; h = n; }
  *lo = l;
  *hi = h;
}

void build_schedule(const std::vector<ShotShape> &shots, int tx, int ty, int kind, int chunk, int max_blocks,
                    std::vector<Item> *items, std::vector<int2> *ranges) {
  items->clear();
  ranges->clear();
  auto sid = [&](int s) { return shots[s].id >= 0 ? shots[s].id : s; };
  struct Col { int shot, tile, nz; };
  std::vector<Col> cols;
  long long units = 0;
  for (int s = 0; s < (int)shots.size(); ++s) {
    const int ntiles = ((shots[s].nx + tx - 1) / tx) * ((shots[s].ny + ty - 1) / ty);
    for (int t = 0; t < ntiles; ++t) cols.push_back({sid(s), t, shots[s].nz});
    units += (long long)ntiles * shots[s].nz;
  }
  if (units == 0 || max_blocks < 1) return;
  if (kind == 0) {
    const long long G = std::min<long long>(max_blocks, units);
    size_t ci = 0;
    int kk = 0;  // next plane of cols[ci]
    for (long long b = 0; b < G; ++b) {
      long long take = (b + 1) * units / G - b * units / G;
      const int first = (int)items->size();
      while (take > 0) {
        const Col &c = cols[ci];
        const int run = (int)std::min<long long>(take, c.nz - kk);
        items->push_back({c.shot, c.tile, kk, kk + run});
        take -= run;
        kk += run;
        if (kk == c.nz) { ++ci; kk = 0; }
      }
      ranges->push_back(make_int2(first, (int)items->size()));
    }
    return;
  }
  // kinds 1 and 2: z-chunks dealt round-robin.  Kind 1 orders them
  // (shot, chunk, tile); kind 2 orders (chunk, tile, shot), so blocks running
  // together hold the same tile of different shots (a shared model tile is
  // then read from L2 by all but the first).
  if (chunk < 1) chunk = 1;
  std::vector<Item> all;
  std::vector<double> cost;   // estimated work of each item
  for (int s = 0; s < (int)shots.size(); ++s) {
    const ShotShape &sh = shots[s];
    const int txs = (sh.nx + tx - 1) / tx, ntiles = txs * ((sh.ny + ty - 1) / ty);
    // share of [a, b) inside a slab pair [0, l) + [r, n) (no slabs: l = r = -1)
    auto slab = [](int a, int b, int l, int r) {
      if (l < 0 || b <= a) return 0.0;
      const int in = std::max(0, std::min(b, l) - a) + std::max(0, b - std::max(a, r));
      return (double)in / (double)(b - a);
    };
    for (int k0 = 0; k0 < sh.nz; k0 += chunk)
      for (int t = 0; t < ntiles; ++t) {
        const int k1 = std::min(k0 + chunk, sh.nz);
        all.push_back({sid(s), t, k0, k1});
        const int x0 = (t % txs) * tx, x1 = std::min(x0 + tx, sh.nx);
        const int y0 = (t / txs) * ty, y1 = std::min(y0 + ty, sh.ny);
        // cells, weighted by the memory-variable traffic of the C-PML
        // directions they lie in (48 of 124 bytes per direction)
        const double pml = slab(x0, x1, sh.xl, sh.xr) + slab(y0, y1, sh.yl, sh.yr) + slab(k0, k1, sh.zl, sh.zr);
        cost.push_back((double)(x1 - x0) * (y1 - y0) * (k1 - k0) * (1.0 + 0.39 * pml));
      }
  }
  if (kind == 2) {
    std::vector<int> order(all.size());
    for (size_t q = 0; q < order.size(); ++q) order[q] = (int)q;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
      if (all[a].k0 != all[b].k0) return all[a].k0 < all[b].k0;
      return all[a].tile < all[b].tile;
    });
    std::vector<Item> a2;
    std::vector<double> c2;
    for (int q : order) { a2.push_back(all[q]); c2.push_back(cost[q]); }
    all.swap(a2);
    cost.swap(c2);
  }
  // Round j hands items [jG, jG + G) to the G blocks, so blocks running
  // together hold neighbouring items.  Block b takes slot b of every round,
  // or slot (b + j) mod G when that rotation evens out the estimated work
  // clearly better (when the tiles per round divide G, the plain deal gives
  // a block the same tile every round, and one block all of a PML tile's
  // work).
  const int G = (int)std::min<long long>(max_blocks, (long long)all.size());
  const long long n = (long long)all.size(), rounds = (n + G - 1) / G;
  auto slot = [&](int b, long long j, bool skew) { return j * G + (skew ? (b + j) % G : b); };
  auto max_load = [&](bool skew) {
    double m = 0.0;
    for (int b = 0; b < G; ++b) {
      double l = 0.0;
      for (long long j = 0; j < rounds; ++j) {
        const long long q = slot(b, j, skew);
        if (q < n) l += cost[q];
      }
      m = std::max(m, l);
    }
    return m;
  };
  const bool skew = max_load(true) < 0.95 * max_load(false);
  for (int b = 0; b < G; ++b) {
    const int first = (int)items->size();
    for (long long j = 0; j < rounds; ++j) {
      const long long q = slot(b, j, skew);
      if (q < n) items->push_back(all[q]);
    }
    ranges->push_back(make_int2(first, (int)items->size()));
  }
}

bool build_flow_schedule(const std::vector<FlowShape> &shots, int tx, int ty, int chunk, int gap, bool overlap,
                         int nsteps, std::vector<FlowItem> *items, std::vector<int> *flag_off,
                         std::vector<int> *nchunks, int *nflags, std::string *why) {
  items->clear();
  flag_off->clear();
  nchunks->clear();
  *nflags = 0;
  if (chunk < 2 || gap < 1 || nsteps < 1 || nsteps > 255 || tx < 1 || ty < 1 || shots.size() >= (1u << 16)) {
    *why = "dataflow schedule: chunk >= 2, gap >= 1, 1 <= nsteps <= 255, fewer than 65536 shots";
    return false;
  }
  // Keys approximate list positions (two per stress item of one step in
  // natural order, leaving room for the velocity items between them): a
  // stress item of step 0 sits at its natural place, every other item `gap`
  // after the last item it waits for (a stress item of a later step also
  // no earlier than its natural place, plus the whole steps before it
  // unless steps may overlap).  The list is ordered by key, ties by (step,
  // kind, shot, chunk, tile): the items are generated in that tie order and
  // sorted stably by key (a counting sort when the keys are dense).
  struct Shape { int txs, tys, nt, J; long long step_base; std::vector<long long> ks, kv, kv_prev; };
  std::vector<Shape> sh(shots.size());
  size_t total = 0;
  for (size_t s = 0; s < shots.size(); ++s) {
    Shape &h = sh[s];
    h.txs = (shots[s].nx + tx - 1) / tx;
    h.tys = (shots[s].ny + ty - 1) / ty;
    h.nt = h.txs * h.tys;
    h.J = (shots[s].nz + chunk - 1) / chunk;
    if (h.J >= (1 << 14) || h.nt >= (1 << 25)) {
      *why = "dataflow schedule: too many z-chunks or tiles for one shot";
      return false;
    }
    h.step_base = 0;
    h.ks.assign((size_t)h.J * h.nt, 0);
    h.kv.assign((size_t)h.J * h.nt, 0);
    flag_off->push_back(*nflags);
    nchunks->push_back(h.J);
    *nflags += 2 * h.J * h.nt;
    total += (size_t)nsteps * 2 * h.J * h.nt;
  }
  // the items one item waits for (chunks c0/c1 of the other kind, on the
  // tile and its four neighbours): the largest key among them
  auto last_dep = [](const Shape &h, const std::vector<long long> &k, int c0, int c1, int x, int y) {
    long long m = -1;
    for (int c : {c0, c1}) {
      if (c < 0 || c >= h.J) continue;
      const long long *kc = k.data() + (size_t)c * h.nt;
      const int t = y * h.txs + x;
      m = std::max(m, kc[t]);
      if (x > 0) m = std::max(m, kc[t - 1]);
      if (x + 1 < h.txs) m = std::max(m, kc[t + 1]);
      if (y > 0) m = std::max(m, kc[t - h.txs]);
      if (y + 1 < h.tys) m = std::max(m, kc[t + h.txs]);
    }
    return m;
  };
  // keys in generation order (step, kind, shot, chunk, tile); the items
  // themselves follow from that order and are written out once sorted
  std::vector<long long> key;
  key.reserve(total);
  for (int r = 0; r < nsteps; ++r) {
    for (size_t s = 0; s < shots.size(); ++s) {   // stress items of step r
      Shape &h = sh[s];
      for (int j = 0; j < h.J; ++j) {
        for (int y = 0, t = 0; y < h.tys; ++y)
          for (int x = 0; x < h.txs; ++x, ++t) {
            long long k = 2ll * ((long long)j * h.nt + t) + h.step_base;
            if (r > 0) k = std::max(k, last_dep(h, h.kv_prev, j, j + 1, x, y) + gap);
            h.ks[(size_t)j * h.nt + t] = k;
            key.push_back(k);
          }
      }
    }
    for (size_t s = 0; s < shots.size(); ++s) {   // velocity items of step r
      Shape &h = sh[s];
      for (int j = 0; j < h.J; ++j) {
        for (int y = 0, t = 0; y < h.tys; ++y)
          for (int x = 0; x < h.txs; ++x, ++t) {
            const long long k = last_dep(h, h.ks, j - 1, j, x, y) + gap;
            h.kv[(size_t)j * h.nt + t] = k;
            key.push_back(k);
          }
      }
      h.kv_prev = h.kv;
      if (!overlap) h.step_base = *std::max_element(h.kv.begin(), h.kv.end()) + 1;
    }
  }
  // stable sort by key
  const size_t n = key.size();
  std::vector<unsigned> order(n);
  long long kmin = 0, kmax = -1;
  if (n) {
    kmin = *std::min_element(key.begin(), key.end());
    kmax = *std::max_element(key.begin(), key.end());
  }
  const unsigned long long range = n ? (unsigned long long)(kmax - kmin) + 1 : 0;
  if (n && range <= 16ull * n + 1024) {
    std::vector<unsigned> cnt(range + 1, 0);
    for (size_t q = 0; q < n; ++q) ++cnt[key[q] - kmin + 1];
    for (size_t v = 1; v <= range; ++v) cnt[v] += cnt[v - 1];
    for (size_t q = 0; q < n; ++q) order[cnt[key[q] - kmin]++] = (unsigned)q;
  } else {
    for (size_t q = 0; q < n; ++q) order[q] = (unsigned)q;
    std::stable_sort(order.begin(), order.end(), [&](unsigned a, unsigned b) { return key[a] < key[b]; });
  }
  // check: every item comes after every item it waits for.  Items are
  // visited in generation order, where an item's index follows from (step,
  // kind, shot, chunk, tile): step r, kind k, shot s start at
  // r * 2 * per_kind + k * per_kind + first[s]
  std::vector<unsigned> pos(n);
  for (size_t q = 0; q < n; ++q) pos[order[q]] = (unsigned)q;
  std::vector<size_t> first(shots.size() + 1, 0);
  for (size_t s = 0; s < shots.size(); ++s) first[s + 1] = first[s] + (size_t)sh[s].J * sh[s].nt;
  const size_t per_kind = first[shots.size()];
  size_t g = 0;
  for (int r = 0; r < nsteps; ++r)
    for (int kind = 0; kind < 2; ++kind)
      for (size_t s = 0; s < shots.size(); ++s) {
        const Shape &h = sh[s];
        const int rd = kind == 0 ? r - 1 : r;   // step of the items waited for
        const size_t dep0 = rd < 0 ? 0 : ((size_t)rd * 2 + (1 - kind)) * per_kind + first[s];
        for (int j = 0; j < h.J; ++j) {
          const int c0 = j, c1 = kind == 0 ? j + 1 : j - 1;
          for (int y = 0, t = 0; y < h.tys; ++y)
            for (int x = 0; x < h.txs; ++x, ++t, ++g) {
              if (rd < 0) continue;   // before the launch: done
              const unsigned me = pos[g];
              for (int c : {c0, c1}) {
                if (c < 0 || c >= h.J) continue;
                const size_t d = dep0 + (size_t)c * h.nt + t;
                bool ok = pos[d] < me;
                if (x > 0) ok = ok && pos[d - 1] < me;
                if (x + 1 < h.txs) ok = ok && pos[d + 1] < me;
                if (y > 0) ok = ok && pos[d - h.txs] < me;
                if (y + 1 < h.tys) ok = ok && pos[d + h.txs] < me;
                if (!ok) {
                  *why = "dataflow schedule: an item does not follow the items it waits for";
                  return false;
                }
              }
            }
        }
      }
  items->resize(n);
  for (size_t q = 0; q < n; ++q) {   // the item of generation index order[q]
    size_t g2 = order[q];
    const int r = (int)(g2 / (2 * per_kind));
    g2 -= (size_t)r * 2 * per_kind;
    const int kind = g2 >= per_kind ? 1 : 0;
    g2 -= (size_t)kind * per_kind;
    const size_t sidx = (size_t)(std::upper_bound(first.begin(), first.end(), g2) - first.begin()) - 1;
    g2 -= first[sidx];
    const Shape &h = sh[sidx];
    const int j = (int)(g2 / h.nt), t = (int)(g2 % h.nt), nz = shots[sidx].nz;
    const int k0 = kind == 0 ? j * chunk : std::max(j * chunk - 1, 0);
    const int k1 = kind == 0 ? std::min((j + 1) * chunk, nz) : (j == h.J - 1 ? nz : (j + 1) * chunk - 1);
    (*items)[q] = FlowItem{{shots[sidx].id, t, k0, k1}, kind, r, j, 0};
  }
  return true;
}

TuneChoice default_choice(int fp64, int nx, int ny, int nz, bool explosive) {
  int n = 0;
  const Variant *v = variants(&n);
  // first variant of the precision (the list is ordered best first for
  // large grids), z-chunks of 10 planes (more for wide grids, below) dealt
  // round-robin, both prefetches;
  // a grid too small to give every SM several chunks gets equal contiguous
  // shares instead (round-robin would leave some blocks with one chunk more)
  int i = 0;
  while (i < n && (v[i].fp64 != 0) != (fp64 != 0)) ++i;
  if (i == n) i = 0;
  TuneChoice c{i, 1, 10, 0, kPrefetchDefault};
  if (nx > 0 && ny > 0 && nz > 0) {
    // among the wide tiles of the same shape class (warps, stages), the one
    // whose width wastes least of a row (101 cells: 112 wide, 90% used,
    // rather than 128 wide, 79%)
    auto used = [&](int tx) { return (double)nx / (double)(((nx + tx - 1) / tx) * tx); };
    const int first = i;
    for (int j = 0; j < n; ++j)
      if (j != first && v[j].fp64 == v[first].fp64 && v[j].loads == LOAD_TMA && v[j].threads == v[first].threads &&
          v[j].ns == v[first].ns && v[j].tx >= 112 && v[j].tx * v[j].ty == v[first].tx * v[first].ty &&
          used(v[j].tx) > used(v[i].tx) + 0.02)
        i = j;
    c.variant = i;
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long tiles = (long long)((nx + v[i].tx - 1) / v[i].tx) * ((ny + v[i].ty - 1) / v[i].ty);
    // with more tiles per plane than blocks, the blocks running together no
    // longer hold neighbouring chunks of one tile column, so each chunk's
    // look-ahead and z-1 planes come from DRAM again: longer chunks keep
    // that share small (measured: 512^3 best at 16-32 planes, 1024^3 at
    // 64-128), as long as every block still gets several of them
    if (tiles > sms) {
      int ch = 16;
      while (ch < 128 && ch * sms < 16 * tiles) ch *= 2;
      while (ch > 10 && tiles * ((nz + ch - 1) / ch) < 8ll * sms) ch /= 2;
      c.chunk = std::max(10, ch);
    }
    const long long chunks = tiles * ((nz + c.chunk - 1) / c.chunk);
    if (chunks < 4ll * std::max(1, sms)) c.kind = 0;
    // a shot whose twelve arrays fit in L2 gains nothing from bringing its
    // y/z-slab memory variables into L2 ahead of use
    const double bytes = 12.0 * nx * ny * nz * (fp64 ? 8.0 : 4.0);
    if (bytes < 96.0 * (1 << 20)) c.prefetch = CTL_PF_X;
    // FP32 shots run faster in the dataflow kernel with overlapping steps:
    // no launch boundaries, no tail of a half-step, and for grids near the
    // L2 size the exchange between the half-steps through L2.  Its work
    // items (tile columns cut into z-chunks) number about 1.5 per block,
    // with at least three chunks per column while the columns alone are
    // fewer than that, whole columns beyond.  Measured (Gcell/s, dataflow
    // against the best two-kernel choice): 101^3 32.2 vs 26.4, 128^3 29.7
    // vs 22.5, 160^3 30.8 vs 25.9, 192^3 38.9 vs 34.1, 224^3 42.6 vs 40.8,
    // 256^3 45.6 vs 44.5, 288^3 42.0 vs 41.2, 384^3 46.1 vs 44.9, 448^3
    // 42.2 vs 41.8, 512^3 47.0 vs 45.4, 1024^3 47.6 vs 44.7; only 320^3 is
    // the other way, 42.8 vs 43.4.  An explosive source injects between the
    // half-steps, so it keeps the two kernels.
    if (!fp64 && !explosive && v[i].flow) {
      // (chunks of equal size: at 256^3 three 86-plane chunks per column ran
      // at 46.5 against 45.6 for four of 64 and 45.6 for 96 + 96 + 64)
      const long long want = 3ll * sms / 2;                              // work items per half-step
      const long long per_col = want <= tiles ? 1 : std::max(3ll, (2 * want + tiles) / (2 * tiles));
      {
        c.kind = kScheduleFlowOverlap;
        c.chunk = std::max(4, (int)((nz + per_col - 1) / per_col));
        c.lag = 0;
        // the memory-variable prefetch pays only once the arrays outgrow
        // the L2 (Gcell/s with none / x slab / x, y, z slabs: 101^3 32.9 /
        // 32.3 / 25.9, 128^3 34.2 / 34.7 / 28.4, 160^3 31.4 / 31.8 / 31.8,
        // 192^3 36.3 / 37.9 / 38.8, 256^3 41.0 / 44.8 / 45.4)
        c.prefetch = bytes < 64.0 * (1 << 20) ? 0 : bytes < 256.0 * (1 << 20) ? CTL_PF_X : kPrefetchDefault;
      }
    }
  }
  return c;
}

// ------------------------------------------------------------ TMA maps --
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

template <typename T>
static ela3d_status encode_map(CUtensorMap *m, const T *base, int nx, int ny, int nz, int px, int bw, int bh) {
  auto fn = encode_fn();
  if (!fn) {
    set_last_error("cuTensorMapEncodeTiled unavailable");
    return ELA3D_ERR_CUDA;
  }
  cuuint64_t gdim[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
  cuuint64_t gstr[2] = {(cuuint64_t)px * sizeof(T), (cuuint64_t)px * ny * sizeof(T)};
  cuuint32_t box[3] = {(cuuint32_t)bw, (cuuint32_t)bh, 1};
  cuuint32_t es[3] = {1, 1, 1};
  CUresult r = fn(m, sizeof(T) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3,
                  const_cast<T *>(base), gdim, gstr, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_last_error("cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return ELA3D_ERR_CUDA;
  }
  return ELA3D_OK;
}

// -------------------------------------------------------------- engine --
template <typename T>
struct Shot {
  ela3d_params p{};
  std::vector<int32_t> rec;
  int px = 0, nsamp = 0;
  int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  char *pool = nullptr;
  T *prof = nullptr;
  size_t pool_bytes = 0, prof_bytes = 0;
  int model_of = -1;   // shot that owns the model arrays (-1: self)
  ShotDesc<T> d{};
  ShotMaps maps{};
  double e_ref = -1.0; // energy monitor reference after the source ended
  struct Guard { size_t off, bytes; const char *after; };
  std::vector<Guard> guards;  // debug guard zones in the pool (empty unless enabled)
  uint64_t key = 0;    // stable identity while shots join and leave
};

template <typename T> struct Fp;
template <> struct Fp<float> {
  static cudaError_t model(const ModelSpec &m, int nx, int ny, int nz, int px, float *a, float *b, float *c,
                           cudaStream_t s) {
    return launch_model_f32(m, nx, ny, nz, px, a, b, c, s);
  }
  static cudaError_t profile(const AxisProfileArgs &a, float *o, cudaStream_t s) { return launch_profile_f32(a, o, s); }
  static cudaError_t stf(const StfArgs &a, float *o, cudaStream_t s) { return launch_stf_f32(a, o, s); }
  static cudaError_t pad(const float *src, float *dst, int nx, int ny, int nz, int px, cudaStream_t s) {
    return launch_pad_f32(src, dst, nx, ny, nz, px, s);
  }
  static cudaError_t explosive(const ShotDesc<float> *d, int n, int tick, const int *dt, cudaStream_t s) {
    return launch_explosive_f32(d, n, tick, dt, s);
  }
  static cudaError_t energy(const ShotDesc<float> *d, int nx, int ny, int nz, double *o, cudaStream_t s) {
    return launch_energy_f32(d, nx, ny, nz, o, s);
  }
};
template <> struct Fp<double> {
  static cudaError_t model(const ModelSpec &m, int nx, int ny, int nz, int px, double *a, double *b, double *c,
                           cudaStream_t s) {
    return launch_model_f64(m, nx, ny, nz, px, a, b, c, s);
  }
  static cudaError_t profile(const AxisProfileArgs &a, double *o, cudaStream_t s) { return launch_profile_f64(a, o, s); }
  static cudaError_t stf(const StfArgs &a, double *o, cudaStream_t s) { return launch_stf_f64(a, o, s); }
  static cudaError_t pad(const float *src, double *dst, int nx, int ny, int nz, int px, cudaStream_t s) {
    return launch_pad_f64(src, dst, nx, ny, nz, px, s);
  }
  static cudaError_t explosive(const ShotDesc<double> *d, int n, int tick, const int *dt, cudaStream_t s) {
    return launch_explosive_f64(d, n, tick, dt, s);
  }
  static cudaError_t energy(const ShotDesc<double> *d, int nx, int ny, int nz, double *o, cudaStream_t s) {
    return launch_energy_f64(d, nx, ny, nz, o, s);
  }
};

static size_t al256(size_t b) { return (b + 255) & ~size_t(255); }

template <typename T>
class Engine final : public EngineBase {
 public:
  Engine() = default;
  ~Engine() override { release(); }

  ela3d_status init() {
    CK(cudaGetDevice(&device_));
    CK(cudaDeviceGetAttribute(&num_sms_, cudaDevAttrMultiProcessorCount, device_));
    CK(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    // shots joining a running engine are prepared on their own stream, so
    // their uploads overlap the launches in flight
    CK(cudaStreamCreateWithFlags(&setup_, cudaStreamNonBlocking));
    CK(cudaMalloc(&d_err_, sizeof(unsigned)));
    CK(cudaMemset(d_err_, 0, sizeof(unsigned)));
    CK(cudaMalloc(&d_tick_, sizeof(int)));
    CK(cudaMemset(d_tick_, 0, sizeof(int)));
    if (const char *e = std::getenv("ELA3D_GRAPH_STEPS")) graph_steps_ = std::max(1, std::atoi(e));
    if (const char *e = std::getenv("ELA3D_FLOW_STEPS")) flow_max_steps_ = std::min(255, std::max(1, std::atoi(e)));
    if (const char *e = std::getenv("ELA3D_FLOW_PASSES")) flow_passes_ = std::max(1, std::atoi(e));
    // ELA3D_PSI_PREFETCH=<bits> overrides the tuned prefetch mode (experiments)
    if (const char *e = std::getenv("ELA3D_PSI_PREFETCH")) prefetch_env_ = std::atoi(e) & (CTL_PF_X | CTL_PF_YZ);
    // ELA3D_GUARD_ZONES=<bytes> (debug): guard zones around every pool array
    if (const char *e = std::getenv("ELA3D_GUARD_ZONES")) {
      const long long b = std::atoll(e);
      if (b > 0) guard_ = al256((size_t)std::min(b, 1ll << 20));
    }
    return ELA3D_OK;
  }

  int nshots() const override { return (int)shots_.size(); }
  int steps_done() const override { return tick_; }
  cudaStream_t stream() const override { return stream_; }

  ela3d_status add_shot(const ela3d_params &p, const float *cp, const float *cs, const float *rho,
                        int shared_model_of, const ModelSpec *spec = nullptr) override {
    ela3d_status st = validate_params(p);
    if (st != ELA3D_OK) return st;
    if ((p.precision == ELA3D_FP64) != (sizeof(T) == 8)) BAD("precision does not match the engine");
    if (shared_model_of >= (int)shots_.size()) BAD("shared model index out of range");
    if (shared_model_of >= 0) {
      const ela3d_params &q = shots_[shared_model_of]->p;
      if (q.nx != p.nx || q.ny != p.ny || q.nz != p.nz) BAD("shared model needs equal grids");
      while (shots_[shared_model_of]->model_of >= 0) shared_model_of = shots_[shared_model_of]->model_of;
    } else if (!spec && (!cp || !cs || !rho)) {
      BAD("model arrays missing");
    }
    if (spec && (spec->kind < 0 || spec->kind > MODEL_MATLAB_ANTICLINE ||
                 (spec->kind == MODEL_LAYERED_DOME && (spec->nlayers < 1 || spec->nlayers > kMaxLayers))))
      BAD("bad model spec");
    auto sh = std::make_unique<Shot<T>>();
    Shot<T> &s = *sh;
    // any failure below returns through CK/BAD: free what was allocated
    struct Undo {
      Engine *e;
      Shot<T> *s;
      float *stage = nullptr;
      bool keep = false;
      ~Undo() {
        if (stage) cudaFreeAsync(stage, e->setup_);
        if (!keep) e->release_shot(*s);
      }
    } undo{this, &s};
    s.p = p;
    s.rec.assign(p.rec, p.rec + 3 * (size_t)p.nrec);
    s.p.rec = s.rec.data();
    s.model_of = shared_model_of;
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    constexpr int kAlign = 128 / (int)sizeof(T);
    s.px = (nx + kAlign - 1) / kAlign * kAlign;
    s.nsamp = p.nstep / p.sampgat;
    const int px = s.px;

    // 1. C-PML profiles in FP64 on the device (then rounded to T)
    s.prof_bytes = sizeof(T) * 6 * (size_t)(px + ny + nz);
    CK(cudaMalloc(&s.prof, s.prof_bytes));
    const double PI = 3.141592653589793238462643;
    AxisProfileArgs a{};
    a.compat = p.pml_mode == ELA3D_PML_COMPAT;
    a.npml = p.npml;
    a.ny = ny;
    a.dy = p.dy;
    a.npower = p.npower;
    a.k_max = p.k_max;
    a.alpha_max = p.alpha_max < 0 ? PI * p.f0 : p.alpha_max;
    a.rcoef = p.rcoef > 0 ? p.rcoef : 1e-3;
    a.vpml = p.vpml;
    a.dt = p.dt;
    const int ns[3] = {nx, ny, nz}, strides[3] = {px, ny, nz};
    const double ds[3] = {p.dx, p.dy, p.dz};
    size_t off[3] = {0, 6 * (size_t)px, 6 * (size_t)(px + ny)};
    for (int ax = 0; ax < 3; ++ax) {
      a.axis = ax;
      a.n = ns[ax];
      a.stride = strides[ax];
      a.d = ds[ax];
      if (p.npml == 0) {  // no layer: identity profiles
        std::vector<T> id(6 * (size_t)strides[ax]);
        for (int q = 0; q < 6; ++q)
          for (int i = 0; i < strides[ax]; ++i) id[(size_t)q * strides[ax] + i] = (q == PR_A || q == PR_AH) ? T(0) : T(1);
        CK(cudaMemcpyAsync(s.prof + off[ax], id.data(), id.size() * sizeof(T), cudaMemcpyHostToDevice, setup_));
      } else {
        CK(Fp<T>::profile(a, s.prof + off[ax], setup_));
      }
    }
    std::vector<T> hprof(6 * (size_t)(px + ny + nz));
    CK(cudaMemcpyAsync(hprof.data(), s.prof, s.prof_bytes, cudaMemcpyDeviceToHost, setup_));
    CK(cudaStreamSynchronize(setup_));
    for (int ax = 0; ax < 3; ++ax) {
      std::vector<double> af(ns[ax]), ah(ns[ax]);
      for (int i = 0; i < ns[ax]; ++i) {
        af[i] = (double)hprof[off[ax] + (size_t)PR_A * strides[ax] + i];
        ah[i] = (double)hprof[off[ax] + (size_t)PR_AH * strides[ax] + i];
      }
      slab_extent(af.data(), ah.data(), ns[ax], &s.lo[ax], &s.hi[ax]);
    }
    // x slab boundaries on 16-byte groups
    constexpr int V = Vec<T>::N;
    int xl = (s.lo[0] + V - 1) / V * V, xr = s.hi[0] / V * V;
    if (xl >= xr || s.lo[0] >= nx) { xl = px; xr = px; }
    int yl = s.lo[1], yr = s.hi[1];
    int zl = s.lo[2], zr = s.hi[2];
    const int xw = xl + (px - xr), yw = yl + (ny - yr), zw = zl + (nz - zr);

    // 2. one pool for fields, model, psi slabs, source table, receivers, traces
    const size_t cells = (size_t)px * ny * nz;
    const size_t nrec = (size_t)p.nrec;
    size_t o = 0;
    // with guard zones on (debug), the pool starts with one and every array
    // is followed by one, covering its alignment slack too
    if (guard_) {
      s.guards.push_back({0, guard_, "the start of the pool"});
      o = guard_;
    }
    auto take = [&](size_t bytes, const char *name) {
      const size_t at = o;
      o += al256(bytes);
      if (guard_) {
        s.guards.push_back({at + bytes, o + guard_ - (at + bytes), name});
        o += guard_;
      }
      return at;
    };
    static const char *kFieldNames[9] = {"vx", "vy", "vz", "sxx", "syy", "szz", "sxy", "sxz", "syz"};
    size_t o_f[9];
    for (int c = 0; c < 9; ++c) o_f[c] = take(cells * sizeof(T), kFieldNames[c]);
    size_t o_m[3] = {0, 0, 0};
    static const char *kModelNames[3] = {"cp", "cs", "rho"};
    if (shared_model_of < 0)
      for (int c = 0; c < 3; ++c) o_m[c] = take(cells * sizeof(T), kModelNames[c]);
    const size_t psx = (size_t)nz * ny * xw, psy = (size_t)nz * yw * px, psz = (size_t)zw * ny * px;
    const size_t o_px = take(6 * psx * sizeof(T), "the x-slab memory variables");
    const size_t o_py = take(6 * psy * sizeof(T), "the y-slab memory variables");
    const size_t o_pz = take(6 * psz * sizeof(T), "the z-slab memory variables");
    const size_t o_stf = take(std::max(1, p.nstep) * sizeof(T), "the source time function");
    const size_t o_rp = take((size_t)(nz + 1) * sizeof(int), "the receiver plane index");
    const size_t o_rs = take(std::max<size_t>(1, nrec) * sizeof(int4), "the sorted receivers");
    const size_t o_seis = take(std::max<size_t>(1, nrec * 3 * s.nsamp) * sizeof(T), "the seismograms");
    const size_t o_trace = take(3 * (size_t)(p.nstep + 1) * sizeof(T), "the source trace");
    s.pool_bytes = o;
    CK(cudaMalloc(&s.pool, s.pool_bytes));
    CK(cudaMemsetAsync(s.pool, 0, s.pool_bytes, setup_));
    for (const auto &g : s.guards) CK(cudaMemsetAsync(s.pool + g.off, kGuardByte, g.bytes, setup_));

    ShotDesc<T> &d = s.d;
    d.nx = nx; d.ny = ny; d.nz = nz; d.px = px;
    d.tick0 = tick_;   // its first step is the engine's next step
    d.nstep = p.nstep;
    d.xl = xl; d.xr = xr; d.xw = xw;
    d.yl = yl; d.yr = yr; d.yw = yw;
    d.zl = zl; d.zr = zr; d.zw = zw;
    d.src_i = p.src_i; d.src_j = p.src_j; d.src_k = p.src_k; d.src_kind = p.src_kind;
    d.nrec = p.nrec; d.nsamp = s.nsamp; d.sampgat = p.sampgat;
    d.dt = (T)p.dt;
    d.idx = T(1) / (T)p.dx;
    d.idy = T(1) / (T)p.dy;
    d.idz = T(1) / (T)p.dz;
    for (int c = 0; c < 3; ++c) d.src_w[c] = (T)p.src_w[c];
    const double ang = p.angle_force * PI / 180.0;
    d.expl_w[0] = (T)std::sin(ang);
    d.expl_w[1] = (T)std::sin(ang);
    d.expl_w[2] = (T)std::cos(ang);
    for (int c = 0; c < 9; ++c) d.f[c] = reinterpret_cast<T *>(s.pool + o_f[c]);
    if (shared_model_of < 0) {
      d.cp = reinterpret_cast<T *>(s.pool + o_m[0]);
      d.cs = reinterpret_cast<T *>(s.pool + o_m[1]);
      d.rho = reinterpret_cast<T *>(s.pool + o_m[2]);
    } else {
      const ShotDesc<T> &od = shots_[shared_model_of]->d;
      d.cp = od.cp; d.cs = od.cs; d.rho = od.rho;
    }
    d.psi_x = reinterpret_cast<T *>(s.pool + o_px);
    d.psi_y = reinterpret_cast<T *>(s.pool + o_py);
    d.psi_z = reinterpret_cast<T *>(s.pool + o_pz);
    d.psx = (long long)psx; d.psy = (long long)psy; d.psz = (long long)psz;
    d.prof_x = s.prof;
    d.prof_y = s.prof + off[1];
    d.prof_z = s.prof + off[2];
    d.stf = reinterpret_cast<T *>(s.pool + o_stf);
    d.rec_plane = reinterpret_cast<int *>(s.pool + o_rp);
    d.rec_sorted = reinterpret_cast<int4 *>(s.pool + o_rs);
    d.seis = reinterpret_cast<T *>(s.pool + o_seis);
    d.src_trace = reinterpret_cast<T *>(s.pool + o_trace);

    // 3. model: generated on the device, or uploaded into the padded layout
    if (shared_model_of < 0 && spec) {
      T *dst[3] = {const_cast<T *>(d.cp), const_cast<T *>(d.cs), const_cast<T *>(d.rho)};
      CK(Fp<T>::model(*spec, nx, ny, nz, px, dst[0], dst[1], dst[2], setup_));
    } else if (shared_model_of < 0) {
      const float *src[3] = {cp, cs, rho};
      T *dst[3] = {const_cast<T *>(d.cp), const_cast<T *>(d.cs), const_cast<T *>(d.rho)};
      if (sizeof(T) == 4) {
        for (int c = 0; c < 3; ++c)
          CK(cudaMemcpy2DAsync(dst[c], px * sizeof(T), src[c], nx * sizeof(float), nx * sizeof(float),
                               (size_t)ny * nz, cudaMemcpyHostToDevice, setup_));
      } else {
        CK(cudaMallocAsync(reinterpret_cast<void **>(&undo.stage), (size_t)nx * ny * nz * sizeof(float), setup_));
        for (int c = 0; c < 3; ++c) {
          CK(cudaMemcpyAsync(undo.stage, src[c], (size_t)nx * ny * nz * sizeof(float), cudaMemcpyHostToDevice,
                             setup_));
          CK(Fp<T>::pad(undo.stage, dst[c], nx, ny, nz, px, setup_));
        }
        CK(cudaStreamSynchronize(setup_));
      }
    }
    // 4. source time function (FP64 on the device)
    if (p.nstep > 0) {
      StfArgs sa{p.nstep, p.stf, p.f0, p.t0, p.factor, p.dt};
      CK(Fp<T>::stf(sa, const_cast<T *>(d.stf), setup_));
    }
    // 5. receivers sorted by (k, j, i) with a per-plane index
    {
      std::vector<int4> rs(nrec);
      for (size_t r = 0; r < nrec; ++r) rs[r] = make_int4(s.rec[3 * r], s.rec[3 * r + 1], s.rec[3 * r + 2], (int)r);
      std::sort(rs.begin(), rs.end(), [](const int4 &u, const int4 &v) {
        if (u.z != v.z) return u.z < v.z;
        if (u.y != v.y) return u.y < v.y;
        if (u.x != v.x) return u.x < v.x;
        return u.w < v.w;
      });
      std::vector<int> rp(nz + 1, 0);
      for (size_t r = 0; r < nrec; ++r) rp[rs[r].z + 1]++;
      for (int k = 0; k < nz; ++k) rp[k + 1] += rp[k];
      CK(cudaMemcpyAsync(const_cast<int *>(d.rec_plane), rp.data(), rp.size() * sizeof(int), cudaMemcpyHostToDevice,
                         setup_));
      if (nrec)
        CK(cudaMemcpyAsync(const_cast<int4 *>(d.rec_sorted), rs.data(), nrec * sizeof(int4), cudaMemcpyHostToDevice,
                           setup_));
      CK(cudaStreamSynchronize(setup_));
    }
    if (p.src_kind == ELA3D_SRC_EXPLOSIVE) any_explosive_ = true;
    undo.keep = true;   // the shot is owned by the engine from here on
    shots_.push_back(std::move(sh));
    if (finalized_) {  // a shot joining a running engine
      Shot<T> &ns = *shots_.back();
      ns.key = next_key_++;
      // (its descriptor and tensor maps reach the device at the next
      // schedule rebuild, when no launch reads the tables any more)
      ela3d_status st2 = encode_shot_maps(ns);
      if (st2 != ELA3D_OK) {
        release_shot(ns);
        shots_.pop_back();
        return st2;
      }
      sched_valid_ = false;
      tables_dirty_ = true;
    } else {
      shots_.back()->key = next_key_++;
    }
    return ELA3D_OK;
  }

  uint64_t last_key() const override { return shots_.empty() ? 0 : shots_.back()->key; }

  // True once every launch enqueued so far has finished (or failed: the
  // caller's sync reports that).
  bool idle() const override { return cudaStreamQuery(stream_) != cudaErrorNotReady; }

  int index_of(uint64_t key) const {
    for (int q = 0; q < (int)shots_.size(); ++q)
      if (shots_[q]->key == key) return q;
    return -1;
  }

  ela3d_status remove_shot(uint64_t key) override {
    const int q = index_of(key);
    if (q < 0) {
      set_last_error("no such shot");
      return ELA3D_ERR_NOT_FOUND;
    }
    for (auto &sp : shots_)
      if (sp->model_of == q) BAD("another shot shares this shot's model");
    CK(cudaStreamSynchronize(stream_));
    release_shot(*shots_[q]);
    shots_.erase(shots_.begin() + q);
    for (auto &sp : shots_)
      if (sp->model_of > q) --sp->model_of;
    any_explosive_ = false;
    for (auto &sp : shots_) any_explosive_ |= sp->p.src_kind == ELA3D_SRC_EXPLOSIVE;
    sched_valid_ = false;
    if (shots_.empty()) {
      invalidate_graph();
      nblocks_ = 0;
      return ELA3D_OK;
    }
    return upload_tables();
  }

  // Device bytes add_shot would allocate for p (slabs estimated from npml,
  // an upper bound of the exact profile-derived extents).
  int64_t footprint(const ela3d_params &p) const override {
    constexpr int kAlign = 128 / (int)sizeof(T), V = Vec<T>::N;
    const int64_t px = (p.nx + kAlign - 1) / kAlign * kAlign;
    const int64_t cells = px * p.ny * p.nz;
    const int64_t w = 2 * (p.npml + 1);
    const int64_t xw = std::min<int64_t>(px, w + 2 * V), yw = std::min<int64_t>(p.ny, w), zw = std::min<int64_t>(p.nz, w);
    int64_t b = 12 * cells + 6 * ((int64_t)p.nz * p.ny * xw + (int64_t)p.nz * yw * px + zw * (int64_t)p.ny * px);
    b = b * (int64_t)sizeof(T) + (int64_t)p.nrec * 3 * (p.nstep / std::max(1, p.sampgat)) * (int64_t)sizeof(T) +
        (int64_t)p.nstep * (int64_t)sizeof(T) + 3 * (int64_t)(p.nstep + 1) * (int64_t)sizeof(T) +
        6 * (px + p.ny + p.nz) * (int64_t)sizeof(T) + 32 * 256;
    return b;
  }

  int shot_steps(uint64_t key) const override {
    const int q = index_of(key);
    if (q < 0) return -1;
    return std::min(tick_ - shots_[q]->d.tick0, shots_[q]->p.nstep);
  }

  // Samples [from, to) of every trace of a shot into host memory laid out
  // [nrec][3][to - from].
  ela3d_status read_samples(uint64_t key, int from, int to, float *out) override {
    const int q = index_of(key);
    if (q < 0) {
      set_last_error("no such shot");
      return ELA3D_ERR_NOT_FOUND;
    }
    const Shot<T> &s = *shots_[q];
    if (from < 0 || to > s.nsamp || from > to) BAD("sample range");
    const int n = to - from, rows = s.p.nrec * 3;
    if (n == 0 || rows == 0) return ELA3D_OK;
    std::vector<T> h((size_t)rows * n);
    CK(cudaMemcpy2DAsync(h.data(), n * sizeof(T), s.d.seis + from, s.nsamp * sizeof(T), n * sizeof(T), rows,
                         cudaMemcpyDeviceToHost, stream_));
    CK(cudaStreamSynchronize(stream_));
    for (size_t i = 0; i < h.size(); ++i) out[i] = (float)h[i];
    return ELA3D_OK;
  }

  void release_shot(Shot<T> &s) {
    if (s.pool) cudaFree(s.pool);
    if (s.prof) cudaFree(s.prof);
    s.pool = nullptr;
    s.prof = nullptr;
  }

  ela3d_status finalize(const TuneChoice *choice) override {
    if (finalized_) return ELA3D_OK;
    if (shots_.empty() && !choice) BAD("no shots");
    int nv = 0;
    const Variant *vs = variants(&nv);
    TuneChoice c = choice ? *choice
                          : default_choice(sizeof(T) == 8, shots_[0]->p.nx, shots_[0]->p.ny, shots_[0]->p.nz,
                                           shots_[0]->p.src_kind == ELA3D_SRC_EXPLOSIVE);
    if (c.variant < 0 || c.variant >= nv || vs[c.variant].fp64 != (sizeof(T) == 8)) BAD("bad kernel variant");
    var_ = &vs[c.variant];
    choice_ = c;
    prefetch_ = prefetch_env_ >= 0 ? prefetch_env_ : (c.prefetch & (CTL_PF_X | CTL_PF_YZ));
    for (auto &sp : shots_) {
      ela3d_status st = encode_shot_maps(*sp);
      if (st != ELA3D_OK) return st;
    }
    CK(cudaFuncSetAttribute(var_->stress, cudaFuncAttributeMaxDynamicSharedMemorySize, var_->stress_smem));
    CK(cudaFuncSetAttribute(var_->velocity, cudaFuncAttributeMaxDynamicSharedMemorySize, var_->vel_smem));
    if (var_->flow)
      CK(cudaFuncSetAttribute(var_->flow, cudaFuncAttributeMaxDynamicSharedMemorySize, var_->flow_smem));
    ela3d_status ost = occupancy(c);
    if (ost != ELA3D_OK) return ost;
    if (!shots_.empty()) {
      ela3d_status st = upload_tables();
      if (st != ELA3D_OK) return st;
    }
    finalized_ = true;
    return rebuild_schedule();
  }

  ela3d_status retune(const TuneChoice &c) override {
    if (!finalized_) return finalize(&c);
    int nv = 0;
    const Variant *vs = variants(&nv);
    if (c.variant < 0 || c.variant >= nv || var_ != &vs[c.variant]) BAD("retune keeps the kernel variant");
    choice_ = c;
    prefetch_ = prefetch_env_ >= 0 ? prefetch_env_ : (c.prefetch & (CTL_PF_X | CTL_PF_YZ));
    ela3d_status ost = occupancy(c);
    if (ost != ELA3D_OK) return ost;
    sched_valid_ = false;
    sched_key_.clear();
    return rebuild_schedule();
  }

  // Resident blocks per SM of the half-step kernels and of the dataflow
  // kernel (its launch is cooperative: every block must be resident).
  ela3d_status occupancy(const TuneChoice &c) {
    int occ_s = 0, occ_v = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_s, var_->stress, var_->threads, var_->stress_smem));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_v, var_->velocity, var_->threads, var_->vel_smem));
    per_sm_ = std::max(1, std::min(occ_s, occ_v));
    if (c.blocks_per_sm > 0) per_sm_ = std::min(per_sm_, c.blocks_per_sm);
    per_sm_flow_ = 0;
    if (var_->flow) {
      int occ_f = 0;
      CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_f, var_->flow, var_->threads, var_->flow_smem));
      per_sm_flow_ = occ_f;
      if (c.blocks_per_sm > 0) per_sm_flow_ = std::min(per_sm_flow_, c.blocks_per_sm);
    }
    return ELA3D_OK;
  }

  // The dataflow kernel runs when the schedule asks for it and it can: a
  // compiled dataflow kernel, resident blocks, and no explosive source (its
  // injection into the stresses runs as a kernel between the steps).
  bool flow_on() const {
    return (choice_.kind == kScheduleFlow || choice_.kind == kScheduleFlowOverlap) && var_ && var_->flow &&
           per_sm_flow_ > 0 && !any_explosive_;
  }

  // Retire shots once they reach their nstep (batches with uneven lengths):
  // their work items leave the schedule, their results stay readable.
  void set_retire(bool on) override { retire_ = on; }

  ela3d_status launch_step(int tick, const int *dtick) {
    int ctl = (inject_ > 0 ? CTL_WITHHOLD_LOADS : 0) | prefetch_;
    if (inject_ > 0) --inject_;
    void *args[] = {&d_desc_, &d_maps_, &d_items_, &d_ranges_, &tick, &dtick, &d_err_, &ctl};
    cudaEvent_t e0 = nullptr, e1 = nullptr, e2 = nullptr;
    const bool timed = timing_ && !capturing_;
    if (timed) {
      e0 = event(); e1 = event(); e2 = event();
      CK(cudaEventRecord(e0, stream_));
    }
    CK(cudaLaunchKernel(var_->stress, dim3(nblocks_), dim3(var_->threads), args, var_->stress_smem, stream_));
    if (timed) CK(cudaEventRecord(e1, stream_));
    CK(cudaLaunchKernel(var_->velocity, dim3(nblocks_), dim3(var_->threads), args, var_->vel_smem, stream_));
    if (timed) {
      CK(cudaEventRecord(e2, stream_));
      pending_.push_back({e0, e1, e2});
    }
    if (any_explosive_) CK(Fp<T>::explosive(d_desc_, (int)shots_.size(), tick, dtick, stream_));
    launches_ += 2 + (any_explosive_ ? 1 : 0);
    return ELA3D_OK;
  }

  // Steps until the active set changes (a shot starts or reaches nstep).
  int steps_to_boundary() const {
    int best = 1 << 30;
    for (auto &sp : shots_) {
      const int start = sp->d.tick0 + 1, end = sp->d.tick0 + sp->p.nstep;  // ticks of its first/last step
      if (tick_ + 1 < start) best = std::min(best, start - (tick_ + 1));
      else if (tick_ + 1 <= end) best = std::min(best, end - tick_);
    }
    return best;
  }

  ela3d_status enqueue(int nsteps) override {
    if (!finalized_) BAD("engine not finalized");
    if (nsteps < 0) BAD("nsteps must be >= 0");
    while (nsteps > 0) {
      int seg = nsteps;
      if (retire_) {
        ela3d_status st = rebuild_schedule();
        if (st != ELA3D_OK) return st;
        seg = std::min(seg, steps_to_boundary());
        if (nblocks_ == 0) {  // nothing active: time passes, no work
          tick_ += seg;
          nsteps -= seg;
          continue;
        }
      }
      nsteps -= seg;
      if (nblocks_ == 0) {
        tick_ += seg;
        continue;
      }
      if (flow_on() && flow_steps_ > 0) {
        while (seg > 0) {
          const int k = std::min(seg, flow_steps_ * flow_passes_);
          ela3d_status st = launch_flow(tick_ + 1, k);
          if (st != ELA3D_OK) return st;
          tick_ += k;
          seg -= k;
          steps_on_schedule_ += k;
        }
        continue;
      }
      // a composition's first graph_steps_ steps run as direct launches; the
      // graph is captured only once it has lasted that long (a serving
      // round whose composition never repeats pays for no capture)
      if (use_graphs_ && !timing_ && inject_ == 0 && !gexec_ && seg >= graph_steps_ &&
          steps_on_schedule_ < graph_steps_) {
        for (int d = std::min(seg, graph_steps_ - steps_on_schedule_); d > 0; --d, --seg) {
          ela3d_status st = launch_step(tick_ + 1, nullptr);
          if (st != ELA3D_OK) return st;
          ++tick_;
          ++steps_on_schedule_;
        }
      }
      const bool graphs = use_graphs_ && !timing_ && inject_ == 0 && seg >= graph_steps_;
      if (graphs) {
        ela3d_status st = ensure_graph();
        if (st != ELA3D_OK) return st;
        CK(launch_tick_set(d_tick_, tick_ + 1, stream_));
        while (seg >= graph_steps_) {
          CK(cudaGraphLaunch(gexec_, stream_));
          tick_ += graph_steps_;
          seg -= graph_steps_;
          launches_ += (int64_t)graph_steps_ * (2 + (any_explosive_ ? 1 : 0));
        }
      }
      for (; seg > 0; --seg) {
        ela3d_status st = launch_step(tick_ + 1, nullptr);
        if (st != ELA3D_OK) return st;
        ++tick_;
        ++steps_on_schedule_;
      }
    }
    return ELA3D_OK;
  }

  ela3d_status encode_shot_maps(Shot<T> &s) {
    const int TX = var_->tx, TY = var_->ty, H = var_->halo;
    ShotDesc<T> &d = s.d;
    const int nx = d.nx, ny = d.ny, nz = d.nz, px = d.px;
    CUtensorMap *m = s.maps.stress;
    ela3d_status st;
#define ENC(map, ptr, bw, bh) \
  if ((st = encode_map<T>(map, ptr, nx, ny, nz, px, bw, bh)) != ELA3D_OK) return st
    ENC(&m[0], d.f[0], TX + H, TY + 1);
    ENC(&m[1], d.f[1], TX + H, TY + 1);
    ENC(&m[2], d.f[2], TX + H, TY + 1);
    ENC(&m[3], d.cs, TX + H, TY + 1);
    ENC(&m[4], d.rho, TX + H, TY + 1);
    ENC(&m[5], d.cp, TX, TY);
    for (int q = 0; q < 6; ++q) ENC(&m[6 + q], d.f[3 + q], TX, TY);
    CUtensorMap *v = s.maps.vel;
    ENC(&v[0], d.f[3], TX + H, TY);      // sxx
    ENC(&v[1], d.f[4], TX, TY + 1);      // syy
    ENC(&v[2], d.f[5], TX, TY);          // szz
    ENC(&v[3], d.f[6], TX + H, TY + 1);  // sxy
    ENC(&v[4], d.f[7], TX + H, TY);      // sxz
    ENC(&v[5], d.f[8], TX, TY + 1);      // syz
    ENC(&v[6], d.rho, TX + H, TY + 1);   // rho
    for (int q = 0; q < 3; ++q) ENC(&v[7 + q], d.f[q], TX, TY);
#undef ENC
    return ELA3D_OK;
  }

  // Shot descriptors and tensor maps to the device (once per composition).
  ela3d_status upload_tables() {
    std::vector<ShotDesc<T>> descs;
    std::vector<ShotMaps> maps;
    for (auto &sp : shots_) { descs.push_back(sp->d); maps.push_back(sp->maps); }
    if (d_desc_) CK(cudaFree(d_desc_));
    if (d_maps_) CK(cudaFree(d_maps_));
    d_desc_ = nullptr;
    d_maps_ = nullptr;
    CK(cudaMalloc(&d_desc_, descs.size() * sizeof(ShotDesc<T>)));
    CK(cudaMalloc(&d_maps_, maps.size() * sizeof(ShotMaps)));
    CK(cudaMemcpyAsync(d_desc_, descs.data(), descs.size() * sizeof(ShotDesc<T>), cudaMemcpyHostToDevice, stream_));
    CK(cudaMemcpyAsync(d_maps_, maps.data(), maps.size() * sizeof(ShotMaps), cudaMemcpyHostToDevice, stream_));
    CK(cudaStreamSynchronize(stream_));
    return ELA3D_OK;
  }

  // Work items for the shots active at the next step (all shots unless
  // retirement is on).  Invalidates the cached graph when the split changes.
  ela3d_status rebuild_schedule() {
    std::vector<ShotShape> shapes;
    std::vector<int> key;
    for (int q = 0; q < (int)shots_.size(); ++q) {
      const ShotDesc<T> &d = shots_[q]->d;
      const int it = tick_ + 1 - d.tick0;
      if (retire_ && (it < 1 || it > shots_[q]->p.nstep)) continue;
      shapes.push_back({d.nx, d.ny, d.nz, q, d.xl, d.xr, d.yl, d.yr, d.zl, d.zr});
      key.push_back(q);
    }
    if (tables_dirty_) {
      CK(cudaStreamSynchronize(stream_));  // no launch reads the old tables any more
      ela3d_status st = upload_tables();
      if (st != ELA3D_OK) return st;
      tables_dirty_ = false;
    }
    if (!sched_key_.empty() && key == sched_key_ && sched_valid_) return ELA3D_OK;
    sched_key_ = key;
    sched_valid_ = true;
    steps_on_schedule_ = 0;
    invalidate_graph();
    if (shapes.empty()) {
      nblocks_ = 0;
      return ELA3D_OK;
    }
    std::vector<Item> items;
    std::vector<int2> ranges;
    const int kind = choice_.kind >= kScheduleFlow ? 1 : choice_.kind;
    build_schedule(shapes, var_->tx, var_->ty, kind, std::max(choice_.chunk, 1), per_sm_ * num_sms_, &items,
                   &ranges);
    if (items.empty()) BAD("empty schedule");
    for (const Item &it : items)
      if (it.k1 <= it.k0) BAD("internal: empty work item");
    CK(cudaStreamSynchronize(stream_));  // kernels in flight may still read the old tables
    if (items.size() > items_cap_) {
      if (d_items_) CK(cudaFree(d_items_));
      d_items_ = nullptr;
      CK(cudaMalloc(&d_items_, items.size() * sizeof(Item)));
      items_cap_ = items.size();
    }
    if (ranges.size() > ranges_cap_) {
      if (d_ranges_) CK(cudaFree(d_ranges_));
      d_ranges_ = nullptr;
      CK(cudaMalloc(&d_ranges_, ranges.size() * sizeof(int2)));
      ranges_cap_ = ranges.size();
    }
    CK(cudaMemcpy(d_items_, items.data(), items.size() * sizeof(Item), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_ranges_, ranges.data(), ranges.size() * sizeof(int2), cudaMemcpyHostToDevice));
    nblocks_ = (int)ranges.size();
    nitems_ = (int)items.size();
    flow_items_ = 0;
    flow_steps_ = 0;
    if (flow_on()) return rebuild_flow(key);
    return ELA3D_OK;
  }

  // The dataflow list of the active shots for up to kFlowSteps steps (fewer
  // when the list would pass kFlowMaxItems items; a launch walks it up to
  // flow_passes_ times), their completion counters, and the descriptors that
  // point at them.
  ela3d_status rebuild_flow(const std::vector<int> &active) {
    std::vector<FlowShape> shapes;
    long long per_step = 0;
    const int C = std::max(choice_.chunk, 2);
    for (int q : active) {
      const ShotDesc<T> &d = shots_[q]->d;
      shapes.push_back({d.nx, d.ny, d.nz, q});
      const long long nt = (long long)((d.nx + var_->tx - 1) / var_->tx) * ((d.ny + var_->ty - 1) / var_->ty);
      per_step += 2 * nt * ((d.nz + C - 1) / C);
    }
    const int K = (int)std::max<long long>(1, std::min<long long>(flow_max_steps_, kFlowMaxItems / std::max(1ll, per_step)));
    std::vector<FlowItem> items;
    std::vector<int> off, nch;
    int nflags = 0;
    std::string why;
    // gap: by default three rounds of the grid, so an item is claimed when
    // the items it waits for have finished (the producer then acquires them
    // and loads the item's first planes while the block still works on its
    // previous item) and for grids near the L2 size while their results are
    // still in L2 (measured at 101^3: one round 31.4, three 32.2 Gcell/s;
    // neutral from 160^3 up)
    const int gap = choice_.lag > 0 ? choice_.lag : std::max(1, 3 * per_sm_flow_ * num_sms_);
    if (!build_flow_schedule(shapes, var_->tx, var_->ty, C, gap, choice_.kind == kScheduleFlowOverlap, K, &items,
                             &off, &nch, &nflags, &why))
      BAD(why);
    CK(cudaStreamSynchronize(stream_));
    if (items.size() > flow_cap_) {
      if (d_flow_) CK(cudaFree(d_flow_));
      d_flow_ = nullptr;
      flow_cap_ = 0;
      CK(cudaMalloc(&d_flow_, items.size() * sizeof(FlowItem)));
      flow_cap_ = items.size();
    }
    if ((size_t)nflags > flags_cap_) {
      if (d_flags_) CK(cudaFree(d_flags_));
      d_flags_ = nullptr;
      flags_cap_ = 0;
      CK(cudaMalloc(&d_flags_, (size_t)nflags * sizeof(int)));
      flags_cap_ = (size_t)nflags;
    }
    CK(cudaMemcpy(d_flow_, items.data(), items.size() * sizeof(FlowItem), cudaMemcpyHostToDevice));
    for (size_t a = 0; a < active.size(); ++a) {
      ShotDesc<T> &d = shots_[active[a]]->d;
      d.flow_flags = d_flags_ + off[a];
      d.flow_chunks = nch[a];
    }
    ela3d_status st = upload_tables();
    if (st != ELA3D_OK) return st;
    flow_items_ = (int)items.size();
    flow_steps_ = K;
    flags_used_ = (size_t)nflags;
    return ELA3D_OK;
  }

  // One launch of the dataflow kernel: steps tick .. tick + nsteps - 1.
  ela3d_status launch_flow(int tick, int nsteps) {
    int ctl = (inject_ > 0 ? CTL_WITHHOLD_LOADS : 0) | prefetch_;
    inject_ = std::max(0, inject_ - nsteps);
    const int *dtick = nullptr;
    void *args[] = {&d_desc_, &d_maps_, &d_flow_, &flow_items_, &flow_steps_, &nsteps, &tick, &dtick, &d_err_, &ctl};
    CK(cudaMemsetAsync(d_flags_, 0, flags_used_ * sizeof(int), stream_));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (timing_) {
      e0 = event(); e1 = event();
      CK(cudaEventRecord(e0, stream_));
    }
    const int grid = std::min(per_sm_flow_ * num_sms_, std::max(1, flow_items_));
    CK(cudaLaunchCooperativeKernel(var_->flow, dim3(grid), dim3(var_->threads), args, var_->flow_smem, stream_));
    if (timing_) {
      CK(cudaEventRecord(e1, stream_));
      pending_.push_back({e0, e1, nullptr, nsteps});
    }
    launches_ += 1;
    return ELA3D_OK;
  }

  void invalidate_graph() {
    if (gexec_) cudaGraphExecDestroy(gexec_);
    gexec_ = nullptr;
  }

  // A replayable graph of graph_steps_ steps reading the step from d_tick_
  // and advancing it at the end.
  ela3d_status ensure_graph() {
    if (gexec_) return ELA3D_OK;
    CK(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
    capturing_ = true;
    ela3d_status st = ELA3D_OK;
    for (int i = 0; i < graph_steps_ && st == ELA3D_OK; ++i) st = launch_step(i, d_tick_);
    cudaError_t e = cudaSuccess;
    if (st == ELA3D_OK) e = launch_tick_add(d_tick_, graph_steps_, stream_);
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(stream_, &g);
    capturing_ = false;
    launches_ -= (int64_t)graph_steps_ * (2 + (any_explosive_ ? 1 : 0));  // counted when replayed
    if (st != ELA3D_OK) { if (g) cudaGraphDestroy(g); return st; }
    if (e != cudaSuccess || e2 != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return status_from_cuda(e != cudaSuccess ? e : e2, "graph capture");
    }
    cudaError_t e3 = cudaGraphInstantiate(&gexec_, g, 0);
    cudaGraphDestroy(g);
    if (e3 != cudaSuccess) { gexec_ = nullptr; return status_from_cuda(e3, "cudaGraphInstantiate"); }
    return ELA3D_OK;
  }

  ela3d_status run_timed(int nsteps, double *ms) override {
    cudaEvent_t a = event(), b = event();
    CK(cudaEventRecord(a, stream_));
    ela3d_status st = enqueue(nsteps);
    if (st != ELA3D_OK) return st;
    CK(cudaEventRecord(b, stream_));
    st = sync();
    if (st != ELA3D_OK) return st;
    float t = 0.f;
    CK(cudaEventElapsedTime(&t, a, b));
    free_events_.push_back(a);
    free_events_.push_back(b);
    if (ms) *ms = t;
    return ELA3D_OK;
  }

  ela3d_status sync() override {
    CK(cudaStreamSynchronize(stream_));
    unsigned err = 0;
    CK(cudaMemcpy(&err, d_err_, sizeof(unsigned), cudaMemcpyDeviceToHost));
    collect_timing();
    if (err) {
      CK(cudaMemset(d_err_, 0, sizeof(unsigned)));
      set_last_error("device-side wait exceeded its limit (error bits " + std::to_string(err) + ")");
      return ELA3D_ERR_TIMEOUT;
    }
    return ELA3D_OK;
  }

  ela3d_status seismograms(int shot, void *out, int out_fp64) override {
    if (shot < 0 || shot >= nshots() || !out) BAD("bad shot or output");
    const Shot<T> &s = *shots_[shot];
    const size_t n = (size_t)s.p.nrec * 3 * s.nsamp;
    if (n == 0) return ELA3D_OK;
    std::vector<T> h(n);
    CK(cudaMemcpyAsync(h.data(), s.d.seis, n * sizeof(T), cudaMemcpyDeviceToHost, stream_));
    CK(cudaStreamSynchronize(stream_));
    convert_out(h.data(), n, out, out_fp64);
    return ELA3D_OK;
  }

  ela3d_status source_trace(int shot, void *out, int out_fp64) override {
    if (shot < 0 || shot >= nshots() || !out) BAD("bad shot or output");
    const Shot<T> &s = *shots_[shot];
    const size_t n = 3 * (size_t)(s.p.nstep + 1);
    std::vector<T> h(n);
    CK(cudaMemcpyAsync(h.data(), s.d.src_trace, n * sizeof(T), cudaMemcpyDeviceToHost, stream_));
    CK(cudaStreamSynchronize(stream_));
    convert_out(h.data(), n, out, out_fp64);
    return ELA3D_OK;
  }

  struct CheckpointHeader {
    char magic[8];          // "ELA3DCK1"
    int32_t version, precision, nx, ny, nz, npml, nstep, nrec, sampgat, pml_mode, step, _pad;
    int64_t pool_bytes;
    double e_ref;
    uint64_t params_hash;   // every parameter the time loop depends on
  };

  // FNV-1a over the values (not the padding) of the parameters that shape
  // the time loop: spacings, dt, C-PML coefficients, source, receivers.  The
  // model and fields travel in the checkpoint; the profiles and the source
  // table are recomputed by the restoring plan from these.
  static uint64_t params_hash(const ela3d_params &p, const std::vector<int32_t> &rec) {
    uint64_t h = 1469598103934665603ull;
    auto mix = [&h](const void *v, size_t n) {
      const unsigned char *b = static_cast<const unsigned char *>(v);
      for (size_t i = 0; i < n; ++i) h = (h ^ b[i]) * 1099511628211ull;
    };
    const double d[] = {p.dx, p.dy, p.dz, p.dt, p.npower, p.k_max, p.alpha_max, p.rcoef, p.vpml,
                        p.f0, p.t0, p.factor, p.src_w[0], p.src_w[1], p.src_w[2], p.angle_force};
    const int32_t n[] = {p.stf, p.src_kind, p.src_i, p.src_j, p.src_k};
    mix(d, sizeof d);
    mix(n, sizeof n);
    if (!rec.empty()) mix(rec.data(), rec.size() * sizeof(int32_t));
    return h;
  }

  int64_t checkpoint_bytes() const override {
    if (shots_.size() != 1) return -1;
    return (int64_t)sizeof(CheckpointHeader) + (int64_t)shots_[0]->pool_bytes;
  }

  CheckpointHeader checkpoint_header() const {
    const Shot<T> &s = *shots_[0];
    CheckpointHeader h{};
    std::memcpy(h.magic, "ELA3DCK1", 8);
    h.version = 2;
    h.precision = sizeof(T) == 8 ? ELA3D_FP64 : ELA3D_FP32;
    h.nx = s.p.nx; h.ny = s.p.ny; h.nz = s.p.nz;
    h.npml = s.p.npml; h.nstep = s.p.nstep; h.nrec = s.p.nrec; h.sampgat = s.p.sampgat;
    h.pml_mode = s.p.pml_mode;
    h.step = tick_ - s.d.tick0;
    h.pool_bytes = (int64_t)s.pool_bytes;
    h.e_ref = s.e_ref;
    h.params_hash = params_hash(s.p, s.rec);
    return h;
  }

  ela3d_status checkpoint_save(void *buf, int64_t bytes) override {
    if (shots_.size() != 1) BAD("checkpoints hold single-shot plans");
    if (!buf || bytes < checkpoint_bytes()) BAD("checkpoint buffer too small");
    const CheckpointHeader h = checkpoint_header();
    CK(cudaStreamSynchronize(stream_));
    std::memcpy(buf, &h, sizeof h);
    CK(cudaMemcpy(static_cast<char *>(buf) + sizeof h, shots_[0]->pool, shots_[0]->pool_bytes,
                  cudaMemcpyDeviceToHost));
    return ELA3D_OK;
  }

  ela3d_status checkpoint_load(const void *buf, int64_t bytes) override {
    if (shots_.size() != 1) BAD("checkpoints hold single-shot plans");
    if (!buf || bytes < (int64_t)sizeof(CheckpointHeader)) BAD("checkpoint buffer too small");
    CheckpointHeader h;
    std::memcpy(&h, buf, sizeof h);
    const CheckpointHeader mine = checkpoint_header();
    if (std::memcmp(h.magic, mine.magic, 8) != 0 || h.version != mine.version) BAD("not an ela3d checkpoint");
    if (h.precision != mine.precision || h.nx != mine.nx || h.ny != mine.ny || h.nz != mine.nz ||
        h.npml != mine.npml || h.nstep != mine.nstep || h.nrec != mine.nrec || h.sampgat != mine.sampgat ||
        h.pml_mode != mine.pml_mode || h.pool_bytes != mine.pool_bytes || h.params_hash != mine.params_hash)
      BAD("checkpoint was written by a plan with other parameters");
    if (bytes < (int64_t)sizeof h + h.pool_bytes) BAD("checkpoint buffer truncated");
    if (h.step < 0) BAD("checkpoint step out of range");  // (a plan may run past nstep)
    Shot<T> &s = *shots_[0];
    CK(cudaStreamSynchronize(stream_));
    CK(cudaMemcpy(s.pool, static_cast<const char *>(buf) + sizeof h, s.pool_bytes, cudaMemcpyHostToDevice));
    tick_ = s.d.tick0 + h.step;
    s.e_ref = h.e_ref;
    return ELA3D_OK;
  }

  ela3d_status field(int shot, int comp, void *out, int out_fp64) override {
    if (shot < 0 || shot >= nshots() || !out) BAD("bad shot or output");
    if (comp < 0 || comp > 8) BAD("bad field component");
    const Shot<T> &s = *shots_[shot];
    const int nx = s.d.nx, ny = s.d.ny, nz = s.d.nz;
    const size_t n = (size_t)nx * ny * nz;
    if ((sizeof(T) == 8) == (out_fp64 != 0)) {
      CK(cudaMemcpy2DAsync(out, nx * sizeof(T), s.d.f[comp], s.d.px * sizeof(T), nx * sizeof(T), (size_t)ny * nz,
                           cudaMemcpyDeviceToHost, stream_));
      CK(cudaStreamSynchronize(stream_));
      return ELA3D_OK;
    }
    std::vector<T> h(n);
    CK(cudaMemcpy2DAsync(h.data(), nx * sizeof(T), s.d.f[comp], s.d.px * sizeof(T), nx * sizeof(T), (size_t)ny * nz,
                         cudaMemcpyDeviceToHost, stream_));
    CK(cudaStreamSynchronize(stream_));
    convert_out(h.data(), n, out, out_fp64);
    return ELA3D_OK;
  }

  ela3d_status energy(int shot, double *out) override {
    if (shot < 0 || shot >= nshots() || !out) BAD("bad shot or output");
    const Shot<T> &s = *shots_[shot];
    const ShotDesc<T> *dd = d_desc_ ? d_desc_ + shot : nullptr;
    if (!dd) BAD("engine not finalized");
    // the result and one partial sum per plane (grown to the largest nz seen)
    if (energy_cap_ < s.d.nz + 1) {
      CK(cudaStreamSynchronize(stream_));
      if (d_energy_) cudaFree(d_energy_);
      d_energy_ = nullptr;
      energy_cap_ = 0;
      CK(cudaMalloc(&d_energy_, sizeof(double) * (size_t)(s.d.nz + 1)));
      energy_cap_ = s.d.nz + 1;
    }
    CK(Fp<T>::energy(dd, s.d.nx, s.d.ny, s.d.nz, d_energy_, stream_));
    CK(cudaMemcpyAsync(out, d_energy_, sizeof(double), cudaMemcpyDeviceToHost, stream_));
    CK(cudaStreamSynchronize(stream_));
    return ELA3D_OK;
  }

  ela3d_status profiles(int shot, int axis, double *out) override {
    if (shot < 0 || shot >= nshots() || !out || axis < 0 || axis > 2) BAD("bad shot, axis or output");
    const Shot<T> &s = *shots_[shot];
    const int n = axis == 0 ? s.d.nx : axis == 1 ? s.d.ny : s.d.nz;
    const int stride = axis == 0 ? s.px : n;
    const size_t off = axis == 0 ? 0 : axis == 1 ? 6 * (size_t)s.px : 6 * (size_t)(s.px + s.d.ny);
    std::vector<T> h(6 * (size_t)stride);
    CK(cudaMemcpyAsync(h.data(), s.prof + off, h.size() * sizeof(T), cudaMemcpyDeviceToHost, stream_));
    CK(cudaStreamSynchronize(stream_));
    for (int q = 0; q < 6; ++q)
      for (int i = 0; i < n; ++i) out[(size_t)q * n + i] = (double)h[(size_t)q * stride + i];
    return ELA3D_OK;
  }

  ela3d_status info(int shot, ela3d_plan_info *out) override {
    if (shot < 0 || shot >= nshots() || !out) BAD("bad shot or output");
    const Shot<T> &s = *shots_[shot];
    out->nx = s.d.nx; out->ny = s.d.ny; out->nz = s.d.nz; out->pitch_x = s.d.px;
    out->step = tick_ - s.d.tick0;
    out->nsamp = s.nsamp;
    out->nrec = s.p.nrec;
    out->precision = sizeof(T) == 8 ? ELA3D_FP64 : ELA3D_FP32;
    out->device_bytes = (int64_t)(s.pool_bytes + s.prof_bytes);
    for (int a = 0; a < 3; ++a) { out->slab_lo[a] = s.lo[a]; out->slab_hi[a] = s.hi[a]; }
    return ELA3D_OK;
  }

  // Fills the padding columns [nx, px) of every field and memory-variable
  // array of every shot with `value` (test hook).
  ela3d_status poison_padding(double value) override {
    CK(cudaStreamSynchronize(stream_));
    for (auto &sp : shots_) {
      const ShotDesc<T> &d = sp->d;
      const int w = d.px - d.nx;
      if (w <= 0) continue;
      auto put = [&](T *dst, size_t dpitch, int width, size_t rows) -> cudaError_t {
        if (width <= 0 || rows == 0) return cudaSuccess;
        std::vector<T> fill((size_t)width * rows, (T)value);
        return cudaMemcpy2D(dst, dpitch * sizeof(T), fill.data(), width * sizeof(T), width * sizeof(T), rows,
                            cudaMemcpyHostToDevice);
      };
      const size_t rows = (size_t)d.ny * d.nz;
      for (int c = 0; c < 9; ++c) CK(put(d.f[c] + d.nx, d.px, w, rows));
      for (int v = 0; v < 6; ++v) {
        CK(put(d.psi_y + v * d.psy + d.nx, d.px, w, (size_t)d.nz * d.yw));
        CK(put(d.psi_z + v * d.psz + d.nx, d.px, w, (size_t)d.zw * d.ny));
        // x slab: a column x >= xr sits at slab index xl + (x - xr)
        const int x0 = std::max(d.nx, d.xr);
        if (d.xw > 0 && x0 < d.px) CK(put(d.psi_x + v * d.psx + d.xl + (x0 - d.xr), d.xw, d.px - x0, rows));
      }
    }
    return ELA3D_OK;
  }

  // Verifies every guard zone of every shot still holds kGuardByte.
  ela3d_status check_guards() override {
    CK(cudaStreamSynchronize(stream_));
    for (auto &sp : shots_) {
      for (const auto &g : sp->guards) {
        std::vector<unsigned char> h(g.bytes);
        CK(cudaMemcpy(h.data(), sp->pool + g.off, g.bytes, cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < g.bytes; ++i)
          if (h[i] != kGuardByte) {
            set_last_error("guard zone after " + std::string(g.after) + " overwritten at byte " +
                           std::to_string(i) + " of " + std::to_string(g.bytes));
            return ELA3D_ERR_CORRUPT;
          }
      }
    }
    return ELA3D_OK;
  }

  ela3d_status inject_timeout(int launches) override {
    if (launches < 0) BAD("launches must be >= 0");
    inject_ = launches;
    return ELA3D_OK;
  }

  int64_t launches() const override { return launches_; }

  int64_t device_bytes() const override {
    int64_t b = 0;
    for (auto &sp : shots_) b += (int64_t)(sp->pool_bytes + sp->prof_bytes);
    return b;
  }

  ela3d_status set_timing(bool on) override {
    timing_ = on;
    if (on) { t_stress_ = t_vel_ = 0.0; n_stress_ = n_vel_ = 0; }
    return ELA3D_OK;
  }

  ela3d_status flow_timing(double *ms, int64_t *launches, int64_t *steps) override {
    CK(cudaStreamSynchronize(stream_));
    collect_timing();
    if (ms) *ms = t_flow_;
    if (launches) *launches = n_flow_;
    if (steps) *steps = steps_flow_;
    return ELA3D_OK;
  }

  ela3d_status timing(double *s_ms, double *v_ms, int64_t *ns, int64_t *nv) override {
    CK(cudaStreamSynchronize(stream_));
    collect_timing();
    if (s_ms) *s_ms = t_stress_;
    if (v_ms) *v_ms = t_vel_;
    if (ns) *ns = n_stress_;
    if (nv) *nv = n_vel_;
    return ELA3D_OK;
  }

  // stability monitor for one shot (called by the plan between chunks)
  ela3d_status check_energy(int shot) {
    double e = 0.0;
    ela3d_status st = energy(shot, &e);
    if (st != ELA3D_OK) return st;
    Shot<T> &s = *shots_[shot];
    if (!std::isfinite(e)) {
      set_last_error("energy is not finite");
      return ELA3D_ERR_UNSTABLE;
    }
    const double t = (tick_ - s.d.tick0) * s.p.dt;
    if (t > 2.5 * s.p.t0 + 2.0 / std::max(1e-30, s.p.f0)) {  // the source has ended
      if (s.e_ref < 0) s.e_ref = e;
      else if (e > 2.0 * s.e_ref + 1e-300) {
        set_last_error("energy grew after the source ended");
        return ELA3D_ERR_UNSTABLE;
      }
    }
    return ELA3D_OK;
  }
  const ela3d_params &params(int shot) const { return shots_[shot]->p; }

 private:
  template <typename U>
  static void convert_out(const U *h, size_t n, void *out, int out_fp64) {
    if (out_fp64) {
      double *o = static_cast<double *>(out);
      for (size_t i = 0; i < n; ++i) o[i] = (double)h[i];
    } else {
      float *o = static_cast<float *>(out);
      for (size_t i = 0; i < n; ++i) o[i] = (float)h[i];
    }
  }

  cudaEvent_t event() {
    cudaEvent_t e = nullptr;
    if (!free_events_.empty()) {
      e = free_events_.back();
      free_events_.pop_back();
    } else {
      cudaEventCreate(&e);
    }
    return e;
  }

  void collect_timing() {
    for (auto &t : pending_) {
      float a = 0.f, b = 0.f;
      if (!t.e2) {
        if (cudaEventElapsedTime(&a, t.e0, t.e1) == cudaSuccess) { t_flow_ += a; ++n_flow_; steps_flow_ += t.flow_steps; }
        free_events_.push_back(t.e0);
        free_events_.push_back(t.e1);
        continue;
      }
      if (cudaEventElapsedTime(&a, t.e0, t.e1) == cudaSuccess) { t_stress_ += a; ++n_stress_; }
      if (cudaEventElapsedTime(&b, t.e1, t.e2) == cudaSuccess) { t_vel_ += b; ++n_vel_; }
      free_events_.push_back(t.e0);
      free_events_.push_back(t.e1);
      free_events_.push_back(t.e2);
    }
    pending_.clear();
  }

  void release() {
    if (stream_) cudaStreamSynchronize(stream_);
    for (auto &sp : shots_) release_shot(*sp);
    shots_.clear();
    for (auto &t : pending_) { cudaEventDestroy(t.e0); cudaEventDestroy(t.e1); cudaEventDestroy(t.e2); }
    for (auto e : free_events_) cudaEventDestroy(e);
    pending_.clear();
    free_events_.clear();
    if (d_desc_) cudaFree(d_desc_);
    if (d_maps_) cudaFree(d_maps_);
    if (d_items_) cudaFree(d_items_);
    if (d_ranges_) cudaFree(d_ranges_);
    if (d_err_) cudaFree(d_err_);
    if (d_energy_) cudaFree(d_energy_);
    if (d_tick_) cudaFree(d_tick_);
    if (d_flow_) cudaFree(d_flow_);
    if (d_flags_) cudaFree(d_flags_);
    d_flow_ = nullptr;
    d_flags_ = nullptr;
    invalidate_graph();
    if (stream_) cudaStreamDestroy(stream_);
    if (setup_) cudaStreamDestroy(setup_);
    d_desc_ = nullptr; d_maps_ = nullptr; d_items_ = nullptr; d_ranges_ = nullptr;
    d_err_ = nullptr; d_energy_ = nullptr; d_tick_ = nullptr; stream_ = nullptr; setup_ = nullptr;
  }

  struct Ev { cudaEvent_t e0, e1, e2; int flow_steps = 0; };   // e2 null: a dataflow launch
  int device_ = 0, num_sms_ = 1;
  cudaStream_t stream_ = nullptr;
  std::vector<std::unique_ptr<Shot<T>>> shots_;
  const Variant *var_ = nullptr;
  TuneChoice choice_{};
  bool finalized_ = false, any_explosive_ = false;
  ShotDesc<T> *d_desc_ = nullptr;
  ShotMaps *d_maps_ = nullptr;
  Item *d_items_ = nullptr;
  int2 *d_ranges_ = nullptr;
  unsigned *d_err_ = nullptr;
  double *d_energy_ = nullptr;
  int energy_cap_ = 0;   // doubles held by d_energy_
  int nblocks_ = 0, nitems_ = 0, per_sm_ = 1;
  size_t items_cap_ = 0, ranges_cap_ = 0;
  std::vector<int> sched_key_;
  bool sched_valid_ = false, retire_ = false;
  bool tables_dirty_ = false;  // a shot joined since the device tables were written
  cudaStream_t setup_ = nullptr;
  int tick_ = 0;
  int inject_ = 0;   // steps left whose launches withhold their loads (test hook)
  int prefetch_ = kPrefetchDefault;  // memory-variable prefetch hints (x slab to L1, y/z slabs to L2)
  int prefetch_env_ = -1;
  size_t guard_ = 0;   // bytes of each debug guard zone (0 = off)
  int steps_on_schedule_ = 0;  // steps run with the current work items
  static constexpr unsigned char kGuardByte = 0xA5;
  int *d_tick_ = nullptr;
  cudaGraphExec_t gexec_ = nullptr;
  bool use_graphs_ = true, capturing_ = false;
  int64_t launches_ = 0;
  uint64_t next_key_ = 1;
  static constexpr int kGraphSteps = 50;
  // steps per replayed graph; ELA3D_GRAPH_STEPS=<n> overrides it (the
  // measurement of one graph per whole run against replays of 50 steps)
  int graph_steps_ = kGraphSteps;
  bool timing_ = false;
  std::vector<Ev> pending_;
  std::vector<cudaEvent_t> free_events_;
  double t_stress_ = 0.0, t_vel_ = 0.0;
  int64_t n_stress_ = 0, n_vel_ = 0;
  // dataflow path (schedule kind 3)
  static constexpr int kFlowSteps = 50;
  // passes over the list per dataflow launch: a launch runs up to
  // kFlowSteps * kFlowPasses steps, the list is built for kFlowSteps
  // (measured: 200-step launches 1% faster than 50-step ones at 101^3 and
  // 256^3; a 200-step list would take 25-40 ms to build on the host)
  static constexpr int kFlowPasses = 4;
  // steps of the dataflow list; ELA3D_FLOW_STEPS=<n> overrides it, and
  // ELA3D_FLOW_PASSES=<n> the passes per launch (experiments)
  int flow_max_steps_ = kFlowSteps;
  int flow_passes_ = kFlowPasses;
  static constexpr long long kFlowMaxItems = 1 << 20;
  FlowItem *d_flow_ = nullptr;
  int *d_flags_ = nullptr;
  size_t flow_cap_ = 0, flags_cap_ = 0, flags_used_ = 0;
  int flow_items_ = 0, flow_steps_ = 0, per_sm_flow_ = 0;
  double t_flow_ = 0.0;
  int64_t n_flow_ = 0, steps_flow_ = 0;

};

std::unique_ptr<EngineBase> make_engine(int fp64, ela3d_status *st) {
  std::unique_ptr<EngineBase> e;
  if (fp64) {
    auto p = std::make_unique<Engine<double>>();
    *st = p->init();
    e = std::move(p);
  } else {
    auto p = std::make_unique<Engine<float>>();
    *st = p->init();
    e = std::move(p);
  }
  return e;
}

ela3d_status engine_check_energy(EngineBase *e, int shot, int fp64) {
  if (fp64) return static_cast<Engine<double> *>(e)->check_energy(shot);
  return static_cast<Engine<float> *>(e)->check_energy(shot);
}

}  // namespace ela3d
