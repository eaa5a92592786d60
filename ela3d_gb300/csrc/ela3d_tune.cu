// ela3d_tune.cu -- the autotuner: times every compiled kernel variant (tile
// shape and pipeline depth) with the work schedules (z-chunk size, shot-major
// or shot-interleaved order) on the caller's own shots and keeps the fastest
// per workload shape.  Results live in a process-wide cache that plan and
// batch creation consult; ELA3D_TUNE_CACHE=<file> persists it across
// processes and ELA3D_AUTOTUNE=1 tunes on a cache miss at creation.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "ela3d_engine.h"

namespace ela3d {

namespace {
std::mutex g_mu;
std::map<std::string, TuneChoice> g_cache;
bool g_loaded = false;

const char *cache_file() {
  const char *f = std::getenv("ELA3D_TUNE_CACHE");
  return (f && *f) ? f : nullptr;
}

void load_locked() {
  if (g_loaded) return;
  g_loaded = true;
  const char *f = cache_file();
  if (!f) return;
  FILE *fp = std::fopen(f, "r");
  if (!fp) return;
  // one line per workload: key variant kind chunk blocks_per_sm prefetch [lag]
  char line[1024], key[512];
  while (std::fgets(line, sizeof line, fp)) {
    TuneChoice c{};
    const int got = std::sscanf(line, "%511s %d %d %d %d %d %d", key, &c.variant, &c.kind, &c.chunk,
                                &c.blocks_per_sm, &c.prefetch, &c.lag);
    if (got == 6 || got == 7) g_cache[key] = c;
  }
  std::fclose(fp);
}

void save_locked() {
  const char *f = cache_file();
  if (!f) return;
  FILE *fp = std::fopen(f, "w");
  if (!fp) return;
  for (auto &kv : g_cache)
    std::fprintf(fp, "%s %d %d %d %d %d %d\n", kv.first.c_str(), kv.second.variant, kv.second.kind,
                 kv.second.chunk, kv.second.blocks_per_sm, kv.second.prefetch, kv.second.lag);
  std::fclose(fp);
}
}  // namespace

// Workload shape: precision, shot count and the sorted set of grid sizes
// and PML widths (what the kernels' speed depends on).
std::string tune_key(const std::vector<ela3d_params> &ps) {
  std::vector<std::string> parts;
  for (auto &p : ps) {
    std::ostringstream o;
    o << p.nx << "x" << p.ny << "x" << p.nz << "p" << p.npml;
    parts.push_back(o.str());
  }
  std::sort(parts.begin(), parts.end());
  std::ostringstream k;
  k << (ps.empty() ? 0 : ps[0].precision) << ":" << ps.size() << ":";
  // many-shot keys keep the distinct shapes with counts
  for (size_t i = 0; i < parts.size();) {
    size_t j = i;
    while (j < parts.size() && parts[j] == parts[i]) ++j;
    k << parts[i] << "*" << (j - i) << ",";
    i = j;
  }
  return k.str();
}

// A cached choice is used only if the library can run it (a cache file may
// come from a library compiled with other variants); otherwise it counts as
// a miss.
bool tune_lookup(const std::vector<ela3d_params> &ps, TuneChoice *out) {
  std::lock_guard<std::mutex> g(g_mu);
  load_locked();
  auto it = g_cache.find(tune_key(ps));
  if (it == g_cache.end()) return false;
  const TuneChoice &c = it->second;
  int nv = 0;
  const Variant *vs = variants(&nv);
  const bool fp64 = !ps.empty() && ps[0].precision == ELA3D_FP64;
  if (c.variant < 0 || c.variant >= nv || (vs[c.variant].fp64 != 0) != fp64 || c.kind < 0 ||
      c.kind > kScheduleFlowOverlap || c.chunk < 0 || c.blocks_per_sm < 0 || c.lag < 0 ||
      (c.kind >= kScheduleFlow && (c.chunk < 2 || !vs[c.variant].flow)))
    return false;
  *out = c;
  out->prefetch &= CTL_PF_X | CTL_PF_YZ;
  return true;
}

void tune_store(const std::vector<ela3d_params> &ps, const TuneChoice &c) {
  std::lock_guard<std::mutex> g(g_mu);
  load_locked();
  g_cache[tune_key(ps)] = c;
  save_locked();
}

// Candidate schedules and prefetch modes for a workload: contiguous shares;
// z-chunks of 6..128 planes round-robin; for batches also shot-interleaved
// chunks; the dataflow kernel; each with both memory-variable prefetches or
// the x slab's only.
// The dataflow kernel (kinds 3 and 4) is tried with 4- to 16-plane chunks.
static std::vector<TuneChoice> schedules(int nshots, bool flow) {
  std::vector<TuneChoice> v;
  for (int pf : {kPrefetchDefault, (int)CTL_PF_X}) {
    v.push_back({0, 0, 16, 0, pf});
    for (int ch : {6, 8, 10, 12, 16, 32, 64, 128}) v.push_back({0, 1, ch, 0, pf});
    if (nshots > 1)
      for (int ch : {8, 16}) v.push_back({0, 2, ch, 0, pf});
    if (flow) {
      for (int ch : {4, 6, 8, 12, 16, 24, 32, 48, 64, 96}) v.push_back({0, kScheduleFlowOverlap, ch, 0, pf, 0});
      for (int ch : {8, 16}) v.push_back({0, kScheduleFlow, ch, 0, pf, 0});
    }
  }
  // the dataflow kernel on grids that fit in L2 runs best without the
  // memory-variable prefetch
  if (flow) {
    for (int ch : {4, 6, 8, 12, 16, 24, 32, 48, 64, 96}) v.push_back({0, kScheduleFlowOverlap, ch, 0, 0, 0});
    for (int ch : {8, 16}) v.push_back({0, kScheduleFlow, ch, 0, 0, 0});
  }
  return v;
}

ela3d_status autotune(const std::vector<ela3d_params> &ps, const std::vector<const float *> &cp,
                      const std::vector<const float *> &cs, const std::vector<const float *> &rho, int steps,
                      TuneChoice *best, double *best_ms, std::vector<std::pair<TuneChoice, double>> *table) {
  if (ps.empty() || steps < 1) return ELA3D_ERR_INVALID_ARG;
  const int fp64 = ps[0].precision == ELA3D_FP64;
  int nv = 0;
  const Variant *vs = variants(&nv);
  double best_t = 1e300;
  TuneChoice bc{-1, 0, 0, 0};
  for (int v = 0; v < nv; ++v) {
    // (the cp.async-filled variant is a measured alternative, 5-6x slower)
    if (vs[v].fp64 != fp64 || vs[v].loads != LOAD_TMA) continue;
    // one engine per variant (the tensor maps depend on the tile); the
    // schedules and prefetch modes are switched in place
    ela3d_status st;
    auto eng = make_engine(fp64, &st);
    for (size_t q = 0; q < ps.size() && st == ELA3D_OK; ++q) {
      int share = -1;
      for (size_t j = 0; j < q && share < 0; ++j)
        if (cp[j] == cp[q] && cs[j] == cs[q] && rho[j] == rho[q] && ps[j].nx == ps[q].nx &&
            ps[j].ny == ps[q].ny && ps[j].nz == ps[q].nz)
          share = (int)j;
      st = eng->add_shot(ps[q], cp[q], cs[q], rho[q], share);
    }
    if (st == ELA3D_ERR_OOM) return st;
    if (st != ELA3D_OK) continue;
    // the dataflow list is rebuilt on the host whenever shots join or
    // retire, which batches and servers do: it is tried for single shots
    std::vector<TuneChoice> cands = schedules((int)ps.size(), vs[v].flow != nullptr && ps.size() == 1);
    if (ps.size() == 1) {
      // the built-in choice for this shot is always among the candidates
      // (its chunk is sized to the shot)
      const TuneChoice d = default_choice(fp64, ps[0].nx, ps[0].ny, ps[0].nz, ps[0].src_kind == ELA3D_SRC_EXPLOSIVE);
      bool have = d.variant != v;
      for (const TuneChoice &c : cands)
        have = have || (c.kind == d.kind && c.chunk == d.chunk && c.prefetch == d.prefetch && c.lag == d.lag);
      if (!have) cands.push_back({0, d.kind, d.chunk, 0, d.prefetch, d.lag});
    }
    for (TuneChoice c : cands) {
      c.variant = v;
      st = eng->retune(c);
      if (st == ELA3D_OK) st = eng->enqueue(2);  // warm-up
      if (st == ELA3D_OK) st = eng->sync();
      double ms = 0.0;
      if (st == ELA3D_OK) st = eng->run_timed(steps, &ms);
      if (st == ELA3D_ERR_OOM) return st;
      if (st != ELA3D_OK) break;  // a variant that does not run is skipped
      if (table) table->push_back({c, ms});
      if (ms < best_t) {
        best_t = ms;
        bc = c;
      }
    }
  }
  if (bc.variant < 0) {
    set_last_error("no kernel variant ran");
    return ELA3D_ERR_CUDA;
  }
  *best = bc;
  if (best_ms) *best_ms = best_t;
  tune_store(ps, bc);
  return ELA3D_OK;
}

}  // namespace ela3d

using namespace ela3d;

extern "C" ela3d_status ela3d_autotune(int32_t nshots, const ela3d_params *params, const float *const *cp,
                                       const float *const *cs, const float *const *rho, int32_t steps,
                                       ela3d_tuning *best, double *best_ms, int32_t *candidates) {
  if (nshots < 1 || !params || !cp || !cs || !rho || !best || steps < 1) return ELA3D_ERR_INVALID_ARG;
  std::vector<ela3d_params> ps(params, params + nshots);
  for (auto &p : ps) {
    ela3d_status st = validate_params(p);
    if (st != ELA3D_OK) return st;
    if (p.precision != ps[0].precision) return ELA3D_ERR_INVALID_ARG;
  }
  std::vector<const float *> a(cp, cp + nshots), b(cs, cs + nshots), c(rho, rho + nshots);
  TuneChoice bc{};
  std::vector<std::pair<TuneChoice, double>> table;
  ela3d_status st = autotune(ps, a, b, c, steps, &bc, best_ms, &table);
  if (st != ELA3D_OK) return st;
  best->variant = bc.variant;
  best->schedule = bc.kind;
  best->chunk = bc.chunk;
  best->blocks_per_sm = bc.blocks_per_sm;
  best->prefetch = bc.prefetch;
  best->lag = bc.lag;
  if (candidates) *candidates = (int32_t)table.size();
  return ELA3D_OK;
}
