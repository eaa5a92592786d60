// ela3d_capi.cu -- the extern "C" entry points of include/ela3d.h.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "ela3d_engine.h"

using namespace ela3d;

struct ela3d_plan {
  std::unique_ptr<EngineBase> eng;
  int fp64 = 0;
  ela3d_params p{};
};

struct ela3d_batch {
  std::unique_ptr<EngineBase> eng;
  int fp64 = 0;
};

// A caller's tuning fields, checked before any device work: -1 (0 for the
// chunk) selects the default; a variant must be compiled into the library
// and match the shots' precision.
ela3d_status ela3d::validate_tuning(const ela3d_tuning *t, int32_t precision) {
  if (!t) return ELA3D_OK;
  int nv = 0;
  const Variant *vs = variants(&nv);
  if (t->variant >= nv || t->variant < -1) {
    set_last_error("no such kernel variant");
    return ELA3D_ERR_INVALID_ARG;
  }
  if (t->variant >= 0 && (vs[t->variant].fp64 != 0) != (precision == ELA3D_FP64)) {
    set_last_error("kernel variant of the other precision");
    return ELA3D_ERR_INVALID_ARG;
  }
  if (t->schedule < -1 || t->schedule > kScheduleFlowOverlap || t->chunk < 0 || t->blocks_per_sm < -1 ||
      t->prefetch < -1 || t->lag < -1) {
    set_last_error("tuning field out of range");
    return ELA3D_ERR_INVALID_ARG;
  }
  if (t->schedule >= kScheduleFlow && t->chunk == 1) {
    set_last_error("the dataflow schedule needs z-chunks of at least 2 planes");
    return ELA3D_ERR_INVALID_ARG;
  }
  return ELA3D_OK;
}

extern "C" {

const char *ela3d_version(void) { return "ela3d-gb300 0.1"; }

const char *ela3d_last_error(void) { return last_error(); }

const char *ela3d_status_string(ela3d_status s) {
  switch (s) {
    case ELA3D_OK: return "ok";
    case ELA3D_ERR_INVALID_ARG: return "invalid argument";
    case ELA3D_ERR_OOM: return "out of device memory";
    case ELA3D_ERR_CUDA: return "CUDA error";
    case ELA3D_ERR_UNSTABLE: return "simulation unstable";
    case ELA3D_ERR_TIMEOUT: return "device wait timed out";
    case ELA3D_ERR_NO_DEVICE: return "no CUDA device";
    case ELA3D_ERR_BUSY: return "busy";
    case ELA3D_ERR_CANCELLED: return "cancelled";
    case ELA3D_ERR_NOT_FOUND: return "not found";
    case ELA3D_ERR_NOT_READY: return "not ready";
    case ELA3D_ERR_CORRUPT: return "device memory guard overwritten";
  }
  return "unknown status";
}

ela3d_status ela3d_params_default(ela3d_params *p) {
  if (!p) return ELA3D_ERR_INVALID_ARG;
  *p = ela3d_params{};
  p->nx = p->ny = p->nz = 500;            // NIMX/NIMY/NIMZ
  p->nstep = 1000;                        // NSTEP
  p->dx = p->dy = p->dz = 10.0;           // DELTAX
  p->dt = 1e-3;                           // DELTATT
  p->npml = 10;                           // NPOINTS_PML
  p->pml_mode = ELA3D_PML_COMPAT;
  p->npower = 2.0;
  p->k_max = 1.0;
  p->alpha_max = -1.0;                    // 2*PI*(f0/2)
  p->rcoef = 1e-3;
  p->vpml = 3000.0;
  p->f0 = 35.0;
  p->t0 = 1.2 / 35.0;
  p->factor = 1e7;
  p->stf = ELA3D_STF_GAUSS_DERIV;
  p->src_kind = ELA3D_SRC_EXPLOSIVE;
  p->src_i = 501 / 2 - 1;                 // ISOURCE = DIMX/2 (1-based)
  p->src_j = 501 / 2 - 1;
  p->src_k = 11 - 1;                      // KSOURCE = 11 (1-based)
  p->sampgat = 2;
  p->src_w[0] = 0.0;
  p->src_w[1] = 0.0;
  p->src_w[2] = 1.0;
  p->angle_force = 0.0;
  p->rec = nullptr;
  p->nrec = 0;
  p->precision = ELA3D_FP32;
  p->it_output = 200;
  p->energy_every = 0;
  return ELA3D_OK;
}

int32_t ela3d_variant_count(void) {
  int n = 0;
  variants(&n);
  return n;
}

ela3d_status ela3d_variant_get(int32_t index, ela3d_variant_info *out) {
  int n = 0;
  const Variant *v = variants(&n);
  if (!out || index < 0 || index >= n) return ELA3D_ERR_INVALID_ARG;
  out->fp64 = v[index].fp64;
  out->tile_x = v[index].tx;
  out->tile_y = v[index].ty;
  out->stages = v[index].ns;
  out->threads = v[index].threads;
  out->stress_smem = v[index].stress_smem;
  out->velocity_smem = v[index].vel_smem;
  out->loads = v[index].loads;
  out->velocity_stages = v[index].ns_vel;
  return ELA3D_OK;
}

// The choice for a workload: fields the caller set win; the rest come from
// the autotuner's cache (tuning on a miss when ELA3D_AUTOTUNE=1), else the
// built-in default.
static TuneChoice resolve_tuning(const std::vector<ela3d_params> &ps, const float *const *cp,
                                 const float *const *cs, const float *const *rho, const ela3d_tuning *t) {
  const ela3d_params &p = ps[0];
  // (the size-aware default applies to single shots; many shots give
  // round-robin chunks enough to go around)
  TuneChoice c = ps.size() == 1 ? default_choice(p.precision == ELA3D_FP64, p.nx, p.ny, p.nz,
                                                 p.src_kind == ELA3D_SRC_EXPLOSIVE)
                                : default_choice(p.precision == ELA3D_FP64, 0, 0, 0);
  const bool explicit_variant = t && t->variant >= 0;
  if (!explicit_variant) {
    TuneChoice cached{};
    if (tune_lookup(ps, &cached)) {
      c = cached;
    } else {
      const char *env = std::getenv("ELA3D_AUTOTUNE");
      if (env && env[0] == '1' && cp && cs && rho) {
        std::vector<const float *> a(cp, cp + ps.size()), b(cs, cs + ps.size()), r(rho, rho + ps.size());
        TuneChoice tuned{};
        if (autotune(ps, a, b, r, 10, &tuned, nullptr, nullptr) == ELA3D_OK) c = tuned;
      }
    }
  }
  if (!t) return c;
  if (t->variant >= 0) c.variant = t->variant;
  if (t->schedule >= 0) c.kind = t->schedule;
  if (t->chunk > 0) c.chunk = t->chunk;
  if (t->blocks_per_sm >= 0) c.blocks_per_sm = t->blocks_per_sm;
  if (t->prefetch >= 0) c.prefetch = t->prefetch & (CTL_PF_X | CTL_PF_YZ);
  if (t->lag >= 0) c.lag = t->lag;
  return c;
}

ela3d_status ela3d_plan_create_tuned(const ela3d_params *p, const float *cp, const float *cs, const float *rho,
                                     const ela3d_tuning *tune, ela3d_plan **out) {
  if (!p || !out) return ELA3D_ERR_INVALID_ARG;
  *out = nullptr;
  ela3d_status st = validate_params(*p);
  if (st == ELA3D_OK) st = validate_tuning(tune, p->precision);
  if (st != ELA3D_OK) return st;
  if (!cp || !cs || !rho) {
    set_last_error("model arrays missing");
    return ELA3D_ERR_INVALID_ARG;
  }
  ela3d_plan *plan = new (std::nothrow) ela3d_plan();
  if (!plan) return ELA3D_ERR_OOM;
  plan->fp64 = p->precision == ELA3D_FP64;
  plan->p = *p;
  plan->eng = make_engine(plan->fp64, &st);
  if (st == ELA3D_OK) st = plan->eng->add_shot(*p, cp, cs, rho, -1);
  if (st == ELA3D_OK) {   // (tuning may time candidates: only for a valid shot)
    const TuneChoice c = resolve_tuning({*p}, &cp, &cs, &rho, tune);
    st = plan->eng->finalize(&c);
  }
  if (st != ELA3D_OK) {
    delete plan;
    return st;
  }
  plan->p.rec = nullptr;  // the engine keeps its own copy
  *out = plan;
  return ELA3D_OK;
}

static_assert(sizeof(ela3d_model_spec) == sizeof(ModelSpec), "model spec layout");

ela3d_status ela3d_plan_create_model(const ela3d_params *p, const ela3d_model_spec *model,
                                     const ela3d_tuning *tune, ela3d_plan **out) {
  if (!p || !model || !out) return ELA3D_ERR_INVALID_ARG;
  *out = nullptr;
  ela3d_status st = validate_params(*p);
  if (st == ELA3D_OK) st = validate_tuning(tune, p->precision);
  if (st != ELA3D_OK) return st;
  ela3d_plan *plan = new (std::nothrow) ela3d_plan();
  if (!plan) return ELA3D_ERR_OOM;
  plan->fp64 = p->precision == ELA3D_FP64;
  plan->p = *p;
  plan->eng = make_engine(plan->fp64, &st);
  ModelSpec spec;
  std::memcpy(&spec, model, sizeof(spec));
  if (st == ELA3D_OK) st = plan->eng->add_shot(*p, nullptr, nullptr, nullptr, -1, &spec);
  if (st == ELA3D_OK) {
    const TuneChoice c = resolve_tuning({*p}, nullptr, nullptr, nullptr, tune);
    st = plan->eng->finalize(&c);
  }
  if (st != ELA3D_OK) {
    delete plan;
    return st;
  }
  plan->p.rec = nullptr;
  *out = plan;
  return ELA3D_OK;
}

ela3d_status ela3d_model_generate(const ela3d_model_spec *model, int32_t nx, int32_t ny, int32_t nz, float *cp,
                                  float *cs, float *rho) {
  if (!model || nx < 1 || ny < 1 || nz < 1 || !cp || !cs || !rho) return ELA3D_ERR_INVALID_ARG;
  ModelSpec spec;
  std::memcpy(&spec, model, sizeof(spec));
  const size_t n = (size_t)nx * ny * nz;
  float *d = nullptr;
  ela3d_status st = status_from_cuda(cudaMalloc(&d, 3 * n * sizeof(float)), "cudaMalloc");
  if (st != ELA3D_OK) return st;
  st = status_from_cuda(launch_model_f32(spec, nx, ny, nz, nx, d, d + n, d + 2 * n, 0), "model kernel");
  if (st == ELA3D_OK) st = status_from_cuda(cudaDeviceSynchronize(), "model kernel");
  if (st == ELA3D_OK) st = status_from_cuda(cudaMemcpy(cp, d, n * sizeof(float), cudaMemcpyDeviceToHost), "copy");
  if (st == ELA3D_OK) st = status_from_cuda(cudaMemcpy(cs, d + n, n * sizeof(float), cudaMemcpyDeviceToHost), "copy");
  if (st == ELA3D_OK)
    st = status_from_cuda(cudaMemcpy(rho, d + 2 * n, n * sizeof(float), cudaMemcpyDeviceToHost), "copy");
  cudaFree(d);
  return st;
}

ela3d_status ela3d_plan_create(const ela3d_params *p, const float *cp, const float *cs, const float *rho,
                               ela3d_plan **out) {
  return ela3d_plan_create_tuned(p, cp, cs, rho, nullptr, out);
}

ela3d_status ela3d_select_device(int32_t ordinal) {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess) return status_from_cuda(e, "cudaGetDeviceCount");
  if (ordinal < 0 || ordinal >= n) {
    set_last_error("device ordinal out of range");
    return ELA3D_ERR_INVALID_ARG;
  }
  return status_from_cuda(cudaSetDevice(ordinal), "cudaSetDevice");
}

ela3d_status ela3d_host_alloc(size_t bytes, void **out) {
  if (!out || bytes == 0) return ELA3D_ERR_INVALID_ARG;
  *out = nullptr;
  return status_from_cuda(cudaHostAlloc(out, bytes, cudaHostAllocDefault), "cudaHostAlloc");
}

ela3d_status ela3d_host_free(void *ptr) {
  if (!ptr) return ELA3D_OK;
  return status_from_cuda(cudaFreeHost(ptr), "cudaFreeHost");
}

ela3d_status ela3d_run_timed(ela3d_plan *plan, int32_t nsteps, double *ms) {
  if (!plan || nsteps < 0) return ELA3D_ERR_INVALID_ARG;
  return plan->eng->run_timed(nsteps, ms);
}

ela3d_status ela3d_enqueue(ela3d_plan *plan, int32_t nsteps) {
  if (!plan) return ELA3D_ERR_INVALID_ARG;
  return plan->eng->enqueue(nsteps);
}

ela3d_status ela3d_sync(ela3d_plan *plan) {
  if (!plan) return ELA3D_ERR_INVALID_ARG;
  return plan->eng->sync();
}

ela3d_status ela3d_run(ela3d_plan *plan, int32_t nsteps) {
  if (!plan) return ELA3D_ERR_INVALID_ARG;
  if (nsteps < 0) return ELA3D_ERR_INVALID_ARG;
  const int every = plan->p.energy_every;
  if (every <= 0) {
    ela3d_status st = plan->eng->enqueue(nsteps);
    if (st != ELA3D_OK) return st;
    return plan->eng->sync();
  }
  int left = nsteps;
  while (left > 0) {
    const int done = plan->eng->steps_done();
    const int chunk = std::min(left, every - done % every);
    ela3d_status st = plan->eng->enqueue(chunk);
    if (st == ELA3D_OK) st = plan->eng->sync();
    if (st != ELA3D_OK) return st;
    left -= chunk;
    if (plan->eng->steps_done() % every == 0) {
      st = engine_check_energy(plan->eng.get(), 0, plan->fp64);
      if (st != ELA3D_OK) return st;
    }
  }
  return ELA3D_OK;
}

ela3d_status ela3d_get_seismograms(ela3d_plan *plan, float *out) {
  if (!plan || !out) return ELA3D_ERR_INVALID_ARG;
  return plan->eng->seismograms(0, out, 0);
}

ela3d_status ela3d_get_seismograms_f64(ela3d_plan *plan, double *out) {
  if (!plan || !out) return ELA3D_ERR_INVALID_ARG;
  return plan->eng->seismograms(0, out, 1);
}

ela3d_status ela3d_checkpoint_size(ela3d_plan *plan, int64_t *bytes) {
  if (!plan || !bytes) return ELA3D_ERR_INVALID_ARG;
  *bytes = plan->eng->checkpoint_bytes();
  return *bytes > 0 ? ELA3D_OK : ELA3D_ERR_INVALID_ARG;
}

ela3d_status ela3d_checkpoint_save(ela3d_plan *plan, void *buf, int64_t bytes) {
  if (!plan || !buf) return ELA3D_ERR_INVALID_ARG;
  return plan->eng->checkpoint_save(buf, bytes);
}

ela3d_status ela3d_checkpoint_load(ela3d_plan *plan, const void *buf, int64_t bytes) {
  if (!plan || !buf) return ELA3D_ERR_INVALID_ARG;
  return plan->eng->checkpoint_load(buf, bytes);
}

ela3d_status ela3d_get_source_trace(ela3d_plan *plan, float *out) {
  if (!plan || !out) return ELA3D_ERR_INVALID_ARG;
  return plan->eng->source_trace(0, out, 0);
}

ela3d_status ela3d_get_source_trace_f64(ela3d_plan *plan, double *out) {
  if (!plan || !out) return ELA3D_ERR_INVALID_ARG;
  return plan->eng->source_trace(0, out, 1);
}

ela3d_status ela3d_get_field(ela3d_plan *plan, int32_t comp, float *out) {
  if (!plan || !out) return ELA3D_ERR_INVALID_ARG;
  return plan->eng->field(0, comp, out, 0);
}

ela3d_status ela3d_get_field_f64(ela3d_plan *plan, int32_t comp, double *out) {
  if (!plan || !out) return ELA3D_ERR_INVALID_ARG;
  return plan->eng->field(0, comp, out, 1);
}

ela3d_status ela3d_energy(ela3d_plan *plan, double *out) {
  if (!plan || !out) return ELA3D_ERR_INVALID_ARG;
  return plan->eng->energy(0, out);
}

ela3d_status ela3d_plan_info_get(ela3d_plan *plan, ela3d_plan_info *out) {
  if (!plan || !out) return ELA3D_ERR_INVALID_ARG;
  return plan->eng->info(0, out);
}

ela3d_status ela3d_set_kernel_timing(ela3d_plan *plan, int32_t enable) {
  if (!plan) return ELA3D_ERR_INVALID_ARG;
  return plan->eng->set_timing(enable != 0);
}

ela3d_status ela3d_get_kernel_timing(ela3d_plan *plan, double *stress_ms, double *velocity_ms,
                                     int64_t *stress_launches, int64_t *velocity_launches) {
  if (!plan) return ELA3D_ERR_INVALID_ARG;
  return plan->eng->timing(stress_ms, velocity_ms, stress_launches, velocity_launches);
}

ela3d_status ela3d_get_flow_timing(ela3d_plan *plan, double *ms, int64_t *launches, int64_t *steps) {
  if (!plan) return ELA3D_ERR_INVALID_ARG;
  return plan->eng->flow_timing(ms, launches, steps);
}

ela3d_status ela3d_plan_check_guards(ela3d_plan *plan) {
  if (!plan) return ELA3D_ERR_INVALID_ARG;
  return plan->eng->check_guards();
}

ela3d_status ela3d_plan_get_profiles(ela3d_plan *plan, int32_t axis, double *out) {
  if (!plan) return ELA3D_ERR_INVALID_ARG;
  return plan->eng->profiles(0, axis, out);
}

ela3d_status ela3d_plan_poison_padding(ela3d_plan *plan, double value) {
  if (!plan) return ELA3D_ERR_INVALID_ARG;
  return plan->eng->poison_padding(value);
}

ela3d_status ela3d_plan_inject_timeout(ela3d_plan *plan, int32_t launches) {
  if (!plan) return ELA3D_ERR_INVALID_ARG;
  return plan->eng->inject_timeout(launches);
}

ela3d_status ela3d_plan_destroy(ela3d_plan *plan) {
  delete plan;
  return ELA3D_OK;
}

ela3d_status ela3d_slab_extent(const double *a_full, const double *a_half, int32_t n, int32_t *lo, int32_t *hi) {
  if (!a_full || !a_half || n < 1 || !lo || !hi) return ELA3D_ERR_INVALID_ARG;
  int l = 0, h = 0;
  slab_extent(a_full, a_half, n, &l, &h);
  *lo = l;
  *hi = h;
  return ELA3D_OK;
}

ela3d_status ela3d_builtin_tuning(const ela3d_params *p, ela3d_tuning *out) {
  if (!p || !out) return ELA3D_ERR_INVALID_ARG;
  const TuneChoice c = default_choice(p->precision == ELA3D_FP64, p->nx, p->ny, p->nz,
                                      p->src_kind == ELA3D_SRC_EXPLOSIVE);
  out->variant = c.variant;
  out->schedule = c.kind;
  out->chunk = c.chunk;
  out->blocks_per_sm = c.blocks_per_sm;
  out->prefetch = c.prefetch;
  out->lag = c.lag;
  return ELA3D_OK;
}

ela3d_status ela3d_flow_schedule_build(int32_t nx, int32_t ny, int32_t nz, int32_t tile_x, int32_t tile_y,
                                       int32_t chunk, int32_t gap, int32_t overlap, int32_t nsteps,
                                       int32_t *nitems, int32_t *items) {
  if (nx < 1 || ny < 1 || nz < 1 || !nitems) return ELA3D_ERR_INVALID_ARG;
  std::vector<FlowItem> it;
  std::vector<int> off, nch;
  int nflags = 0;
  std::string why;
  if (!build_flow_schedule({FlowShape{nx, ny, nz, 0}}, tile_x, tile_y, chunk, gap, overlap != 0, nsteps, &it, &off,
                           &nch, &nflags, &why)) {
    set_last_error(why);
    return ELA3D_ERR_INVALID_ARG;
  }
  if (items) {
    if (*nitems < (int32_t)it.size()) return ELA3D_ERR_INVALID_ARG;
    for (size_t q = 0; q < it.size(); ++q) {
      int32_t *o = items + 6 * q;
      o[0] = it[q].kind; o[1] = it[q].step; o[2] = it[q].chunk;
      o[3] = it[q].it.tile; o[4] = it[q].it.k0; o[5] = it[q].it.k1;
    }
  }
  *nitems = (int32_t)it.size();
  return ELA3D_OK;
}

ela3d_status ela3d_schedule_build(int32_t nx, int32_t ny, int32_t nz, int32_t tile_x, int32_t tile_y,
                                  int32_t schedule, int32_t chunk, int32_t max_blocks, int32_t *nitems,
                                  int32_t *nblocks, int32_t *items, int32_t *block_first) {
  if (nx < 1 || ny < 1 || nz < 1 || tile_x < 1 || tile_y < 1 || max_blocks < 1 || !nitems || !nblocks)
    return ELA3D_ERR_INVALID_ARG;
  std::vector<Item> it;
  std::vector<int2> rg;
  build_schedule({ShotShape{nx, ny, nz}}, tile_x, tile_y, schedule, chunk, max_blocks, &it, &rg);
  if (items) {
    if (*nitems < (int32_t)it.size()) return ELA3D_ERR_INVALID_ARG;
    for (size_t q = 0; q < it.size(); ++q) {
      items[3 * q] = it[q].tile;
      items[3 * q + 1] = it[q].k0;
      items[3 * q + 2] = it[q].k1;
    }
  }
  if (block_first) {
    if (*nblocks < (int32_t)rg.size()) return ELA3D_ERR_INVALID_ARG;
    for (size_t b = 0; b < rg.size(); ++b) block_first[b] = rg[b].x;
    block_first[rg.size()] = rg.empty() ? 0 : rg.back().y;
  }
  *nitems = (int32_t)it.size();
  *nblocks = (int32_t)rg.size();
  return ELA3D_OK;
}

ela3d_status ela3d_batch_create(int32_t nshots, const ela3d_params *params, const float *const *cp,
                                const float *const *cs, const float *const *rho, const ela3d_tuning *tune,
                                ela3d_batch **out) {
  if (!out || nshots < 1 || !params || !cp || !cs || !rho) return ELA3D_ERR_INVALID_ARG;
  *out = nullptr;
  for (int i = 0; i < nshots; ++i) {
    ela3d_status st = validate_params(params[i]);
    if (st != ELA3D_OK) {
      set_last_error("shot " + std::to_string(i) + ": " + last_error());
      return st;
    }
    if (params[i].precision != params[0].precision) {
      set_last_error("all shots of a batch need the same precision");
      return ELA3D_ERR_INVALID_ARG;
    }
    if (!cp[i] || !cs[i] || !rho[i]) {
      set_last_error("model arrays missing");
      return ELA3D_ERR_INVALID_ARG;
    }
  }
  if (validate_tuning(tune, params[0].precision) != ELA3D_OK) return ELA3D_ERR_INVALID_ARG;
  ela3d_batch *b = new (std::nothrow) ela3d_batch();
  if (!b) return ELA3D_ERR_OOM;
  b->fp64 = params[0].precision == ELA3D_FP64;
  ela3d_status st;
  b->eng = make_engine(b->fp64, &st);
  for (int i = 0; i < nshots && st == ELA3D_OK; ++i) {
    int share = -1;
    for (int j = 0; j < i && share < 0; ++j)
      if (cp[j] == cp[i] && cs[j] == cs[i] && rho[j] == rho[i] && params[j].nx == params[i].nx &&
          params[j].ny == params[i].ny && params[j].nz == params[i].nz)
        share = j;
    st = b->eng->add_shot(params[i], cp[i], cs[i], rho[i], share);
  }
  if (st == ELA3D_OK) {
    b->eng->set_retire(true);
    const TuneChoice c = resolve_tuning(std::vector<ela3d_params>(params, params + nshots), cp, cs, rho, tune);
    st = b->eng->finalize(&c);
  }
  if (st != ELA3D_OK) {
    delete b;
    return st;
  }
  *out = b;
  return ELA3D_OK;
}

ela3d_status ela3d_batch_run(ela3d_batch *b, int32_t nsteps) {
  if (!b || nsteps < 0) return ELA3D_ERR_INVALID_ARG;
  ela3d_status st = b->eng->enqueue(nsteps);
  if (st != ELA3D_OK) return st;
  return b->eng->sync();
}

ela3d_status ela3d_batch_run_timed(ela3d_batch *b, int32_t nsteps, double *ms) {
  if (!b || nsteps < 0) return ELA3D_ERR_INVALID_ARG;
  return b->eng->run_timed(nsteps, ms);
}

ela3d_status ela3d_batch_get_seismograms(ela3d_batch *b, int32_t shot, float *out) {
  if (!b || !out) return ELA3D_ERR_INVALID_ARG;
  return b->eng->seismograms(shot, out, 0);
}

ela3d_status ela3d_batch_get_source_trace(ela3d_batch *b, int32_t shot, float *out) {
  if (!b || !out) return ELA3D_ERR_INVALID_ARG;
  return b->eng->source_trace(shot, out, 0);
}

ela3d_status ela3d_batch_get_field(ela3d_batch *b, int32_t shot, int32_t comp, float *out) {
  if (!b || !out) return ELA3D_ERR_INVALID_ARG;
  return b->eng->field(shot, comp, out, 0);
}

ela3d_status ela3d_batch_info(ela3d_batch *b, int32_t shot, ela3d_plan_info *out) {
  if (!b || !out) return ELA3D_ERR_INVALID_ARG;
  return b->eng->info(shot, out);
}

ela3d_status ela3d_batch_destroy(ela3d_batch *b) {
  delete b;
  return ELA3D_OK;
}

}  // extern "C"
