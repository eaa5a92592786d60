// ela3d_server.cu -- continuous-batching request loop (ela3d_server_* in
// include/ela3d.h).  No counterpart in the reference, which runs one shot
// per process.
//
// A worker thread owns one engine (the batched kernels).  Each round it
//  1. enqueues up to `steps_per_round` time steps of every running shot in
//     one launch pair per step (shots that reach their nstep inside the
//     round stop there);
//  2. while the device works, admits queued requests in arrival order while
//     their device footprint fits the budget, a slot is free and the
//     running shots hold fewer cells than the fill target (a request larger
//     than the whole budget is refused with ELA3D_ERR_BUSY); their uploads
//     run on the engine's setup stream, and they join at the next round;
//  3. copies each running shot's new seismogram samples to its host buffer
//     (clients read them while the shot runs);
//  4. retires finished and cancelled shots, which frees their memory for
//     later admissions.
// Requests that arrive while others run join at the next round boundary,
// so their work overlaps on the device with the shots already running.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "ela3d_engine.h"

using namespace ela3d;

namespace {

// Running cells at which the batched kernels fill the GPU (a 256^3 shot
// alone streams at 0.9 of the HBM roofline): below it the worker keeps
// admitting queued requests before it waits for the device.
constexpr double kFullCells = 16.0 * 1024 * 1024;

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

enum ReqState { RQ_QUEUED = 0, RQ_RUNNING = 1, RQ_DONE = 2, RQ_FAILED = 3, RQ_CANCELLED = 4 };

struct Request {
  uint64_t ticket = 0;
  ela3d_params p{};
  std::vector<int32_t> rec;
  std::vector<float> cp, cs, rho;  // host copies until admitted
  bool generated = false;          // model generated on the device instead
  ModelSpec spec{};
  int64_t footprint = 0;
  int state = RQ_QUEUED;
  ela3d_status error = ELA3D_OK;
  std::string message;             // the worker's error text for a failed request
  uint64_t key = 0;                // engine shot while running
  int nsamp = 0, samples_ready = 0;
  std::vector<float> seis;         // [nrec][3][nsamp]
  double t_submit = 0, t_admit = 0, t_done = 0;
  bool cancel = false;
  ela3d_request_callback on_done = nullptr;  // called once when the request ends
  void *on_done_user = nullptr;
};

struct Callback {
  ela3d_request_callback fn;
  uint64_t ticket;
  ela3d_status status;
  void *user;
};

}  // namespace

struct ela3d_server {
  ela3d_server_config cfg{};
  int device = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done, cv_idle;
  int waiters = 0;          // threads inside ela3d_server_wait
  std::deque<uint64_t> queue;
  std::map<uint64_t, std::unique_ptr<Request>> reqs;
  std::vector<uint64_t> running;
  std::unique_ptr<EngineBase> eng;
  int64_t budget = 0, used = 0;
  uint64_t next_ticket = 1;
  bool stop = false;
  std::thread worker;
  // statistics
  int64_t n_submitted = 0, n_completed = 0, n_failed = 0, n_cancelled = 0, rounds = 0;
  double cell_updates = 0, busy_s = 0, t_first = 0, t_last = 0;
  std::vector<double> latencies;
  ela3d_status fatal = ELA3D_OK;
  std::vector<Callback> callbacks;   // due, to be called without the lock

  void finish(Request &r, int state, ela3d_status err) {
    r.state = state;
    r.error = err;
    // (error texts are per thread: keep the worker's for the client)
    if (state == RQ_FAILED) r.message = err == ELA3D_ERR_BUSY ? "request larger than the server's device budget"
                                                                : std::string(last_error());
    r.t_done = now_s();
    r.cp.clear(); r.cp.shrink_to_fit();
    r.cs.clear(); r.cs.shrink_to_fit();
    r.rho.clear(); r.rho.shrink_to_fit();
    if (r.on_done) {
      callbacks.push_back({r.on_done, r.ticket, state == RQ_DONE ? ELA3D_OK : err, r.on_done_user});
      r.on_done = nullptr;
    }
    if (state == RQ_DONE) {
      ++n_completed;
      latencies.push_back(r.t_done - r.t_submit);
      cell_updates += (double)r.p.nx * r.p.ny * r.p.nz * r.p.nstep;
      t_last = r.t_done;
    } else if (state == RQ_CANCELLED) {
      ++n_cancelled;
    } else {
      ++n_failed;
    }
  }

  // Calls the due completion callbacks; the lock must not be held (a
  // callback may call back into the server).
  void run_callbacks() {
    std::vector<Callback> due;
    {
      std::lock_guard<std::mutex> g(mu);
      due.swap(callbacks);
    }
    for (const Callback &c : due) c.fn(c.ticket, c.status, c.user);
  }

  // Cells the running shots hold.  Called with the lock held (clients add
  // to and remove from `reqs`).
  double running_cells() const {
    double c = 0.0;
    for (uint64_t t : running) {
      const ela3d_params &q = reqs.at(t)->p;
      c += (double)q.nx * q.ny * q.nz;
    }
    return c;
  }

  // The next request to admit, in arrival order, taken off the queue (with
  // its device bytes booked), or null when the front request must wait for
  // memory, a slot or the fill target.  Cancelled and oversize requests at
  // the front are finished on the way.  Called with the lock held.
  Request *take_admissible() {
    while (!queue.empty()) {
      Request &r = *reqs[queue.front()];
      if (r.cancel) {
        queue.pop_front();
        finish(r, RQ_CANCELLED, ELA3D_ERR_CANCELLED);
        cv_done.notify_all();
        continue;
      }
      if (r.footprint > budget) {
        queue.pop_front();
        finish(r, RQ_FAILED, ELA3D_ERR_BUSY);
        cv_done.notify_all();
        continue;
      }
      const double active_cells = running_cells();
      const bool slot = cfg.max_active <= 0 || (int)running.size() < cfg.max_active;
      const bool fill = cfg.fill_cells <= 0 || active_cells < (double)cfg.fill_cells;
      if (!slot || !fill || used + r.footprint > budget) return nullptr;
      queue.pop_front();
      used += r.footprint;
      return &r;
    }
    return nullptr;
  }

  void loop() {
    cudaSetDevice(device);
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEventCreate(&ev0);
    cudaEventCreate(&ev1);
    std::unique_lock<std::mutex> lk(mu);
    while (true) {
      cv_work.wait(lk, [&] { return stop || !queue.empty() || !running.empty(); });
      if (stop) break;
      // cancellations of running shots take effect at this round boundary
      std::vector<Request *> cancelled;
      for (uint64_t t : running)
        if (reqs[t]->cancel) cancelled.push_back(reqs[t].get());
      if (!cancelled.empty()) {
        lk.unlock();
        for (Request *r : cancelled) eng->remove_shot(r->key);
        lk.lock();
        for (Request *r : cancelled) {
          used -= r->footprint;
          running.erase(std::remove(running.begin(), running.end(), r->ticket), running.end());
          finish(*r, RQ_CANCELLED, ELA3D_ERR_CANCELLED);
        }
        cv_done.notify_all();
      }
      // this round: the shots running now, up to the configured number of
      // steps, no further than the longest remaining shot
      std::vector<uint64_t> run_now = running;
      int round = 0;
      if (!run_now.empty()) {
        int longest = 0;
        for (uint64_t t : run_now) {
          const Request &r = *reqs[t];
          longest = std::max(longest, r.p.nstep - std::max(0, eng->shot_steps(r.key)));
        }
        round = std::max(1, std::min(std::max(1, cfg.steps_per_round), longest));
      }
      lk.unlock();

      ela3d_status st = ELA3D_OK;
      if (round > 0) {
        cudaEventRecord(ev0, eng->stream());
        st = eng->enqueue(round);
        cudaEventRecord(ev1, eng->stream());
      }
      // admissions, in arrival order, while the device runs the round (a
      // joining shot is prepared on its own stream and takes part from the
      // next round on); once the round has finished, the rest wait for the
      // next boundary.  With nothing running, the first admission starts
      // the device and the others join while it works.
      for (bool any = false;;) {
        double cells_now = 0.0;   // held by the running shots after this admission
        Request *r = nullptr;
        {
          std::lock_guard<std::mutex> g(mu);
          r = take_admissible();
        }
        if (!r) break;
        ela3d_params p = r->p;
        p.rec = r->rec.data();
        const ela3d_status sa = r->generated ? eng->add_shot(p, nullptr, nullptr, nullptr, -1, &r->spec)
                                             : eng->add_shot(p, r->cp.data(), r->cs.data(), r->rho.data(), -1);
        {
          std::lock_guard<std::mutex> g(mu);
          if (sa != ELA3D_OK) {
            used -= r->footprint;
            finish(*r, RQ_FAILED, sa);
          } else {
            r->key = eng->last_key();
            r->state = RQ_RUNNING;
            r->t_admit = now_s();
            r->cp.clear(); r->cp.shrink_to_fit();
            r->cs.clear(); r->cs.shrink_to_fit();
            r->rho.clear(); r->rho.shrink_to_fit();
            running.push_back(r->ticket);
            any = true;
          }
          cells_now = running_cells();
          cv_done.notify_all();
        }
        // stop admitting for this round once the device has finished it --
        // unless the running shots are still too few to fill it, in which
        // case the next round would be small anyway
        if ((round > 0 ? eng->idle() : any) && cells_now >= kFullCells) break;
      }
      run_callbacks();
      if (round == 0) {
        lk.lock();
        continue;
      }

      if (st == ELA3D_OK) st = eng->sync();
      float round_ms = 0.0f;
      if (st == ELA3D_OK) cudaEventElapsedTime(&round_ms, ev0, ev1);
      // stream new samples of the shots that ran
      struct Chunk { Request *r; int from, to, steps; std::vector<float> data; ela3d_status st; };
      std::vector<Chunk> chunks;
      for (uint64_t t : run_now) {
        Request *r = nullptr;
        {
          std::lock_guard<std::mutex> g(mu);
          r = reqs[t].get();
        }
        const int steps = eng->shot_steps(r->key);
        const int ready = std::min(r->nsamp, steps / std::max(1, r->p.sampgat));
        Chunk c{r, r->samples_ready, ready, steps, {}, ELA3D_OK};
        if (st == ELA3D_OK && ready > c.from) {
          c.data.resize((size_t)r->p.nrec * 3 * (ready - c.from));
          c.st = eng->read_samples(r->key, c.from, ready, c.data.data());
        }
        if (st != ELA3D_OK || c.st != ELA3D_OK || steps >= r->p.nstep) eng->remove_shot(r->key);
        chunks.push_back(std::move(c));
      }

      lk.lock();
      busy_s += round_ms / 1e3;
      ++rounds;
      for (Chunk &c : chunks) {
        Request &r = *c.r;
        const int n = c.to - c.from;
        if (n > 0 && !c.data.empty()) {
          for (int row = 0; row < r.p.nrec * 3; ++row)
            std::memcpy(&r.seis[(size_t)row * r.nsamp + c.from], &c.data[(size_t)row * n], n * sizeof(float));
          r.samples_ready = c.to;
        }
        const bool failed = st != ELA3D_OK || c.st != ELA3D_OK;
        if (failed || c.steps >= r.p.nstep) {
          used -= r.footprint;
          running.erase(std::remove(running.begin(), running.end(), r.ticket), running.end());
          finish(r, failed ? RQ_FAILED : RQ_DONE, failed ? (st != ELA3D_OK ? st : c.st) : ELA3D_OK);
        }
      }
      if (st != ELA3D_OK) fatal = st;
      cv_done.notify_all();
      lk.unlock();
      run_callbacks();
      lk.lock();
    }
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
  }
};

extern "C" {

ela3d_status ela3d_server_config_default(ela3d_server_config *c) {
  if (!c) return ELA3D_ERR_INVALID_ARG;
  *c = ela3d_server_config{};
  c->hbm_budget_bytes = 0;
  c->max_active = 0;
  c->fill_cells = 0;
  c->steps_per_round = 50;
  c->precision = ELA3D_FP32;
  c->tune.variant = -1;
  c->tune.schedule = -1;
  c->tune.chunk = 0;
  c->tune.blocks_per_sm = -1;
  c->tune.prefetch = -1;
  c->tune.lag = -1;
  return ELA3D_OK;
}

ela3d_status ela3d_server_create(const ela3d_server_config *cfg, ela3d_server **out) {
  if (!cfg || !out) return ELA3D_ERR_INVALID_ARG;
  *out = nullptr;
  if (cfg->precision != ELA3D_FP32 && cfg->precision != ELA3D_FP64) return ELA3D_ERR_INVALID_ARG;
  if (validate_tuning(&cfg->tune, cfg->precision) != ELA3D_OK) return ELA3D_ERR_INVALID_ARG;
  ela3d_server *s = new (std::nothrow) ela3d_server();
  if (!s) return ELA3D_ERR_OOM;
  s->cfg = *cfg;
  ela3d_status st = status_from_cuda(cudaGetDevice(&s->device), "cudaGetDevice");
  if (st == ELA3D_OK) s->eng = make_engine(cfg->precision == ELA3D_FP64, &st);
  if (st == ELA3D_OK) {
    size_t fr = 0, tot = 0;
    st = status_from_cuda(cudaMemGetInfo(&fr, &tot), "cudaMemGetInfo");
    s->budget = cfg->hbm_budget_bytes > 0 ? cfg->hbm_budget_bytes : (int64_t)(0.8 * (double)fr);
  }
  if (st == ELA3D_OK) {
    ela3d_params probe{};
    ela3d_params_default(&probe);
    probe.precision = cfg->precision;
    TuneChoice c = default_choice(cfg->precision == ELA3D_FP64, 0, 0, 0);
    if (cfg->tune.variant >= 0) c.variant = cfg->tune.variant;
    if (cfg->tune.schedule >= 0) c.kind = cfg->tune.schedule;
    if (cfg->tune.chunk > 0) c.chunk = cfg->tune.chunk;
    if (cfg->tune.blocks_per_sm >= 0) c.blocks_per_sm = cfg->tune.blocks_per_sm;
    if (cfg->tune.prefetch >= 0) c.prefetch = cfg->tune.prefetch & (CTL_PF_X | CTL_PF_YZ);
    if (cfg->tune.lag >= 0) c.lag = cfg->tune.lag;
    s->eng->set_retire(true);
    st = s->eng->finalize(&c);
  }
  if (st != ELA3D_OK) {
    delete s;
    return st;
  }
  s->worker = std::thread([s] { s->loop(); });
  *out = s;
  return ELA3D_OK;
}

static ela3d_status submit_common(ela3d_server *s, std::unique_ptr<Request> r, uint64_t *ticket) {
  std::lock_guard<std::mutex> g(s->mu);
  if (s->fatal != ELA3D_OK) return s->fatal;
  r->ticket = s->next_ticket++;
  if (s->n_submitted == 0) s->t_first = r->t_submit;
  ++s->n_submitted;
  *ticket = r->ticket;
  s->queue.push_back(r->ticket);
  s->reqs[r->ticket] = std::move(r);
  s->cv_work.notify_all();
  return ELA3D_OK;
}

ela3d_status ela3d_server_submit_model(ela3d_server *s, const ela3d_params *p, const ela3d_model_spec *model,
                                       uint64_t *ticket) {
  if (!s || !p || !model || !ticket) return ELA3D_ERR_INVALID_ARG;
  ela3d_status st = validate_params(*p);
  if (st != ELA3D_OK) return st;
  if (p->precision != s->cfg.precision) {
    set_last_error("request precision differs from the server's");
    return ELA3D_ERR_INVALID_ARG;
  }
  auto r = std::make_unique<Request>();
  r->p = *p;
  r->rec.assign(p->rec, p->rec + 3 * (size_t)p->nrec);
  r->p.rec = nullptr;
  r->generated = true;
  std::memcpy(&r->spec, model, sizeof(ModelSpec));
  r->footprint = s->eng->footprint(*p);
  r->nsamp = p->nstep / p->sampgat;
  r->seis.assign((size_t)p->nrec * 3 * r->nsamp, 0.0f);
  r->t_submit = now_s();
  return submit_common(s, std::move(r), ticket);
}

ela3d_status ela3d_server_submit(ela3d_server *s, const ela3d_params *p, const float *cp, const float *cs,
                                 const float *rho, uint64_t *ticket) {
  if (!s || !p || !ticket) return ELA3D_ERR_INVALID_ARG;
  ela3d_status st = validate_params(*p);
  if (st != ELA3D_OK) return st;
  if (p->precision != s->cfg.precision) {
    set_last_error("request precision differs from the server's");
    return ELA3D_ERR_INVALID_ARG;
  }
  if (!cp || !cs || !rho) {
    set_last_error("model arrays missing");
    return ELA3D_ERR_INVALID_ARG;
  }
  auto r = std::make_unique<Request>();
  r->p = *p;
  r->rec.assign(p->rec, p->rec + 3 * (size_t)p->nrec);
  r->p.rec = nullptr;
  const size_t n = (size_t)p->nx * p->ny * p->nz;
  r->cp.assign(cp, cp + n);
  r->cs.assign(cs, cs + n);
  r->rho.assign(rho, rho + n);
  r->footprint = s->eng->footprint(*p);
  r->nsamp = p->nstep / p->sampgat;
  r->seis.assign((size_t)p->nrec * 3 * r->nsamp, 0.0f);
  r->t_submit = now_s();
  return submit_common(s, std::move(r), ticket);
}

ela3d_status ela3d_server_poll(ela3d_server *s, uint64_t ticket, int32_t *state, int32_t *samples_ready) {
  if (!s) return ELA3D_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> g(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return ELA3D_ERR_NOT_FOUND;
  if (state) *state = it->second->state;
  if (samples_ready) *samples_ready = it->second->samples_ready;
  if (it->second->state != RQ_FAILED) return ELA3D_OK;
  set_last_error(it->second->message);
  return it->second->error;
}

ela3d_status ela3d_server_read(ela3d_server *s, uint64_t ticket, int32_t first, int32_t count, float *out) {
  if (!s || !out || first < 0 || count < 0) return ELA3D_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> g(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return ELA3D_ERR_NOT_FOUND;
  const Request &r = *it->second;
  if (first + count > r.samples_ready) return ELA3D_ERR_NOT_READY;
  for (int row = 0; row < r.p.nrec * 3; ++row)
    std::memcpy(out + (size_t)row * count, &r.seis[(size_t)row * r.nsamp + first], count * sizeof(float));
  return ELA3D_OK;
}

ela3d_status ela3d_server_wait(ela3d_server *s, uint64_t ticket, int32_t timeout_ms) {
  if (!s) return ELA3D_ERR_INVALID_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  // counted, so that ela3d_server_destroy can let every waiter leave first
  struct Count {
    ela3d_server *s;
    explicit Count(ela3d_server *q) : s(q) { ++s->waiters; }
    ~Count() {
      if (--s->waiters == 0) s->cv_idle.notify_all();
    }
  } count(s);
  auto done = [&] {
    auto it = s->reqs.find(ticket);
    return it == s->reqs.end() || it->second->state >= RQ_DONE;
  };
  if (timeout_ms < 0) s->cv_done.wait(lk, done);
  else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), done)) return ELA3D_ERR_NOT_READY;
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return ELA3D_ERR_NOT_FOUND;
  if (it->second->state == RQ_DONE) return ELA3D_OK;
  if (it->second->state == RQ_FAILED) set_last_error(it->second->message);
  return it->second->error != ELA3D_OK ? it->second->error : ELA3D_ERR_CANCELLED;
}

ela3d_status ela3d_server_cancel(ela3d_server *s, uint64_t ticket) {
  if (!s) return ELA3D_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> g(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return ELA3D_ERR_NOT_FOUND;
  if (it->second->state <= RQ_RUNNING) it->second->cancel = true;
  s->cv_work.notify_all();
  return ELA3D_OK;
}

ela3d_status ela3d_server_on_done(ela3d_server *s, uint64_t ticket, ela3d_request_callback cb, void *user) {
  if (!s || !cb) return ELA3D_ERR_INVALID_ARG;
  Callback now{nullptr, ticket, ELA3D_OK, user};
  {
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return ELA3D_ERR_NOT_FOUND;
    Request &r = *it->second;
    if (r.state < RQ_DONE) {
      r.on_done = cb;
      r.on_done_user = user;
      return ELA3D_OK;
    }
    now.fn = cb;   // already over: called right here, on this thread
    now.status = r.state == RQ_DONE ? ELA3D_OK : (r.error != ELA3D_OK ? r.error : ELA3D_ERR_CANCELLED);
  }
  now.fn(now.ticket, now.status, now.user);
  return ELA3D_OK;
}

ela3d_status ela3d_server_release(ela3d_server *s, uint64_t ticket) {
  if (!s) return ELA3D_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> g(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return ELA3D_ERR_NOT_FOUND;
  if (it->second->state < RQ_DONE) return ELA3D_ERR_BUSY;
  s->reqs.erase(it);
  return ELA3D_OK;
}

ela3d_status ela3d_server_stats_get(ela3d_server *s, ela3d_server_stats *o) {
  if (!s || !o) return ELA3D_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> g(s->mu);
  *o = ela3d_server_stats{};
  o->submitted = s->n_submitted;
  o->completed = s->n_completed;
  o->failed = s->n_failed;
  o->cancelled = s->n_cancelled;
  o->queued = (int64_t)s->queue.size();
  o->running = (int64_t)s->running.size();
  o->rounds = s->rounds;
  o->cell_updates = s->cell_updates;
  o->busy_seconds = s->busy_s;
  o->wall_seconds = s->n_completed ? s->t_last - s->t_first : 0.0;
  o->device_bytes_in_use = s->used;
  o->device_bytes_budget = s->budget;
  if (!s->latencies.empty()) {
    std::vector<double> l = s->latencies;
    std::sort(l.begin(), l.end());
    auto pct = [&](double q) {
      const double pos = q * (double)(l.size() - 1);
      const size_t i = (size_t)pos;
      const double f = pos - (double)i;
      return i + 1 < l.size() ? l[i] * (1 - f) + l[i + 1] * f : l[i];
    };
    o->latency_p50_s = pct(0.50);
    o->latency_p99_s = pct(0.99);
    o->latency_max_s = l.back();
  }
  return ELA3D_OK;
}

ela3d_status ela3d_server_destroy(ela3d_server *s) {
  if (!s) return ELA3D_OK;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stop = true;
    s->cv_work.notify_all();
  }
  if (s->worker.joinable()) s->worker.join();
  {
    // unfinished requests end as cancelled; threads waiting on them return
    // ELA3D_ERR_CANCELLED before the server's memory goes away
    std::unique_lock<std::mutex> lk(s->mu);
    for (auto &kv : s->reqs)
      if (kv.second->state < RQ_DONE) s->finish(*kv.second, RQ_CANCELLED, ELA3D_ERR_CANCELLED);
    s->cv_done.notify_all();
    s->cv_idle.wait(lk, [&] { return s->waiters == 0; });
  }
  s->run_callbacks();
  delete s;
  return ELA3D_OK;
}

}  // extern "C"
