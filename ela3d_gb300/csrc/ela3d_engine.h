// ela3d_engine.h -- host engine: a set of shots resident on one GPU,
// advanced together by the two stencil kernels (one launch per half-step).
// A single-shot plan is an engine with one shot; the batch and the server
// build on the same class.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <memory>
#include <string>
#include <vector>

#include "../../include/ela3d.h"
#include "ela3d_internal.h"

namespace ela3d {

void set_last_error(const std::string &msg);
const char *last_error();
ela3d_status status_from_cuda(cudaError_t e, const char *what);

// Validates a parameter block (grid, spacing, source, receivers).
ela3d_status validate_params(const ela3d_params &p);
// A caller's tuning fields (null = all defaults) for shots of `precision`.
ela3d_status validate_tuning(const ela3d_tuning *t, int32_t precision);

// Slab extents of one axis from its profile arrays: cells [0, lo) and
// [hi, n) may have a != 0; every cell in [lo, hi) has a == 0 in both the
// full and the half profile.  Returns lo == hi == n when the layer covers
// everything.  (Host logic, unit-tested without a GPU.)
void slab_extent(const double *a_full, const double *a_half, int n, int *lo, int *hi);

// Work schedule.  Units are (shot, tile, plane); kind 0 gives every block a
// contiguous, equal share of the units in (shot, tile, plane) order; kind 1
// splits each tile column into z-chunks of `chunk` planes and deals the
// chunks round-robin in (shot, chunk, tile) order so that blocks running at
// the same time work on neighbouring tiles; kind 2 deals them in
// (chunk, tile, shot) order (same tile of many shots at once).
struct ShotShape {
  int nx, ny, nz;
  int id = -1;   // shot index written into the items (-1: position in the list)
  // C-PML slab bounds (cells x < xl or x >= xr lie in the x slab, ...);
  // only the schedule's cost estimate uses them (-1: no slabs)
  int xl = -1, xr = -1, yl = -1, yr = -1, zl = -1, zr = -1;
};
void build_schedule(const std::vector<ShotShape> &shots, int tx, int ty, int kind, int chunk,
                    int max_blocks, std::vector<Item> *items, std::vector<int2> *ranges);

// Dataflow schedules (kinds 3 and 4): the work items of `nsteps` time steps
// of the shots, for the dataflow kernel.  Each shot's planes are cut into
// z-chunks of `chunk` (>= 2) planes; stress chunk j covers [j*chunk,
// (j+1)*chunk), velocity chunk j the same range one plane lower (the first
// from 0, the last to nz).  Item dependencies: stress of tile t, chunk j,
// step r waits for velocity of chunks j, j+1 at step r-1 on t and its four
// neighbours; velocity waits for stress of chunks j-1, j at step r there.
// Order: a stress item of step 0 at its natural place (chunk by chunk,
// tile by tile), every other item `gap` places after the last item it
// waits for -- by default three rounds of the grid, so that it is claimed
// when those have finished (for grids near the L2 size, while their results
// are still in L2); stress items of a later step come after the whole
// previous step unless `overlap`.  The list is generated in tie order and
// sorted stably by key; 1 <= nsteps <= 255.  Every
// item is checked to follow the items it waits for, which is what makes
// the kernel's waits end.  flag_off[s] is shot s's offset into the
// completion counters ([2][chunks][tiles] ints each), *nflags their total.
// False (with *why) on bad arguments or a failed order check.
struct FlowShape {
  int nx, ny, nz;
  int id;   // shot index written into the items
};
bool build_flow_schedule(const std::vector<FlowShape> &shots, int tx, int ty, int chunk, int gap, bool overlap,
                         int nsteps, std::vector<FlowItem> *items, std::vector<int> *flag_off,
                         std::vector<int> *nchunks, int *nflags, std::string *why);

// A kernel variant, its work schedule and the memory-variable prefetch mode.
constexpr int kPrefetchDefault = CTL_PF_X | CTL_PF_YZ;
// Schedule kinds 0-2 launch the two half-step kernels once per step; kinds
// 3 and 4 run many steps per launch of the dataflow kernel (chunk planes
// per z-chunk, lag = the gap of build_flow_schedule, 0 = three rounds of
// the grid; kind 4 lets consecutive steps overlap).
constexpr int kScheduleFlow = 3;
constexpr int kScheduleFlowOverlap = 4;
struct TuneChoice {
  int variant;     // index into variants()
  int kind, chunk; // schedule
  int blocks_per_sm;  // 0 = occupancy limit
  int prefetch = kPrefetchDefault;  // CTL_PF_* bits
  int lag = 0;     // kinds 3, 4: gap in items (0 = three rounds of the grid)
};
// Built-in choice when the autotuner's cache has none for the workload.
TuneChoice default_choice(int fp64, int nx, int ny, int nz, bool explosive = false);

// Autotuner (ela3d_tune.cu): process-wide cache of measured best choices
// keyed by the workload shape.
bool tune_lookup(const std::vector<ela3d_params> &ps, TuneChoice *out);
void tune_store(const std::vector<ela3d_params> &ps, const TuneChoice &c);
ela3d_status autotune(const std::vector<ela3d_params> &ps, const std::vector<const float *> &cp,
                      const std::vector<const float *> &cs, const std::vector<const float *> &rho, int steps,
                      TuneChoice *best, double *best_ms, std::vector<std::pair<TuneChoice, double>> *table);

class EngineBase {
 public:
  virtual ~EngineBase() = default;
  // The model comes from host arrays (cp, cs, rho), from another shot
  // (shared_model_of >= 0), or from a generator run on the device (spec).
  virtual ela3d_status add_shot(const ela3d_params &p, const float *cp, const float *cs, const float *rho,
                                int shared_model_of, const ModelSpec *spec = nullptr) = 0;
  virtual ela3d_status finalize(const TuneChoice *choice) = 0;
  // A finalized engine switches to another schedule / prefetch mode of the
  // same kernel variant (the autotuner's inner loop).
  virtual ela3d_status retune(const TuneChoice &choice) = 0;
  virtual ela3d_status enqueue(int nsteps) = 0;
  // enqueue bracketed by events on the engine's stream; waits, returns ms
  virtual ela3d_status run_timed(int nsteps, double *ms) = 0;
  virtual ela3d_status sync() = 0;
  virtual ela3d_status seismograms(int shot, void *out, int out_fp64) = 0;
  virtual ela3d_status field(int shot, int comp, void *out, int out_fp64) = 0;
  virtual ela3d_status source_trace(int shot, void *out, int out_fp64) = 0;
  // Checkpoint of a single-shot engine: a header and the shot's whole device
  // pool (fields, model, C-PML memory variables, traces), restorable into an
  // engine created with the same parameters.
  virtual int64_t checkpoint_bytes() const = 0;
  virtual ela3d_status checkpoint_save(void *buf, int64_t bytes) = 0;
  virtual ela3d_status checkpoint_load(const void *buf, int64_t bytes) = 0;
  virtual ela3d_status energy(int shot, double *out) = 0;
  // The shot's C-PML profiles of one axis as stored on the device, in
  // double: a, b, 1/K, a_half, b_half, 1/K_half, n values each (test hook).
  virtual ela3d_status profiles(int shot, int axis, double *out) = 0;
  virtual ela3d_status info(int shot, ela3d_plan_info *out) = 0;
  virtual ela3d_status set_timing(bool on) = 0;
  virtual ela3d_status inject_timeout(int launches) = 0;
  virtual ela3d_status poison_padding(double value) = 0;
  virtual ela3d_status check_guards() = 0;
  virtual void set_retire(bool on) = 0;
  // live composition (serving): shots may join after finalize and leave
  virtual uint64_t last_key() const = 0;  // key of the most recently added shot
  virtual bool idle() const = 0;           // every enqueued launch has finished
  virtual ela3d_status remove_shot(uint64_t key) = 0;
  virtual int64_t footprint(const ela3d_params &p) const = 0;
  virtual int shot_steps(uint64_t key) const = 0;
  virtual ela3d_status read_samples(uint64_t key, int from, int to, float *out) = 0;
  virtual int64_t launches() const = 0;
  virtual int64_t device_bytes() const = 0;
  virtual ela3d_status timing(double *s_ms, double *v_ms, int64_t *ns, int64_t *nv) = 0;
  // Dataflow launches timed since timing was enabled: ms, launches, steps.
  virtual ela3d_status flow_timing(double *ms, int64_t *launches, int64_t *steps) = 0;
  virtual int nshots() const = 0;
  virtual int steps_done() const = 0;
  virtual cudaStream_t stream() const = 0;
};

std::unique_ptr<EngineBase> make_engine(int fp64, ela3d_status *st);

// Energy-based stability check of one shot (ELA3D_ERR_UNSTABLE on failure).
ela3d_status engine_check_energy(EngineBase *e, int shot, int fp64);

}  // namespace ela3d
