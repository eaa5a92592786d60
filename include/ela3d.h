/*
 * ela3d.h -- C ABI of the GB300 SEISMIC_CPML engine (libela3d.so).
 *
 * The reference (thejatmik/ela3d) has no library API: the simulation call is
 * the body of main() in seismicCPML_3d_isotropic_simpelmodel.cpp, and its
 * parameter surface is the set of locals assigned at the top of main().  Each
 * entry point below names the reference code it stands in for.  All sizes and
 * indices are plain integers, all buffers plain host pointers; no CUDA or
 * PyTorch types cross this boundary.
 *
 * Conventions
 *  - Every call returns ela3d_status (0 = OK) and never exits the process
 *    (the reference's HANDLE_ERROR calls exit(), seismicCPML_3d_isotropic_cudazerocopy.cu:142-151).
 *  - Grid indices are 0-based.  Cell (i, j, k) is the reference's 1-based
 *    cell (i+1, j+1, k+1); x is the fastest axis, k grows downwards (depth).
 *  - Host model and output arrays are compact nx*ny*nz, x fastest, the layout
 *    of the reference's model*.bin and v*%05i.bin files.
 *  - A plan owns its device memory and one CUDA stream.  Use one plan from
 *    one thread at a time.  A server object is internally synchronised.
 */
#ifndef ELA3D_H
#define ELA3D_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ELA3D_VERSION_MAJOR 0
#define ELA3D_VERSION_MINOR 1

typedef enum ela3d_status {
    ELA3D_OK = 0,
    ELA3D_ERR_INVALID_ARG = 1,
    ELA3D_ERR_OOM = 2,
    ELA3D_ERR_CUDA = 3,
    ELA3D_ERR_UNSTABLE = 4,   /* energy monitor saw growth or a non-finite value */
    ELA3D_ERR_TIMEOUT = 5,    /* a device-side wait gave up (kernel returned early) */
    ELA3D_ERR_NO_DEVICE = 6,
    ELA3D_ERR_BUSY = 7,       /* admission refused: not enough device memory / slots */
    ELA3D_ERR_CANCELLED = 8,
    ELA3D_ERR_NOT_FOUND = 9,
    ELA3D_ERR_NOT_READY = 10,
    ELA3D_ERR_CORRUPT = 11    /* a guard zone around a device array was overwritten */
} ela3d_status;

/* Arithmetic of the time loop.  FP32 is the production path; FP64 is the
 * checking build of the same kernels. */
enum { ELA3D_FP32 = 0, ELA3D_FP64 = 1 };

/* C-PML profile variant.  COMPAT reproduces the reference CPU program's
 * profile code as written (simpelmodel.cpp:142-361: a_x_half never set at
 * :223, z normalised by the y thickness and the zmin half-node test reading a
 * stale y abscissa at :326-350).  CLEAN is the textbook C-PML of the same
 * formulas.  The time-loop kernels are identical for both. */
enum { ELA3D_PML_COMPAT = 0, ELA3D_PML_CLEAN = 1 };

/* Source time function: Ricker (elatic_3d_unified_cuda_memory.cu:441), first
 * derivative of a Gaussian (simpelmodel.cpp:610), Gaussian (:438 commented). */
enum { ELA3D_STF_RICKER = 0, ELA3D_STF_GAUSS_DERIV = 1, ELA3D_STF_GAUSS = 2 };

/* Injection: FORCE adds w_c*s*dt/rho_c to velocity component c, rho averaged
 * as in that component's update (cudazerocopy.cu:451-453); EXPLOSIVE adds
 * s*dt*(lambda+2mu) into the normal stresses with the angle weights of
 * simpelmodel.cpp:611-622. */
enum { ELA3D_SRC_FORCE = 0, ELA3D_SRC_EXPLOSIVE = 1 };

/* Field components for ela3d_get_field. */
enum {
    ELA3D_VX = 0, ELA3D_VY = 1, ELA3D_VZ = 2,
    ELA3D_SXX = 3, ELA3D_SYY = 4, ELA3D_SZZ = 5,
    ELA3D_SXY = 6, ELA3D_SXZ = 7, ELA3D_SYZ = 8
};

/* The reference's parameter surface (simpelmodel.cpp:19-78,148-153). */
typedef struct ela3d_params {
    int32_t nx, ny, nz;       /* NIMX, NIMY, NIMZ (cells) */
    int32_t nstep;            /* NSTEP: length of the seismogram buffers */
    double dx, dy, dz;        /* DELTAX/Y/Z [m] */
    double dt;                /* DELTATT [s] */
    int32_t npml;             /* NPOINTS_PML on all six faces */
    int32_t pml_mode;         /* ELA3D_PML_* */
    double npower;            /* NPOWER */
    double k_max;             /* K_MAX_PML */
    double alpha_max;         /* ALPHA_MAX_PML; < 0 selects pi*f0 as the reference */
    double rcoef;             /* Rcoef */
    double vpml;              /* vpml (the reference fixes 3000 m/s) */
    double f0, t0, factor;    /* source frequency, delay, amplitude */
    int32_t stf;              /* ELA3D_STF_* */
    int32_t src_kind;         /* ELA3D_SRC_* */
    int32_t src_i, src_j, src_k;  /* ISOURCE/JSOURCE/KSOURCE, 0-based */
    int32_t sampgat;          /* record every sampgat steps (step % sampgat == 0) */
    double src_w[3];          /* FORCE weights for vx, vy, vz */
    double angle_force;       /* ANGLE_FORCE [deg] for EXPLOSIVE */
    const int32_t *rec;       /* nrec receiver cells (i, j, k), 0-based */
    int32_t nrec;
    int32_t precision;        /* ELA3D_FP32 / ELA3D_FP64 */
    int32_t it_output;        /* IT_OUTPUT, carried for the caller: snapshots are
                                 read with ela3d_get_field between ela3d_run
                                 calls of it_output steps (0 = none) */
    int32_t energy_every;     /* stability check cadence in steps (0 = off) */
} ela3d_params;

typedef struct ela3d_plan ela3d_plan;

typedef struct ela3d_plan_info {
    int32_t nx, ny, nz, pitch_x;   /* device row pitch in elements */
    int32_t step;                  /* steps completed */
    int32_t nsamp;                 /* samples per seismogram trace */
    int32_t nrec;
    int32_t precision;
    int64_t device_bytes;          /* device memory owned by the plan */
    int32_t slab_lo[3], slab_hi[3]; /* C-PML slab: cells [0,lo) and [hi,n) per axis */
} ela3d_plan_info;

/* ---- library ---------------------------------------------------------- */
const char *ela3d_version(void);
const char *ela3d_status_string(ela3d_status s);
/* Message of the last failed call on this thread (empty if none). */
const char *ela3d_last_error(void);

/* Fills p with the reference CPU program's defaults (simpelmodel.cpp:19-78):
 * 500^3 cells, dx=10, dt=1e-3, NSTEP=1000, npml=10, NPOWER=2, K_MAX=1,
 * alpha_max=pi*f0, Rcoef=1e-3, vpml=3000, f0=35, t0=1.2/f0, factor=1e7,
 * Gaussian-derivative explosive source at (DIMX/2, DIMY/2, 11) in 1-based
 * cells, sampgat=2, IT_OUTPUT=200, COMPAT profiles, FP32. */
ela3d_status ela3d_params_default(ela3d_params *p);

/* Makes device `ordinal` current for this thread's later calls (the
 * reference always uses device 0; one process per GPU selects its own). */
ela3d_status ela3d_select_device(int32_t ordinal);

/* Page-locked host buffers: model arrays and read-back buffers in them copy
 * to and from the device at the link's full rate (pageable memory goes
 * through a staging copy).  No counterpart: the reference's GPU program
 * copies its model from malloc'd arrays (cudazerocopy.cu:539-541,631-633).
 * ela3d_host_free takes only pointers from ela3d_host_alloc (or NULL). */
ela3d_status ela3d_host_alloc(size_t bytes, void **out);
ela3d_status ela3d_host_free(void *ptr);

/* ---- single shot -------------------------------------------------------- */
/* Replaces main()'s setup: allocations and zero fill (simpelmodel.cpp:80-140),
 * model fill (:41-59), profile precompute (:142-361).  cp, cs, rho are host
 * arrays of nx*ny*nz float32, copied; the caller keeps ownership. */
ela3d_status ela3d_plan_create(const ela3d_params *p, const float *cp, const float *cs,
                               const float *rho, ela3d_plan **out);
/* Advances nsteps time steps (the it loop, simpelmodel.cpp:376-726) and
 * waits for completion; resumable.  Returns ELA3D_ERR_UNSTABLE when the
 * energy monitor trips, ELA3D_ERR_TIMEOUT when a kernel gave up a wait.
 * Steps past nstep keep propagating the wavefield with no source and no
 * recording (nstep sizes the source table and the seismogram buffers). */
ela3d_status ela3d_run(ela3d_plan *plan, int32_t nsteps);
/* ela3d_run bracketed by CUDA events on the plan's stream; *ms receives the
 * device time of the nsteps steps. */
ela3d_status ela3d_run_timed(ela3d_plan *plan, int32_t nsteps, double *ms);
/* Queues nsteps on the plan's stream without waiting. */
ela3d_status ela3d_enqueue(ela3d_plan *plan, int32_t nsteps);
/* Waits for queued work and reports device-side errors. */
ela3d_status ela3d_sync(ela3d_plan *plan);
/* Seismograms [nrec][3][nsamp] (vx, vy, vz), nsamp = nstep / sampgat: the
 * receiver gather of simpelmodel.cpp:593-602 sampled as at :625. */
ela3d_status ela3d_get_seismograms(ela3d_plan *plan, float *out);
ela3d_status ela3d_get_seismograms_f64(ela3d_plan *plan, double *out);
/* Current field, compact nx*ny*nz (snapshot of simpelmodel.cpp:685-722). */
ela3d_status ela3d_get_field(ela3d_plan *plan, int32_t comp, float *out);
ela3d_status ela3d_get_field_f64(ela3d_plan *plan, int32_t comp, double *out);
/* Source-point trace, [3][nstep + 1]: the components the source acts on at
 * its cell, right after each step's injection (index it = 1..nstep; index 0
 * is 0) -- sxx syy szz for an explosive source, as the reference's FP64 GPU
 * program records into recsrc{x,y,z}.txt
 * (elatic_3d_unified_cuda_memory.cu:463-465,1202-1223); vx vy vz for a force. */
ela3d_status ela3d_get_source_trace(ela3d_plan *plan, float *out);
ela3d_status ela3d_get_source_trace_f64(ela3d_plan *plan, double *out);
/* Total kinetic + strain energy [J], FP64 device reduction (no counterpart
 * in the reference; the stability monitor). */
ela3d_status ela3d_energy(ela3d_plan *plan, double *out);
/* The same energy of caller-owned FP32 device arrays -- fields[9] = vx vy vz
 * sxx syy szz sxy sxz syz and the model cp cs rho, each [nz][ny][pitch_x],
 * x fastest -- written to *out (device memory) on `stream` (a cudaStream_t;
 * NULL = the default stream); asynchronous.  Allocates no device memory,
 * for callers that cannot allocate where they need the number (allocator
 * hooks, host callbacks, loops that cannot afford cudaMalloc's device
 * synchronisation).  Its intermediate sums live in a fixed array inside the
 * library: nz <= 16384 (a larger nz returns ELA3D_ERR_INVALID_ARG), nothing
 * in it needs to start at zero, and calls overlapping in time on one device
 * race for it -- serialise them.  Every call looks up the array's address
 * on the current device; the first call on a device is its set-up (it also
 * loads the library's kernels there), so when capturing work into a CUDA
 * graph, make that first call before the capture begins.  No counterpart in
 * the reference. */
ela3d_status ela3d_energy_noalloc(const float *const *fields, const float *cp, const float *cs,
                                  const float *rho, int32_t nx, int32_t ny, int32_t nz, int32_t pitch_x,
                                  double dx, double dy, double dz, double *out, void *stream);
ela3d_status ela3d_plan_info_get(ela3d_plan *plan, ela3d_plan_info *out);
/* Checkpoint / resume: the plan's complete time-stepping state (the nine
 * fields, the C-PML memory variables, the model, the seismograms and source
 * trace so far, the step count) as one host buffer of
 * ela3d_checkpoint_size bytes.  ela3d_checkpoint_load restores it into a
 * plan created with the same parameters (in this process or another), which
 * then continues exactly as the saved plan would have; a checkpoint of a
 * plan with other sizes, spacings, time step, C-PML coefficients, source or
 * receivers is refused (ELA3D_ERR_INVALID_ARG).  The model travels in the
 * checkpoint.  The reference's
 * snapshots hold vx, vy, vz only and cannot resume a run; no counterpart. */
ela3d_status ela3d_checkpoint_size(ela3d_plan *plan, int64_t *bytes);
ela3d_status ela3d_checkpoint_save(ela3d_plan *plan, void *buf, int64_t bytes);
ela3d_status ela3d_checkpoint_load(ela3d_plan *plan, const void *buf, int64_t bytes);
/* Per-kernel CUDA-event timing of subsequent launches (0 = off). */
ela3d_status ela3d_set_kernel_timing(ela3d_plan *plan, int32_t enable);
/* Sums since timing was enabled: stress and velocity kernel milliseconds
 * and launch counts. */
ela3d_status ela3d_get_kernel_timing(ela3d_plan *plan, double *stress_ms, double *velocity_ms,
                                     int64_t *stress_launches, int64_t *velocity_launches);
/* The same for dataflow launches (schedule 3): milliseconds, launches and
 * the time steps they ran. */
ela3d_status ela3d_get_flow_timing(ela3d_plan *plan, double *ms, int64_t *launches, int64_t *steps);
ela3d_status ela3d_plan_destroy(ela3d_plan *plan);
/* Test hook for the failure path: the kernels of the plan's next `steps`
 * time steps withhold their shared-memory loads, so their bounded device
 * waits expire (20 ms) and the next ela3d_sync/ela3d_run reports
 * ELA3D_ERR_TIMEOUT.  Nothing faults or hangs; the CUDA context stays usable,
 * the plan's fields are left partly updated.  No reference counterpart. */
ela3d_status ela3d_plan_inject_timeout(ela3d_plan *plan, int32_t steps);
/* Test hook: writes `value` (e.g. NaN) into every padding column
 * x in [nx, pitch_x) of the nine fields and of the C-PML memory-variable
 * arrays -- cells no update may read into the grid.  No counterpart. */
ela3d_status ela3d_plan_poison_padding(ela3d_plan *plan, double value);
/* Test hook: the plan's C-PML profiles of one axis (0 = x, 1 = y, 2 = z)
 * as the kernels read them, widened to double: a, b, 1/K, a_half, b_half,
 * 1/K_half, n values each (n = nx, ny or nz), so 6n values into `out`.
 * Checked against the reference's profile code (simpelmodel.cpp:142-361). */
ela3d_status ela3d_plan_get_profiles(ela3d_plan *plan, int32_t axis, double *out);
/* Debug check: with the environment variable ELA3D_GUARD_ZONES=<bytes> set
 * when a plan is created, every array in its device pool is followed (and
 * the pool preceded) by a zone of that many bytes filled with 0xA5; this
 * call verifies every zone is intact (ELA3D_ERR_CORRUPT names the array a
 * write ran past).  OK when guard zones are off.  No counterpart. */
ela3d_status ela3d_plan_check_guards(ela3d_plan *plan);

/* ---- kernel variants and tuning ----------------------------------------- */
/* A compiled instance of the stress/velocity kernel pair: real type, x-y
 * tile and shared-memory pipeline depth.  No counterpart in the reference
 * (its kernels use fixed 10^3 thread blocks, cudazerocopy.cu:1361-1369). */
typedef struct ela3d_variant_info {
    int32_t fp64, tile_x, tile_y, stages, threads;   /* stages: of the stress
                                                        (and dataflow) kernel's ring */
    int32_t stress_smem, velocity_smem;
    int32_t loads;   /* 0: stages filled by TMA tiled loads; 1: by cp.async
                        copies of the whole loading warp (a measured
                        alternative, not a default) */
    int32_t velocity_stages;   /* stages of the velocity kernel's ring */
} ela3d_variant_info;

/* Work schedule: kind 0 = equal contiguous share of (tile, plane) units per
 * block; kind 1 = z-chunks of `chunk` planes dealt round-robin, shot by
 * shot; kind 2 = the same chunks interleaved across shots (blocks running
 * together hold the same tile of different shots, so a shared model tile is
 * read from DRAM once).  -1 (chunk: 0) selects the built-in choice; a
 * field out of range or a variant of the other precision is
 * ELA3D_ERR_INVALID_ARG, reported before any device work. */
typedef struct ela3d_tuning {
    int32_t variant;        /* index < ela3d_variant_count(), or -1 */
    int32_t schedule;       /* 0, 1, 2, 3 or 4 (dataflow, below), or -1 */
    int32_t chunk;          /* planes per z-chunk for schedules 1-4 (>= 2 for
                               3 and 4), or 0 */
    int32_t blocks_per_sm;  /* cap on resident blocks per SM, 0 = occupancy limit, -1 */
    int32_t prefetch;       /* prefetch of the C-PML memory variables by the
                               loading warp: bit 1 (2) x slab into L1, bit 2 (4)
                               y and z slabs into L2; -1 = built-in choice
                               (6; 2 or 0 for shots whose arrays fit in or
                               near the L2) */
    int32_t lag;            /* schedules 3 and 4: places in the work list
                               between an item and the last item it waits
                               for; 0 or -1 = three rounds of the grid */
} ela3d_tuning;
/* Schedules 3 and 4 (dataflow): instead of two kernels per time step, one
 * persistent, cooperative kernel advances up to 200 steps per launch.  Its
 * work items are the stress or velocity half-step of one (x-y tile,
 * z-chunk) at one step; each item waits (on device counters) for exactly
 * the items whose results it reads or overwrites.  The host places every
 * item `lag` places after the last item it waits for, so it runs soon
 * after them, while their results are still in L2; schedule 3 keeps the
 * time steps in sequence, schedule 4 lets a step start where the previous
 * one is done.  Results are bit-identical to schedules 0-2.  Shots with an
 * explosive source run the two-kernel path with schedule 1.  The work list
 * is built on the host for the shots running, again whenever shots join or
 * retire, so these schedules suit a plan or a batch of shots that run
 * together; the autotuner tries them for single shots, and schedule 4 is
 * the built-in choice for a single FP32 shot without an explosive source,
 * its z-chunks sized for about 1.5 work items per block (ela3d_builtin_tuning
 * reports the choice). */

/* Times every compiled variant with the candidate schedules on these shots
 * (`steps` time steps each, after a warm-up) and returns the fastest choice;
 * it is also cached for the workload's shape, so later plans and batches of
 * that shape use it.  ELA3D_TUNE_CACHE=<file> keeps the cache across
 * processes; ELA3D_AUTOTUNE=1 makes plan and batch creation tune on a cache
 * miss.  candidates (may be NULL) receives the number of choices timed.
 * No reference counterpart. */
ela3d_status ela3d_autotune(int32_t nshots, const ela3d_params *params, const float *const *cp,
                            const float *const *cs, const float *const *rho, int32_t steps,
                            ela3d_tuning *best, double *best_ms, int32_t *candidates);
int32_t ela3d_variant_count(void);
ela3d_status ela3d_variant_get(int32_t index, ela3d_variant_info *out);
/* ela3d_plan_create with an explicit kernel variant and schedule. */
ela3d_status ela3d_plan_create_tuned(const ela3d_params *p, const float *cp, const float *cs,
                                     const float *rho, const ela3d_tuning *tune, ela3d_plan **out);

/* ---- earth models generated on the device -------------------------------- */
/* Instead of host arrays, a plan or server request may name a model to be
 * generated by a GPU kernel directly in its device arrays (no host arrays,
 * no upload):
 *  HOMOGENEOUS     cp0, cs0, rho0 everywhere (simpelmodel.cpp:45-59);
 *  LAYERED_DOME    nlayers layers bounded by interfaces
 *                  depth[i] - dome_amp exp(-r^2 / (2 dome_sigma^2)) (cells,
 *                  r from (dome_xc, dome_yc)); cs = cp / cs_ratio[L],
 *                  rho = rho_coef cp^rho_pow; cp and rho get independent
 *                  uniform +-perturb relative noise from a counter-based hash
 *                  of (seed, cell);
 *  MATLAB_ANTICLINE the five-medium anticline of generate_3d_model_anticline.m
 *                  (exactly that model at 201^3; depths scale with nz/201).
 * Values are rounded to float32 (the model's precision) in every plan type. */
enum { ELA3D_MODEL_HOMOGENEOUS = 0, ELA3D_MODEL_LAYERED_DOME = 1, ELA3D_MODEL_MATLAB_ANTICLINE = 2 };
typedef struct ela3d_model_spec {
    int32_t kind, nlayers;
    double cp[8], cs_ratio[8], depth[8];
    double dome_amp, dome_sigma, dome_xc, dome_yc;
    double rho_coef, rho_pow, perturb;
    uint64_t seed;
    double cp0, cs0, rho0;
} ela3d_model_spec;
/* ela3d_plan_create with a generated model. */
ela3d_status ela3d_plan_create_model(const ela3d_params *p, const ela3d_model_spec *model,
                                     const ela3d_tuning *tune, ela3d_plan **out);
/* The generated model as host arrays (nx*ny*nz float32 each), for
 * inspection or for other tools. */
ela3d_status ela3d_model_generate(const ela3d_model_spec *model, int32_t nx, int32_t ny, int32_t nz,
                                  float *cp, float *cs, float *rho);

/* ---- batches of shots ---------------------------------------------------- */
/* Many shots resident together and advanced by the same two launches per
 * time step (the persistent kernels deal (shot, tile, z-run) items to all
 * SMs).  Shots may differ in size, model, source, receivers, dt and nstep
 * (same precision).  Shots whose cp, cs and rho pointers and grid equal an
 * earlier shot's share that shot's device model.  A shot stops being
 * computed once it has done its nstep steps; its results stay readable.
 * Runs of 50 or more steps replay a captured CUDA graph.  The reference runs
 * one shot per process (no counterpart). */
typedef struct ela3d_batch ela3d_batch;
ela3d_status ela3d_batch_create(int32_t nshots, const ela3d_params *params, const float *const *cp,
                                const float *const *cs, const float *const *rho, const ela3d_tuning *tune,
                                ela3d_batch **out);
/* Advances every unfinished shot by up to nsteps steps and waits. */
ela3d_status ela3d_batch_run(ela3d_batch *b, int32_t nsteps);
/* ela3d_batch_run timed with CUDA events on the batch's stream. */
ela3d_status ela3d_batch_run_timed(ela3d_batch *b, int32_t nsteps, double *ms);
ela3d_status ela3d_batch_get_seismograms(ela3d_batch *b, int32_t shot, float *out);
ela3d_status ela3d_batch_get_field(ela3d_batch *b, int32_t shot, int32_t comp, float *out);
ela3d_status ela3d_batch_get_source_trace(ela3d_batch *b, int32_t shot, float *out);
ela3d_status ela3d_batch_info(ela3d_batch *b, int32_t shot, ela3d_plan_info *out);
ela3d_status ela3d_batch_destroy(ela3d_batch *b);

/* ---- serving: continuous batching ---------------------------------------- */
/* A request loop on one GPU.  Shot requests of any size are queued and
 * admitted in arrival order while their device footprint fits the budget
 * (and a slot is free, and the fill target is not reached); admitted shots
 * stay resident and are advanced
 * together by the batched kernels, `steps_per_round` steps per round;
 * requests arriving meanwhile join at the next round, and finished shots
 * leave, freeing memory.  Seismogram samples are copied back after every
 * round and can be read while the shot runs.  A request whose footprint
 * exceeds the whole budget fails with ELA3D_ERR_BUSY.  No reference
 * counterpart (the reference runs one hard-coded shot per process). */
typedef struct ela3d_server ela3d_server;
typedef struct ela3d_server_config {
    int64_t hbm_budget_bytes;   /* device bytes for shot state; 0 = 80% of free memory */
    int32_t max_active;         /* concurrent shots; 0 = no limit */
    int32_t steps_per_round;    /* time steps between admission rounds (default 50) */
    int32_t precision;          /* of every request */
    int32_t fill_cells;         /* admit (in arrival order) only while the running
                                   shots hold fewer cells than this, so early
                                   requests finish early once the GPU is full;
                                   0 = no target */
    ela3d_tuning tune;
} ela3d_server_config;
/* Request states reported by ela3d_server_poll. */
enum { ELA3D_REQ_QUEUED = 0, ELA3D_REQ_RUNNING = 1, ELA3D_REQ_DONE = 2, ELA3D_REQ_FAILED = 3,
       ELA3D_REQ_CANCELLED = 4 };
typedef struct ela3d_server_stats {
    int64_t submitted, completed, failed, cancelled, queued, running, rounds;
    double cell_updates;        /* of completed requests */
    double busy_seconds;        /* wall time of the device rounds */
    double wall_seconds;        /* first submission to last completion */
    double latency_p50_s, latency_p99_s, latency_max_s;  /* submission to completion */
    int64_t device_bytes_in_use, device_bytes_budget;
} ela3d_server_stats;

ela3d_status ela3d_server_config_default(ela3d_server_config *c);
/* Starts the worker thread on the calling thread's current device. */
ela3d_status ela3d_server_create(const ela3d_server_config *cfg, ela3d_server **out);
/* Queues one shot; the parameters, receivers and model are copied. */
ela3d_status ela3d_server_submit(ela3d_server *s, const ela3d_params *p, const float *cp, const float *cs,
                                 const float *rho, uint64_t *ticket);
/* State and number of seismogram samples available so far. */
ela3d_status ela3d_server_poll(ela3d_server *s, uint64_t ticket, int32_t *state, int32_t *samples_ready);
/* ela3d_server_submit with a model generated on the device at admission. */
ela3d_status ela3d_server_submit_model(ela3d_server *s, const ela3d_params *p, const ela3d_model_spec *model,
                                       uint64_t *ticket);
/* Samples [first, first+count) of every trace, [nrec][3][count]; returns
 * ELA3D_ERR_NOT_READY if they have not all arrived. */
ela3d_status ela3d_server_read(ela3d_server *s, uint64_t ticket, int32_t first, int32_t count, float *out);
/* Waits for a request to finish (timeout_ms < 0: no limit). */
ela3d_status ela3d_server_wait(ela3d_server *s, uint64_t ticket, int32_t timeout_ms);
/* Stops a queued or running request at the next round boundary. */
ela3d_status ela3d_server_cancel(ela3d_server *s, uint64_t ticket);
/* Completion callback: called exactly once when the request ends, with
 * ELA3D_OK (done), its error, or ELA3D_ERR_CANCELLED.  The server's worker
 * thread calls it with no lock held, so it may call the other
 * ela3d_server_* functions except ela3d_server_destroy; a request that has
 * already ended gets its call at once, on the registering thread, and those
 * ended by ela3d_server_destroy get theirs on the destroying thread before
 * it returns.  One callback per request (a later registration replaces an
 * earlier one). */
typedef void (*ela3d_request_callback)(uint64_t ticket, ela3d_status status, void *user);
ela3d_status ela3d_server_on_done(ela3d_server *s, uint64_t ticket, ela3d_request_callback cb, void *user);
/* Forgets a finished request (frees its host results). */
ela3d_status ela3d_server_release(ela3d_server *s, uint64_t ticket);
ela3d_status ela3d_server_stats_get(ela3d_server *s, ela3d_server_stats *out);
/* Stops the worker at the end of its current round; queued and running
 * requests end as cancelled, and threads blocked in ela3d_server_wait return
 * ELA3D_ERR_CANCELLED before this call returns.  No call may pass the server
 * after that. */
ela3d_status ela3d_server_destroy(ela3d_server *s);

/* ---- host-side planning (no GPU needed) ---------------------------------- */
/* C-PML slab extent of one axis from its 'a' profiles: cells [0, lo) and
 * [hi, n) may carry memory variables; every cell of [lo, hi) has a = 0 in
 * both the full- and half-node profile, so its memory variables stay 0 and
 * are not stored (the reference stores all 18 for every cell,
 * simpelmodel.cpp:89-106).  lo == hi == n when the layer covers the axis. */
ela3d_status ela3d_slab_extent(const double *a_full, const double *a_half, int32_t n,
                               int32_t *lo, int32_t *hi);
/* Host-only: the built-in kernel choice for a single shot with these
 * parameters (variant, schedule, chunk, prefetch; no tuning cache, no
 * device work; the current device's SM count, 152 without a device).  No
 * reference counterpart. */
ela3d_status ela3d_builtin_tuning(const ela3d_params *p, ela3d_tuning *out);
/* Host-only test hook: the dataflow work list (schedules 3 and 4) of one
 * nx*ny*nz shot for `nsteps` steps, tiles tile_x*tile_y, z-chunks of
 * `chunk` planes, `gap` places after each item's last dependency, steps
 * overlapping if `overlap`.  *nitems receives the item count; items (if not
 * NULL, room for *nitems on entry) receives per item (kind, step, chunk,
 * tile, k0, k1).  ELA3D_ERR_INVALID_ARG on bad sizes or when an item would
 * not follow the items it waits for.  No reference counterpart. */
ela3d_status ela3d_flow_schedule_build(int32_t nx, int32_t ny, int32_t nz, int32_t tile_x, int32_t tile_y,
                                       int32_t chunk, int32_t gap, int32_t overlap, int32_t nsteps,
                                       int32_t *nitems, int32_t *items);
/* The work split the kernels use for one grid: items (tile, k0, k1) per
 * block.  With items == NULL only the counts are returned.  No reference
 * counterpart (its launch is a fixed 3-D grid, cudazerocopy.cu:1361-1369). */
ela3d_status ela3d_schedule_build(int32_t nx, int32_t ny, int32_t nz, int32_t tile_x, int32_t tile_y,
                                  int32_t schedule, int32_t chunk, int32_t max_blocks,
                                  int32_t *nitems, int32_t *nblocks,
                                  int32_t *items /* nitems x 3 */, int32_t *block_first /* nblocks+1 */);

#ifdef __cplusplus
}
#endif
#endif
