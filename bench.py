"""Benchmark: Gcell-updates/s of the SEISMIC_CPML time loop on GB300.

Workload (one "step" = one time step, stress + velocity half-steps, over
every cell of one shot): the 256^3 four-layer anticline shot in FP32
(dt 1e-3 s, 16 PML cells, Ricker 12 Hz on vz, 201-receiver line), synthetic
model from numpy default_rng(0).  Every step streams ~2.4 GB, far more than
the 129 MB L2, so no flush is needed between steps.

Own arm (default): per rank one resident shot; W untimed warm-up steps, then
K steps timed with CUDA events on the plan's stream between barriers, max
over ranks (the library's own path: replayed 50-step CUDA graphs).  Also
reported:
  roofline  the dominant kernel's algorithmic bytes per launch / its mean
            CUDA-event duration (a separate pass of directly launched,
            individually timed kernels), against MEASURED_PEAKS.json hbm_gbs;
  e2e       one full 2000-step shot through the C ABI from host arrays
            (plan creation with the model upload, the run, the seismogram
            read-back), wall clock;
  accuracy  that shot's every seismogram and final field component against
            the FP64 build of the same kernels (relative L2);
  cpu_baseline  the reference CPU program (oracle/_ref, else the oracle's C
            restatement) on 1 core, a bounded sample of the same shot;
  reference_gpu_program  the reference's own FP32 CUDA program, built from
            its source into oracle/_ref, at the same grid size on this GPU.
Also in the same line: "batched" (64 shots of the 256^3 anticline sharing
one model, advanced together), "uneven" (48 uneven grids together vs one
at a time) and "serving" (a Poisson request stream swept to saturation,
p50/p99 latency), each next to the single-shot path on the same GPU, each
with an FP64 re-run of sampled shots (fp64_check); and "large_grid" (one
512^3 shot, its model generated on the GPU).
Reference arm (--impl reference): the reference CPU program itself on all
host cores (one process per core, each a bounded sample of the same shot),
rank 0 only.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "Gcell-updates/s"
WORKLOAD = "anticline_256"
FIELD_NAMES = ("vx", "vy", "vz", "sxx", "syy", "szz", "sxy", "sxz", "syz")  # ela3d_get_field order


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ------------------------------------------------------------------ env --
from ela3d_gb300.dist import Group, env as dist_env, shard  # noqa: E402


def cuda_sync():
    try:
        import torch

        if torch.cuda.is_available():
            torch.cuda.synchronize()
    except Exception:
        pass


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,utilization.gpu,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(prefix="ela3d_clocks_", suffix=".csv")
            self.fh = os.fdopen(fd, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            if self.path:
                self.fh.close()
                os.unlink(self.path)

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 10:
                continue
            try:
                rows.append({"sm": float(f[1]), "max": float(f[2]), "util": float(f[4]), "hw": f[6], "hwt": f[7],
                             "swt": f[8], "pcap": f[9]})
            except ValueError:
                continue
        os.unlink(self.path)
        load = [r for r in rows if r["util"] >= 50] or rows
        if not load:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        reasons = set()
        for r in load:
            for key, name in (("hw", "hw_slowdown"), ("hwt", "hw_thermal_slowdown"), ("swt", "sw_thermal_slowdown"),
                              ("pcap", "sw_power_cap")):
                if r[key].lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(r["sm"] for r in load), "sm_max_mhz": max(r["max"] for r in load),
                "reasons": sorted(reasons), "samples": len(load)}


def measured_peaks() -> tuple[float, str]:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic(kernel: str, key: str = "dram_bytes_per_launch_full_grid") -> float | None:
    """DRAM bytes per launch (or, with key dram_bytes_per_step_full_grid,
    per time step) from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_{WORKLOAD}.txt")
    try:
        for line in open(path):
            if line.startswith(key + ":"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


def fp64_check(pairs) -> dict:
    """Accuracy of FP32 results against the FP64 build of the same kernels:
    `pairs` is a list of (label, ShotParams, cp, cs, rho, steps, fp32
    seismograms [nrec, 3, nsamp]); each shot is re-run alone in FP64 for the
    same steps and the first steps // sampgat samples are compared."""
    import ela3d_gb300 as E

    rows = []
    for label, p, cp, cs, rho, steps, s32 in pairs:
        with E.Plan(p.with_(precision=1), cp, cs, rho) as pl:
            pl.run(steps)
            s64 = pl.seismograms(fp64=True)
        n = steps // p.sampgat
        a, b = s32[..., :n].astype(np.float64), s64[..., :n]
        norms = np.array([np.linalg.norm(b[r]) for r in range(b.shape[0])])
        # per receiver only where the wave has arrived (a trace of pure
        # round-off before the first arrival has no meaningful relative error)
        live = np.flatnonzero(norms >= 1e-3 * norms.max()) if norms.size else []
        per = [float(np.linalg.norm(a[r] - b[r]) / norms[r]) for r in live]
        rows.append({"shot": label, "steps": steps, "rel_l2": float(np.linalg.norm(a - b) / np.linalg.norm(b)),
                     "max_rel_l2_per_receiver": max(per) if per else None,
                     "receivers_with_signal": f"{len(per)} of {b.shape[0]}"})
    return {"what": "FP32 seismograms vs the same shot re-run alone in FP64 (relative L2)", "shots": rows,
            "max_rel_l2": max(r["rel_l2"] for r in rows) if rows else None}


def shot_accuracy(p, cp, cs, rho, seis32, fields32) -> dict:
    """Relative L2 error of every seismogram (one receiver's vx, vy, vz
    record, wherever the FP64 record is not all zero) and of each final
    field component of the FP32 shot against the FP64 build run on the same
    inputs for the same steps."""
    import ela3d_gb300 as E

    with E.Plan(p.with_(precision=1), cp, cs, rho) as pl:
        pl.run(p.nstep)
        s64 = pl.seismograms(fp64=True)
        f64 = [pl.field(c, fp64=True) for c in range(9)]
    rel = lambda a, b: float(np.linalg.norm(a.astype(np.float64) - b) / np.linalg.norm(b))  # noqa: E731
    per = [rel(seis32[r], s64[r]) for r in range(s64.shape[0]) if np.any(s64[r])]
    wave = {name: rel(a, b) for name, a, b in zip(FIELD_NAMES, fields32, f64) if np.any(b)}
    return {"what": f"FP32 shot vs the FP64 build, {p.nstep} steps (relative L2)",
            "max_rel_l2_per_seismogram": max(per) if per else None, "seismograms": len(per),
            "rel_l2_all_seismograms": rel(seis32, s64), "final_wavefield_rel_l2": wave,
            "max_final_wavefield_rel_l2": max(wave.values()) if wave else None}


# ------------------------------------------------------------ workload --
def workload(nstep: int = 2000):
    from ela3d_gb300 import configs

    return configs.anticline_256(nstep=nstep)


def config_block(p, extra=None):
    c = {"workload": f"{WORKLOAD}: {p.nx}x{p.ny}x{p.nz} cells, four-layer dome model, FP32, dt {p.dt} s, "
                     f"{p.nstep}-step shot, {p.npml} PML cells, Ricker {p.f0:g} Hz on vz, {p.nrec} receivers",
         "grid": [p.nx, p.ny, p.nz], "npml": p.npml, "nstep_shot": p.nstep,
         "l2": "inputs larger than L2 (about 2.4 GB streamed per step vs 129 MB L2); no flush",
         "parallelism": "one shot per GPU (shots are independent)"}
    if extra:
        c.update(extra)
    return c


# --------------------------------------------------------- CPU baseline --
def cpu_reference_rate(p, cp, cs, rho, steps: int, procs: int, fp64: bool = False) -> dict:
    """Runs the reference CPU program (oracle/_ref; its float64 build with
    fp64) or, if it was not built, the oracle's C restatement, as `procs`
    concurrent processes each doing `steps` time steps of the shot; returns
    the aggregate rate."""
    import oracle

    exe = oracle.reference_binary(fp64)
    cells = p.cells
    warm = 1
    wd = tempfile.mkdtemp(prefix="ela3d_cpu_")
    try:
        if exe:
            for name, a in (("cp", cp), ("cs", cs), ("rho", rho)):
                np.ascontiguousarray(a, np.float64 if fp64 else np.float32).tofile(os.path.join(wd, f"m_{name}.bin"))
            runs = []
            for q in range(procs):
                d = os.path.join(wd, f"r{q}")
                os.makedirs(d)
                oracle.write_config(os.path.join(d, "cfg.txt"), p.with_(nstep=steps + warm), steps + warm,
                                    os.path.join(wd, "m_"), time_from=warm + 1)
                runs.append((d, subprocess.Popen([exe, os.path.join(d, "cfg.txt")], cwd=d,
                                                 stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)))
            spans = []
            for d, pr in runs:
                if pr.wait() != 0:
                    raise RuntimeError("reference program failed")
                t0, t1, n = open(os.path.join(d, "steps.txt")).read().split()
                spans.append((float(t0), float(t1), int(n)))
            start = min(s[0] for s in spans)
            end = max(s[1] for s in spans)
            total = sum(cells * s[2] for s in spans)
            kind = "reference"
        else:
            import multiprocessing as mp

            ctx = mp.get_context("spawn")
            with ctx.Pool(procs) as pool:
                res = pool.starmap(_port_worker, [(p, cp, cs, rho, steps, fp64)] * procs)
            start = min(r[0] for r in res)
            end = max(r[1] for r in res)
            total = cells * steps * procs
            kind = "port"
    finally:
        import shutil

        shutil.rmtree(wd, ignore_errors=True)
    value = total / (end - start) / 1e9
    return {"value": value, "unit": METRIC, "cores": procs, "kind": kind,
            "sample": f"{procs} process(es) x {steps} time steps of the {p.nx}^3 shot "
                      f"({'reference CPU program' if kind == 'reference' else 'C restatement'}"
                      f"{', float64 build' if fp64 else ''}), {(end - start):.1f} s wall",
            "seconds": end - start}


REF_GPU_PROGRAMS = {
    "ref_gpu_f32": "the reference's FP32 CUDA program (seismicCPML_3d_isotropic_cudazerocopy.cu: five stencil "
                   "kernels per step plus gather and source, 8x8x8-thread blocks, arrays in device memory)",
    "ref_gpu_f64": "the reference's FP64 CUDA program (elatic_3d_unified_cuda_memory.cu: five stencil kernels "
                   "per step plus gather and source, 5x5x5-thread blocks, arrays in managed memory prefetched "
                   "to the GPU before the loop)",
}


def reference_gpu_rate(n: int, steps: int, warm: int, program: str = "ref_gpu_f32") -> dict:
    """One of the reference's own GPU programs (built by oracle/make_ref.py
    into oracle/_ref) on this GPU: an n^3 grid, `warm` untimed steps, then
    `steps` timed by the program (file output off).  Its own constant medium
    and source; the kernels are the reference's, unchanged."""
    exe = os.path.join(ROOT, "oracle", "_ref", program)
    if not os.path.exists(exe):
        return {"value": None, "unavailable": f"reference GPU program not built (oracle/_ref/{program})"}
    wd = tempfile.mkdtemp(prefix="ela3d_refgpu_")
    try:
        r = subprocess.run([exe, str(n), str(steps + warm), str(warm), "0"], cwd=wd, capture_output=True,
                           text=True, timeout=600)
    finally:
        import shutil

        shutil.rmtree(wd, ignore_errors=True)
    for line in r.stdout.splitlines():
        if line.startswith("ELA3D_REF_GPU"):
            f = line.split()
            got = dict(zip(f[1::2], f[2::2]))
            if int(got["status"]) != 0:
                return {"value": None, "unavailable": f"reference GPU program reported CUDA status {got['status']}"}
            secs = float(got["seconds"])
            return {"value": n ** 3 * int(got["steps"]) / secs / 1e9, "unit": METRIC,
                    "ms_per_step": secs * 1e3 / int(got["steps"]),
                    "what": f"{REF_GPU_PROGRAMS[program]}, {n}^3, {warm} warm-up + {got['steps']} timed steps, "
                            f"wall clock around its loop, file output off"}
    return {"value": None, "unavailable": f"reference GPU program exited {r.returncode} without a timing line"}


def _port_worker(p, cp, cs, rho, steps, fp64=False):
    import oracle

    t0 = time.perf_counter()
    oracle.run(p.with_(rec=np.zeros((0, 3), np.int32)), cp, cs, rho, steps, fp64=fp64, want_fields=False)
    t1 = time.perf_counter()
    return (t0, t1)


# --------------------------------------------------------------- arms --
def run_ours(args, rank, world, local):
    import ela3d_gb300 as E
    from ela3d_gb300.metrics import bytes_per_cell

    E.select_device(local)
    dist = Group(world)
    p, cp, cs, rho = workload()
    cells = p.cells
    tune = {"variant": -1, "schedule": -1, "chunk": 0}
    tune_info = {"source": "built-in default"}
    if not args.no_autotune:
        best, ms_best, cand = E.autotune([(p, cp, cs, rho)], steps=30)
        tune = best.as_dict()
        v = E.variants()[best.variant]
        tune_info = {"source": "ela3d_autotune", "candidates": cand, "tile": [v.tile_x, v.tile_y],
                     "stages": v.stages, "schedule": best.schedule, "chunk": best.chunk, "prefetch": best.prefetch}
    # explicit tuning fields (profiling comparisons)
    for key, val in (("variant", args.variant), ("prefetch", args.prefetch), ("schedule", args.schedule),
                     ("chunk", args.chunk)):
        if val >= 0:
            tune[key] = val
            tune_info[key] = val
    clocks = ClockSampler(local)
    plan = E.Plan(p, cp, cs, rho, **tune)
    plan.run(args.warmup)
    clocks.start()
    dist.barrier()
    cuda_sync()
    ms = plan.run_timed(args.steps)    # the library's own path: replayed CUDA graphs
    cuda_sync()
    dist.barrier()
    # per-kernel CUDA events (direct launches, no graphs) for the roofline
    plan.set_kernel_timing(True)
    plan.run_timed(args.kernel_steps)
    s_ms, v_ms, ns, nv = plan.kernel_timing()
    f_ms, f_launches, f_steps = plan.flow_timing()
    plan.set_kernel_timing(False)
    plan.close()
    two_path = None
    if f_launches and not ns:
        # the two half-step kernels, timed too (the path the dataflow kernel
        # replaces at this size; also the one explosive sources and batches run)
        with E.Plan(p, cp, cs, rho, schedule=1, chunk=10) as alt:
            alt.run(3)
            alt.set_kernel_timing(True)
            alt.run_timed(args.kernel_steps)
            s_ms, v_ms, ns, nv = alt.kernel_timing()
        two_path = "two half-step kernels (schedule 1, 10-plane z-chunks), timed in a separate plan"
    t_max = dist.max(ms / 1e3)
    value = cells * args.steps * world / t_max / 1e9
    if f_launches:
        # dataflow kernel: one launch per up to 200 steps (its 50-step work
        # list walked up to four times; the kernel-timing pass reports the
        # same split: f_launches launches for f_steps steps)
        launches = -(-args.steps // 200)
    else:
        # kernels launched in the timed region: one step-counter set, 50-step
        # graphs of 100 stencil launches plus a counter update, the rest direct
        launches = 1 + (args.steps // 50) * 101 + (args.steps % 50) * 2

    # e2e: one whole shot through the C ABI from host arrays
    e2e = None
    accuracy = None
    if not args.no_e2e:
        # the inputs wait in page-locked host memory (ela3d_host_alloc), as a
        # caller streaming shots would hold them; the timed region copies
        # them in, runs the whole shot and reads the seismograms back
        host = [E.pinned_copy(a, np.float32) for a in (cp, cs, rho)]
        seis = E.pinned_empty((p.nrec, 3, p.nsamp), np.float32)
        dist.barrier()
        t0 = time.perf_counter()
        shot = E.Plan(p, *host, **tune)
        shot.sync()
        t1 = time.perf_counter()
        shot.run(p.nstep)
        t2 = time.perf_counter()
        shot.seismograms(out=seis)
        t3 = time.perf_counter()
        t_e2e = dist.max(t3 - t0)
        e2e = {"value": cells * p.nstep * world / t_e2e / 1e9, "unit": METRIC,
               "h2d_bytes_per_step": int(3 * cells * 4 / p.nstep),
               "d2h_bytes_per_step": int(seis.nbytes / p.nstep),
               "what": f"full {p.nstep}-step shot: plan creation with model upload from page-locked host "
                       f"arrays, run, seismogram read-back into a page-locked buffer",
               "seconds": t_e2e, "create_s": t1 - t0, "run_s": t2 - t1, "read_s": t3 - t2}
        if rank == 0 and not args.no_accuracy:
            accuracy = shot_accuracy(p, cp, cs, rho, seis, [shot.field(c) for c in range(9)])
        shot.close()
    clk = clocks.stop()

    bpc = bytes_per_cell(p.nx, p.ny, p.nz, p.npml)
    peak, peak_kind = measured_peaks()
    kern = {}
    for name, tot, n, b in (("stress_kernel", s_ms, ns, bpc["stress"]), ("velocity_kernel", v_ms, nv, bpc["velocity"])):
        if not n:
            continue
        per = tot / n / 1e3
        ach = b * cells / per / 1e9
        kern[name] = {"launches": n, "mean_ms": per * 1e3, "bytes_per_launch": b * cells, "achieved_gbs": ach,
                      "frac": ach / measured_peaks()[0]}
        if two_path:
            kern[name]["path"] = two_path
    if f_launches:
        per_step = f_ms / f_steps / 1e3
        kern["flow_kernel"] = {"launches": f_launches, "steps": f_steps, "mean_ms": f_ms / f_launches,
                               "ms_per_step": per_step * 1e3, "bytes_per_step": bpc["step"] * cells,
                               "achieved_gbs": bpc["step"] * cells / per_step / 1e9}
    # the dominant kernel of the path the timed run used
    dom = "flow_kernel" if f_launches else max(kern, key=lambda k: kern[k]["mean_ms"])
    # the dataflow kernel runs many steps per launch: its achieved rate and
    # traffic are per time step
    traffic = profile_traffic(dom, "dram_bytes_per_step_full_grid" if dom == "flow_kernel"
                              else "dram_bytes_per_launch_full_grid")
    roof = {"bound": "hbm", "kernel": dom, "achieved": kern[dom]["achieved_gbs"], "peak": peak, "unit": "GB/s",
            "frac": kern[dom]["achieved_gbs"] / peak, "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
            "traffic": traffic, "traffic_per": "time step" if dom == "flow_kernel" else "launch",
            "bytes_per_cell_update": bpc["step"],
            "step_achieved_gbs": bpc["step"] * cells * args.steps / (ms / 1e3) / 1e9,
            "kernels": kern}
    roof["step_frac"] = roof["step_achieved_gbs"] / peak

    extra = {}
    if rank == 0 and world == 1 and not args.no_c0:
        extra["c0"] = homogeneous_101(args)
    if args.large > 0 and rank == 0 and not args.no_batched:
        extra["large_grid"] = large_grid(args.large)
    if not args.no_batched:
        extra["batched"] = batched_shots(args, value, e2e["value"] if e2e else None)   # shots split across ranks
        if world == 1 and not args.batched_only:
            extra["uneven"] = uneven_batch(args)
            extra["serving"] = serving(args)

    cpu = None
    ref_gpu = ref_gpu64 = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            cpu = cpu_reference_rate(p, cp, cs, rho, steps=args.cpu_steps, procs=1)
        except Exception as e:  # reported, not fatal
            cpu = {"value": None, "error": str(e)}
        try:
            ref_gpu = reference_gpu_rate(p.nx, steps=200, warm=10)
            if ref_gpu.get("value"):
                ref_gpu["ours_over_reference_gpu"] = value / ref_gpu["value"]
        except Exception as e:  # reported, not fatal
            ref_gpu = {"value": None, "error": str(e)}
        try:
            # an edge divisible by its 5-thread blocks, so they cover the grid
            ref_gpu64 = reference_gpu_rate(255, steps=50, warm=5, program="ref_gpu_f64")
            ours64 = fp64_rate(255, steps=50)
            ref_gpu64["ours_fp64_same_grid"] = ours64
            if ref_gpu64.get("value"):
                ref_gpu64["ours_fp64_over_reference_gpu_fp64"] = ours64["value"] / ref_gpu64["value"]
        except Exception as e:  # reported, not fatal
            ref_gpu64 = {"value": None, "error": str(e)}
    dist.close()
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t_max * 1e3 / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded anticline model)",
                "config": config_block(p, {"steps_timed": args.steps, "tuning": tune_info}),
                "e2e": e2e, "gpu_launches": int(launches * world), "roofline": roof,
                "cpu_baseline": cpu, "reference_gpu_program": ref_gpu, "reference_gpu_program_fp64": ref_gpu64,
                "clocks": clk, "accuracy": accuracy}
        line.update(extra)
        print(json.dumps(line), flush=True)


def large_grid(n: int, steps: int = 100) -> dict:
    """One n^3 shot of the same anticline, its model generated on the device
    (no host arrays): the single-shot rate where the C-PML layers are a
    smaller share of the cells (--large N; 0 turns it off)."""
    import ela3d_gb300 as E
    from ela3d_gb300 import media
    from ela3d_gb300.metrics import bytes_per_cell

    npml, f0 = 16, 12.0
    p = E.ShotParams(nx=n, ny=n, nz=n, nstep=steps + 20, dt=1e-3, npml=npml, f0=f0, t0=1.2 / f0, factor=1e7,
                     stf=0, src_kind=0, src=(n // 2, n // 2, npml + 3), src_w=(0.0, 0.0, 1.0), sampgat=1,
                     rec=np.array([[x, n // 2, npml + 3] for x in range(n // 2 - 100, n // 2 + 101)], np.int32))
    with E.Plan.from_model(p, media.anticline_256_spec(n)) as plan:
        plan.run(20)
        ms = plan.run_timed(steps)
        info = plan.info()
    cells = p.cells
    bpc = bytes_per_cell(n, n, n, npml)["step"]
    peak, _ = measured_peaks()
    value = cells * steps / (ms / 1e3) / 1e9
    return {"workload": f"{n}^3 anticline (16 PML cells), model generated on the GPU, FP32", "metric": METRIC,
            "value": value, "steps_timed": steps, "ms_per_step": ms / steps, "bytes_per_cell_update": bpc,
            "frac_of_hbm": value * 1e9 * bpc / 1e9 / peak, "device_bytes": int(info.device_bytes),
            "timing": "CUDA events around replayed 50-step graphs, built-in kernel choice"}


def fp64_rate(n: int, steps: int) -> dict:
    """This library's FP64 build on an n^3 anticline (model generated on the
    GPU), built-in kernel choice: the rate beside the reference's FP64 GPU
    program at the same grid size."""
    import ela3d_gb300 as E
    from ela3d_gb300 import media

    npml, f0 = 16, 12.0
    p = E.ShotParams(nx=n, ny=n, nz=n, nstep=steps + 5, dt=1e-3, npml=npml, f0=f0, t0=1.2 / f0, src=(n // 2, n // 2, npml + 3),
                     precision=1)
    with E.Plan.from_model(p, media.anticline_256_spec(n)) as plan:
        plan.run(5)
        ms = plan.run_timed(steps)
    return {"value": n ** 3 * steps / (ms / 1e3) / 1e9, "unit": METRIC, "ms_per_step": ms / steps,
            "what": f"this library's FP64 build, {n}^3 anticline, {steps} steps, CUDA events"}


def homogeneous_101(args) -> dict:
    """The 101^3 homogeneous cube (10 PML cells, 1000 steps): FP32 and FP64
    device rates with the built-in kernel choice, the HBM fraction at its
    152.5 B (FP32) per cell-update, one full shot end to end, its accuracy
    against the reference CPU program's own FP32 and FP64 runs of the same
    shot (the committed fixture tests/golden/ref_homogeneous_101_full.npz),
    and the reference program's FP32 and FP64 rates on one core."""
    import ela3d_gb300 as E
    from ela3d_gb300 import configs
    from ela3d_gb300.metrics import bytes_per_cell

    p, cp, cs, rho = configs.homogeneous_101()
    cells = p.cells
    peak, _ = measured_peaks()
    steps = args.c0_steps
    out = {"workload": "homogeneous_101: 101^3 cube, cp 3300 m/s, cs cp/1.732, rho 2800, dt 1.6e-3 s, "
                       "1000-step shot, 10 PML cells, Ricker 7 Hz on vz at the centre, 11 receivers",
           "metric": METRIC}
    seis = {}
    tune = {}
    if args.c0_schedule >= 0:   # explicit choice for the FP32 shot (profiling comparisons)
        tune = {"schedule": args.c0_schedule, "chunk": max(args.c0_chunk, 0)}
    if args.c0_variant >= 0:
        tune["variant"] = args.c0_variant
    if tune:
        out["tuning"] = tune
    for tag, prec in (("fp32", 0), ("fp64", 1)):
        q = p.with_(precision=prec)
        bpc = bytes_per_cell(p.nx, p.ny, p.nz, p.npml, word=8 if prec else 4)["step"]
        with E.Plan(q, cp, cs, rho, **(tune if prec == 0 else {})) as pl:   # built-in kernel choice
            pl.run(args.warmup)
            ms = pl.run_timed(steps)
            pl.set_kernel_timing(True)
            pl.run(min(steps, 200))
            f_ms, f_launches, f_steps = pl.flow_timing()
            s_ms, v_ms, ns, nv = pl.kernel_timing()
        rate = cells * steps / (ms / 1e3) / 1e9
        row = {"value": rate, "ms_per_step": ms / steps, "steps_timed": steps, "bytes_per_cell_update": bpc,
               "frac_of_hbm": rate * bpc / peak}
        if f_launches:
            per = f_ms / f_steps
            row["kernel"] = {"name": "flow_kernel", "launches": f_launches, "steps": f_steps,
                             "ms_per_step": per, "achieved_gbs": bpc * cells / per / 1e6,
                             "frac": bpc * cells / per / 1e6 / peak}
        elif ns:
            per = (s_ms + v_ms) / ns
            row["kernel"] = {"name": "stress_kernel + velocity_kernel", "launches": ns + nv,
                             "ms_per_step": per, "achieved_gbs": bpc * cells / per / 1e6,
                             "frac": bpc * cells / per / 1e6 / peak}
        out[tag] = row
        # one whole shot end to end through the C ABI from page-locked host
        # arrays (as the headline shot's end-to-end rate)
        host = [E.pinned_copy(a, np.float32) for a in (cp, cs, rho)]
        out_buf = E.pinned_empty((q.nrec, 3, q.nsamp), np.float64 if prec else np.float32)
        t0 = time.perf_counter()
        with E.Plan(q, *host) as pl:
            pl.run(p.nstep)
            seis[tag] = pl.seismograms(fp64=bool(prec), out=out_buf)
        row["e2e"] = {"value": cells * p.nstep / (time.perf_counter() - t0) / 1e9, "unit": METRIC,
                      "what": f"full {p.nstep}-step shot: plan creation with model upload from page-locked host "
                              f"arrays, run, seismogram read-back into a page-locked buffer"}
    # accuracy against the reference program's own runs of this shot
    gold = os.path.join(ROOT, "tests", "golden", "ref_homogeneous_101_full.npz")
    if os.path.exists(gold):
        g = np.load(gold)
        rel = lambda a, b: float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))  # noqa: E731
        per = lambda a, b: max(rel(a[r], b[r]) for r in range(b.shape[0]) if np.any(b[r]))  # noqa: E731
        r64 = g["seis_f64"]
        out["accuracy_vs_reference_program"] = {
            "what": "relative L2 of the seismograms against the reference CPU program's runs of the same shot",
            "fp32_gpu_vs_fp64_program": {"all": rel(seis["fp32"], r64), "worst_seismogram": per(seis["fp32"], r64)},
            "fp32_gpu_vs_fp32_program": {"all": rel(seis["fp32"], g["seis_f32"].astype(np.float64))},
            "fp32_program_vs_fp64_program": {"all": rel(g["seis_f32"], r64), "worst_seismogram": per(g["seis_f32"], r64)},
            "fp64_gpu_vs_fp64_program": {"all": rel(seis["fp64"], r64), "worst_seismogram": per(seis["fp64"], r64)}}
    if not args.no_cpu_baseline:
        for tag, fp64 in (("fp32", False), ("fp64", True)):
            try:
                out[f"cpu_reference_{tag}"] = cpu_reference_rate(p, cp, cs, rho, steps=args.c0_cpu_steps, procs=1,
                                                                 fp64=fp64)
            except Exception as e:  # reported, not fatal
                out[f"cpu_reference_{tag}"] = {"value": None, "error": str(e)}
    out["timing"] = ("CUDA events around the library's run (built-in kernel choice), after warm-up; kernel row: "
                     "per-launch CUDA events of a second pass; e2e: wall clock")
    return out


def batched_shots(args, single_value: float, single_wall_value: float | None = None) -> dict:
    """64 shots of the 256^3 anticline (8 x 8 source grid at z = npml + 3,
    one shared model) advanced together; graph replay, CUDA-event timing.
    Compared with the single-shot path both device time to device time and
    wall clock to wall clock (batch creation, run and read-back against one
    whole shot's end-to-end rate)."""
    import ela3d_gb300 as E
    from ela3d_gb300 import configs
    from ela3d_gb300.metrics import bytes_per_cell

    shots, cp, cs, rho = configs.anticline_256_shots(args.batch_shots)
    rank, world, _ = dist_env()
    shots = shard(shots, rank, world)   # independent shots: no data-path collective
    cells = sum(p.cells for p in shots)
    tune = {"schedule": args.batch_schedule, "chunk": args.batch_chunk}
    tune_info = {"source": "command line"}
    if not args.no_autotune:
        # tuned on 16 of the shots over 10 steps: with 8 shots and 5 steps the
        # pick varied between runs and at times chose a tile 3% slower for
        # the whole batch
        best, _, cand = E.autotune([(p, cp, cs, rho) for p in shots[:16]], steps=10)
        tune = best.as_dict()
        tune_info = {"source": "ela3d_autotune on 16 of the shots, 10 steps", "candidates": cand, **tune}
    t0 = time.perf_counter()
    with E.Batch([(p, cp, cs, rho) for p in shots], **tune) as b:
        t_create = time.perf_counter() - t0
        b.run(args.warmup)
        ms = b.run_timed(args.batch_steps)
        t1 = time.perf_counter()
        b.run(0)
        seis = [b.seismograms(q) for q in range(len(shots))]
        t_read = time.perf_counter() - t1
        t_wall = time.perf_counter() - t0
    g = Group(world)
    value = g.sum(cells) * args.batch_steps / (g.max(ms) / 1e3) / 1e9
    wall_value = g.sum(cells) * (args.warmup + args.batch_steps) / g.max(t_wall) / 1e9
    # two shots drawn by seed, checked against FP64
    pick = sorted(np.random.default_rng(2024).choice(len(shots), size=min(2, len(shots)), replace=False).tolist())
    steps_run = args.warmup + args.batch_steps
    check = fp64_check([(f"shot {q}", shots[q], cp, cs, rho, steps_run, seis[q]) for q in pick])
    bpc = bytes_per_cell(256, 256, 256, 16)["step"]
    peak, _ = measured_peaks()
    return {"workload": f"anticline_256_shots: {len(shots)} shots of 256^3 sharing one model, FP32, "
                        f"8x8 source grid at z=19, 201-receiver line each",
            "metric": METRIC, "value": value, "steps_timed": args.batch_steps,
            "ms_per_step": ms / args.batch_steps, "single_shot_value": single_value,
            "ratio_vs_single_shot": value / single_value,
            "wall_value": wall_value, "single_shot_wall_value": single_wall_value,
            "ratios": {"device_over_device": value / single_value,
                       "wall_over_wall": wall_value / single_wall_value if single_wall_value else None},
            "frac_of_hbm_at_142B": value * bpc / peak,
            "create_s": t_create, "readback_s": t_read,
            "tuning": tune_info, "fp64_check": check,
            "timing": "CUDA events around replayed 50-step graphs; model stored once"}


def uneven_batch(args) -> dict:
    """48 grids with edges from multiples of 16 in [64, 320] (seed 1): all
    together vs the same instances one at a time (each alone on the GPU)."""
    import ela3d_gb300 as E
    from ela3d_gb300 import configs
    from ela3d_gb300.metrics import bytes_per_cell

    inst = configs.uneven_batch(count=args.uneven_count)
    steps = args.uneven_steps
    cells = sum(p.cells for p, *_ in inst)
    tune = {}
    tune_info = {"source": "built-in default"}
    if not args.no_autotune:
        # the batch is known in advance: tuned on all of it (3 steps per candidate)
        best, _, cand = E.autotune(inst, steps=3)
        tune = best.as_dict()
        tune_info = {"source": "ela3d_autotune on the whole batch", "candidates": cand, **tune}
    # each instance alone, with the better of the built-in and the tuned
    # kernel choice per instance
    alone_default_s = alone_s = alone_wall_s = 0.0
    for p, cp, cs, rho in inst:
        times = []
        for kw in [{}] + ([tune] if tune else []):
            t0 = time.perf_counter()
            with E.Plan(p, cp, cs, rho, **kw) as pl:
                pl.run(3)
                times.append(pl.run_timed(steps) / 1e3)
                pl.seismograms()
            if not kw:   # wall clock of the plain path: creation, run, read-back
                alone_wall_s += time.perf_counter() - t0
        alone_default_s += times[0]
        alone_s += min(times)
    alone = cells * steps / alone_s / 1e9
    t0 = time.perf_counter()
    with E.Batch(inst, **tune) as b:
        b.run(3)
        ms = b.run_timed(steps)
        # two instances drawn by seed, as computed in the batch, against FP64
        pick = sorted(np.random.default_rng(2).choice(len(inst), 2, replace=False).tolist())
        seis = {q: b.seismograms(q) for q in pick}
        for q in range(len(inst)):
            b.seismograms(q)
    batch_wall_s = time.perf_counter() - t0
    value = cells * steps / (ms / 1e3) / 1e9
    wall_value = cells * (steps + 3) / batch_wall_s / 1e9
    alone_wall = cells * (steps + 3) / alone_wall_s / 1e9
    sizes = [p.cells for p, *_ in inst]
    check = fp64_check([(f"instance {q}", *inst[q], 3 + steps, seis[q]) for q in pick])
    # algorithmic bytes of one step of every instance (each at its own PML share)
    step_bytes = sum(p.cells * bytes_per_cell(p.nx, p.ny, p.nz, p.npml)["step"] for p, *_ in inst)
    peak, _ = measured_peaks()
    return {"workload": f"uneven_batch: {len(inst)} grids, edges from multiples of 16 in [64, 320] (seed 1), "
                        f"{min(sizes) / 1e6:.2f}-{max(sizes) / 1e6:.1f} Mcells, random 3-6 layer domes, FP32",
            "metric": METRIC, "value": value, "steps_timed": steps,
            "single_shot_sequential_value": alone, "single_shot_default_value": cells * steps / alone_default_s / 1e9,
            "ratio_vs_single_shot": value / alone, "tuning": tune_info,
            "wall_value": wall_value, "single_shot_sequential_wall_value": alone_wall,
            "ratios": {"device_over_device": value / alone, "wall_over_wall": wall_value / alone_wall},
            "bytes_per_cell_update": step_bytes / cells,
            "frac_of_hbm": step_bytes * steps / (ms / 1e3) / 1e9 / peak,
            "single_shot_frac_of_hbm": step_bytes * steps / alone_s / 1e9 / peak, "fp64_check": check,
            "timing": "CUDA events; the same steps of every instance, batched vs one plan at a time (each "
                      "with the better of the built-in and the tuned kernel choice; default value: built-in only)"}


def serving(args) -> dict:
    """Request stream with Poisson arrivals, swept to saturation.  Requests
    are seeded draws of configs.serving_request (lognormal edges in
    [64, 384]); the stream is a bounded sample: `serve_count` requests
    simulating `serve_t_end` seconds each (the full stream is 2000 requests
    of 2 s).  Compared with the same requests run one at a time."""
    import threading

    import ela3d_gb300 as E
    from ela3d_gb300 import configs
    from ela3d_gb300.metrics import bytes_per_cell

    reqs = [configs.serving_request(1000 + q, t_end=args.serve_t_end) for q in range(args.serve_count)]
    work = [p.cells * p.nstep for p, *_ in reqs]
    total = float(sum(work))
    tune = {}
    tune_info = {"source": "built-in default"}
    if not args.no_autotune:
        # tuned on every eighth request (a cross-section of the sizes)
        best, _, cand = E.autotune(reqs[::8], steps=5)
        tune = best.as_dict()
        tune_info = {"source": "ela3d_autotune on every eighth request", "candidates": cand, **tune}
    # the plain single-shot path: each request alone, device time of its run,
    # with the better of the built-in and the tuned kernel choice per request
    t0 = time.perf_counter()
    alone_each = []
    for p, cp, cs, rho in reqs:
        with E.Plan(p, cp, cs, rho) as pl:
            alone_each.append(pl.run_timed(p.nstep) / 1e3)
            pl.seismograms()
    alone_wall = time.perf_counter() - t0
    alone_default_s = sum(alone_each)
    if tune:
        for q, (p, cp, cs, rho) in enumerate(reqs):
            with E.Plan(p, cp, cs, rho, **tune) as pl:
                alone_each[q] = min(alone_each[q], pl.run_timed(p.nstep) / 1e3)
    alone_s = sum(alone_each)
    alone = total / alone_s / 1e9
    rng = np.random.default_rng(7)
    capacity = None
    rows = []
    served = {}
    for load in args.serve_loads:
        with E.Server(steps_per_round=args.serve_round, **tune) as srv:
            gaps = None
            if load > 0 and capacity:
                rate = load * capacity                       # requests per second
                gaps = rng.exponential(1.0 / rate, len(reqs))
            tickets = []

            def client():
                for q, r in enumerate(reqs):
                    if gaps is not None:
                        time.sleep(gaps[q])
                    tickets.append(srv.submit(*r))

            t_start = time.perf_counter()
            th = threading.Thread(target=client)
            th.start()
            th.join()
            for t in tickets:
                srv.wait(t)
            wall = time.perf_counter() - t_start
            st = srv.stats()
            if load == 0:   # every 50th request, as served in FP32
                served = {q: srv.read(tickets[q]) for q in range(0, len(reqs), 50)}
        thr = total / wall / 1e9
        busy = total / st["busy_seconds"] / 1e9
        if load == 0:
            capacity = len(reqs) / wall
        rows.append({"offered_load": "saturation" if load == 0 else load,
                     "arrival_rate_per_s": None if load == 0 else load * capacity,
                     "requests": len(reqs), "gcells_per_s_wall": thr, "gcells_per_s_busy": busy,
                     "p50_latency_s": st["latency_p50_s"], "p99_latency_s": st["latency_p99_s"],
                     "max_latency_s": st["latency_max_s"], "rounds": st["rounds"], "failed": st["failed"]})
    sat = rows[0]
    # the same saturated stream with a fill target: admission in arrival
    # order only while the running shots hold fewer cells than the target
    with E.Server(steps_per_round=args.serve_round, fill_cells=args.serve_fill, **tune) as srv:
        t_start = time.perf_counter()
        tickets = [srv.submit(*r) for r in reqs]
        for t in tickets:
            srv.wait(t)
        wall = time.perf_counter() - t_start
        st = srv.stats()
    fill_row = {"fill_cells": args.serve_fill, "gcells_per_s_wall": total / wall / 1e9,
                "p50_latency_s": st["latency_p50_s"], "p99_latency_s": st["latency_p99_s"],
                "max_latency_s": st["latency_max_s"], "rounds": st["rounds"]}
    sizes = [p.cells for p, *_ in reqs]
    # algorithmic bytes of the whole stream (each request at its own PML share)
    stream_bytes = sum(p.cells * p.nstep * bytes_per_cell(p.nx, p.ny, p.nz, p.npml)["step"] for p, *_ in reqs)
    peak, _ = measured_peaks()
    busy_s = total / (sat["gcells_per_s_busy"] * 1e9)
    check = fp64_check([(f"request {q}", *reqs[q], reqs[q][0].nstep, s) for q, s in served.items()])
    return {"workload": f"serving stream: {len(reqs)} requests (seeded lognormal edges in [64, 384], "
                        f"{min(sizes) / 1e6:.2f}-{max(sizes) / 1e6:.1f} Mcells, t_end {args.serve_t_end} s "
                        f"each; the full stream is 2000 requests of 2 s), FP32",
            "metric": METRIC, "value": sat["gcells_per_s_wall"], "p50_latency_s": sat["p50_latency_s"],
            "p99_latency_s": sat["p99_latency_s"],
            "single_shot_sequential_value": alone, "single_shot_default_value": total / alone_default_s / 1e9,
            "single_shot_sequential_wall_value": total / alone_wall / 1e9, "tuning": tune_info,
            "ratio_vs_single_shot": sat["gcells_per_s_wall"] / alone,
            "ratios": {"device_over_device": sat["gcells_per_s_busy"] / alone,
                       "wall_over_wall": sat["gcells_per_s_wall"] / (total / alone_wall / 1e9)},
            "bytes_per_cell_update": stream_bytes / total,
            "frac_of_hbm_busy": stream_bytes / busy_s / 1e9 / peak,
            "single_shot_frac_of_hbm": stream_bytes / alone_s / 1e9 / peak,
            "sweep": rows, "saturation_with_fill_target": fill_row, "steps_per_round": args.serve_round,
            "fp64_check": check,
            "timing": "wall clock from first submission to last completion (requests submitted from host "
                      "arrays, seismograms streamed back); single-shot value = device time of each request "
                      "run alone with the better of the built-in and the tuned kernel choice (default value: "
                      "built-in choice only; wall value: built-in choice, plan creation and read-back included)"}


# ------------------------------------------------- full-size configs --
def single_shot_rates(tune: dict) -> dict:
    """One whole 2000-step 256^3 anticline shot: device rate (CUDA events)
    and end-to-end wall rate (plan creation with the model upload, run,
    seismogram read-back)."""
    import ela3d_gb300 as E

    p, cp, cs, rho = workload()
    t0 = time.perf_counter()
    with E.Plan(p, cp, cs, rho, **tune) as pl:
        ms = pl.run_timed(p.nstep)
        pl.seismograms()
    wall = time.perf_counter() - t0
    return {"value": p.cells * p.nstep / (ms / 1e3) / 1e9, "wall_value": p.cells * p.nstep / wall / 1e9,
            "steps": p.nstep}


def uneven_full(args) -> dict:
    """The 48 uneven grids each run to t = 2 s (its own nstep), all in one
    batch (shots retire at their nstep) against each alone for its nstep."""
    import ela3d_gb300 as E
    from ela3d_gb300 import configs
    from ela3d_gb300.metrics import bytes_per_cell

    inst = configs.uneven_batch(count=args.uneven_count)
    work = float(sum(p.cells * p.nstep for p, *_ in inst))
    tune, tune_info = {}, {"source": "built-in default"}
    if not args.no_autotune:
        best, _, cand = E.autotune(inst, steps=3)
        tune = best.as_dict()
        tune_info = {"source": "ela3d_autotune on the whole batch", "candidates": cand, **tune}
    alone_s = alone_wall_s = 0.0
    for p, cp, cs, rho in inst:
        t0 = time.perf_counter()
        with E.Plan(p, cp, cs, rho) as pl:   # the plain path: built-in choice
            alone_s += pl.run_timed(p.nstep) / 1e3
            pl.seismograms()
        alone_wall_s += time.perf_counter() - t0
    longest = max(p.nstep for p, *_ in inst)
    pick = sorted(np.random.default_rng(2).choice(len(inst), 2, replace=False).tolist())
    t0 = time.perf_counter()
    with E.Batch(inst, **tune) as b:
        ms = b.run_timed(longest)
        seis = {q: b.seismograms(q) for q in range(len(inst))}
    wall_s = time.perf_counter() - t0
    check = fp64_check([(f"instance {q}", *inst[q], inst[q][0].nstep, seis[q]) for q in pick])
    step_bytes = sum(p.cells * p.nstep * bytes_per_cell(p.nx, p.ny, p.nz, p.npml)["step"] for p, *_ in inst)
    peak, _ = measured_peaks()
    value = work / (ms / 1e3) / 1e9
    alone = work / alone_s / 1e9
    return {"workload": f"uneven_batch at its named size: {len(inst)} grids, each to t = 2 s "
                        f"({min(p.nstep for p, *_ in inst)}-{longest} steps), FP32",
            "metric": METRIC, "value": value, "wall_value": work / wall_s / 1e9, "cell_updates": work,
            "single_shot_sequential_value": alone, "single_shot_sequential_wall_value": work / alone_wall_s / 1e9,
            "ratios": {"device_over_device": value / alone, "wall_over_wall": alone_wall_s / wall_s},
            "frac_of_hbm": step_bytes / (ms / 1e3) / 1e9 / peak, "tuning": tune_info, "fp64_check": check,
            "timing": "device: CUDA events around the batch run (shots retire at their nstep) and around each "
                      "instance alone (built-in choice); wall: creation, run and read-back of all instances"}


def serving_full(args) -> dict:
    """The serving stream at its named size: 2000 requests of 2 s simulated
    time (lognormal edges in [64, 384], per-request seeded models generated
    on the GPU at admission), all submitted at once (saturation) and with
    Poisson arrivals at a fraction of that rate; every 50th request re-run
    alone in FP64; the plain single-shot path timed on every 10th request."""
    import threading

    import ela3d_gb300 as E
    from ela3d_gb300 import configs
    from ela3d_gb300.metrics import bytes_per_cell

    n = args.full_serve_count
    reqs = [configs.serving_request_spec(1000 + q, t_end=2.0) for q in range(n)]
    work = [float(p.cells * p.nstep) for p, _ in reqs]
    total = sum(work)
    tune, tune_info = {}, {"source": "built-in default"}
    if not args.no_autotune:
        # tuned on eight requests spread over the stream, with host models
        sample = [configs.serving_request(1000 + q, t_end=0.25) for q in range(0, n, max(1, n // 8))][:8]
        best, _, cand = E.autotune(sample, steps=5)
        tune = best.as_dict()
        tune_info = {"source": "ela3d_autotune on eight requests", "candidates": cand, **tune}
    # the plain single-shot path on every 10th request
    sub = list(range(0, n, 10))
    sub_work = sum(work[q] for q in sub)
    alone_s = alone_wall_s = 0.0
    for q in sub:
        p, spec = reqs[q]
        t0 = time.perf_counter()
        with E.Plan.from_model(p, spec) as pl:
            alone_s += pl.run_timed(p.nstep) / 1e3
            pl.seismograms()
        alone_wall_s += time.perf_counter() - t0
    alone, alone_wall = sub_work / alone_s / 1e9, sub_work / alone_wall_s / 1e9
    rows, served, capacity = [], {}, None
    rng = np.random.default_rng(7)
    for load in args.full_serve_loads:
        with E.Server(steps_per_round=args.serve_round, **tune) as srv:
            gaps = rng.exponential(1.0 / (load * capacity), n) if load > 0 and capacity else None
            tickets = []

            def client():
                for q, (p, spec) in enumerate(reqs):
                    if gaps is not None:
                        time.sleep(gaps[q])
                    tickets.append(srv.submit_model(p, spec))

            t_start = time.perf_counter()
            th = threading.Thread(target=client)
            th.start()
            th.join()
            for q, t in enumerate(tickets):
                srv.wait(t)
                if load == 0 and q % 50 == 0:
                    served[q] = srv.read(t)
                srv.release(t)
            wall = time.perf_counter() - t_start
            st = srv.stats()
        if load == 0:
            capacity = n / wall
        rows.append({"offered_load": "saturation" if load == 0 else load,
                     "arrival_rate_per_s": None if load == 0 else load * capacity, "requests": n,
                     "gcells_per_s_wall": total / wall / 1e9, "gcells_per_s_busy": total / st["busy_seconds"] / 1e9,
                     "p50_latency_s": st["latency_p50_s"], "p99_latency_s": st["latency_p99_s"],
                     "max_latency_s": st["latency_max_s"], "rounds": st["rounds"], "failed": st["failed"],
                     "wall_s": wall})
    sat = rows[0]
    # every 50th request alone in FP64 (model generated on the device)
    chk = []
    for q, s32 in served.items():
        p, spec = reqs[q]
        with E.Plan.from_model(p.with_(precision=1), spec) as pl:
            pl.run(p.nstep)
            s64 = pl.seismograms(fp64=True)
        a, b = s32.astype(np.float64), s64
        chk.append(float(np.linalg.norm(a - b) / np.linalg.norm(b)))
    stream_bytes = sum(p.cells * p.nstep * bytes_per_cell(p.nx, p.ny, p.nz, p.npml)["step"] for p, _ in reqs)
    peak, _ = measured_peaks()
    sizes = [p.cells for p, _ in reqs]
    return {"workload": f"serving stream at its named size: {n} requests of 2 s simulated time (seeded lognormal "
                        f"edges in [64, 384], {min(sizes) / 1e6:.2f}-{max(sizes) / 1e6:.1f} Mcells, models "
                        f"generated on the GPU at admission), FP32",
            "metric": METRIC, "value": sat["gcells_per_s_wall"], "cell_updates": total,
            "p50_latency_s": sat["p50_latency_s"], "p99_latency_s": sat["p99_latency_s"],
            "single_shot_sequential_value": alone, "single_shot_sequential_wall_value": alone_wall,
            "single_shot_sample": f"every 10th request ({len(sub)}) alone, built-in choice",
            "ratios": {"device_over_device": sat["gcells_per_s_busy"] / alone,
                       "wall_over_wall": sat["gcells_per_s_wall"] / alone_wall},
            "frac_of_hbm_busy": stream_bytes / (total / (sat["gcells_per_s_busy"] * 1e9)) / 1e9 / peak,
            "sweep": rows, "tuning": tune_info, "steps_per_round": args.serve_round,
            "fp64_check": {"what": "every 50th request's FP32 seismograms as served vs the request re-run alone in "
                                   "FP64 (relative L2)", "requests": len(chk), "max_rel_l2": max(chk) if chk else None,
                           "median_rel_l2": float(np.median(chk)) if chk else None}}


def run_full(args) -> None:
    """--full: the named configurations at their full sizes (opt-in; minutes
    of GPU time each), one JSON line."""
    import ela3d_gb300 as E

    E.select_device(0)
    clocks = ClockSampler(0)
    clocks.start()
    out = {"metric": METRIC, "full_configs": {}}
    if "batched" in args.full:
        single = single_shot_rates({})
        args.batch_steps = 2000
        out["full_configs"]["batched"] = batched_shots(args, single["value"], single["wall_value"])
        out["full_configs"]["batched"]["single_shot"] = single
    if "uneven" in args.full:
        out["full_configs"]["uneven"] = uneven_full(args)
    if "serve" in args.full:
        out["full_configs"]["serving"] = serving_full(args)
    out["clocks"] = clocks.stop()
    print(json.dumps(out), flush=True)


def run_reference(args, rank, world, local):
    if rank != 0:
        return
    p, cp, cs, rho = workload()
    procs = os.cpu_count() or 1
    steps = max(1, min(args.steps, args.ref_steps_cap))
    r = cpu_reference_rate(p, cp, cs, rho, steps=steps, procs=procs)
    line = {"metric": METRIC, "value": r["value"], "unit": METRIC, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r["seconds"] * 1e3 / steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded anticline model)",
            "impl": "reference", "config": config_block(p, {"steps_timed": steps}),
            "cpu_baseline": {k: r[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": r["value"], "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end shot (short profiling runs)")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the FP64 re-run of the end-to-end shot (accuracy of every seismogram and field)")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the batched, uneven, serving and larger-grid workloads")
    ap.add_argument("--batched-only", action="store_true",
                    help="of the batched, uneven and serving workloads run only the first (profiling runs)")
    ap.add_argument("--no-autotune", action="store_true", help="use the built-in kernel choice")
    ap.add_argument("--prefetch", type=int, default=-1,
                    help="C-PML memory-variable prefetch mode of the single-shot plan (ela3d_tuning.prefetch: "
                         "0 none, 2 x slab into L1, 6 also y/z slabs into L2); -1 = tuned or built-in")
    ap.add_argument("--large", type=int, default=512,
                    help="also time one N^3 anticline shot generated on the GPU (0: off)")
    ap.add_argument("--variant", type=int, default=-1,
                    help="kernel variant (tile shape, stages) of the single-shot plan, an index of "
                         "ela3d_gb300.variants(); -1 = tuned or built-in")
    ap.add_argument("--schedule", type=int, default=-1,
                    help="work schedule of the single-shot plan (0 contiguous shares, 1 z-chunks round-robin); "
                         "-1 = tuned or built-in")
    ap.add_argument("--chunk", type=int, default=-1, help="z-chunk planes for --schedule 1; -1 = tuned or built-in")
    ap.add_argument("--batch-shots", type=int, default=64)
    ap.add_argument("--batch-steps", type=int, default=100)
    ap.add_argument("--batch-schedule", type=int, default=2)
    ap.add_argument("--batch-chunk", type=int, default=16)
    ap.add_argument("--uneven-count", type=int, default=48)
    ap.add_argument("--uneven-steps", type=int, default=100)
    ap.add_argument("--serve-count", type=int, default=64)
    ap.add_argument("--serve-t-end", type=float, default=0.25)
    ap.add_argument("--serve-round", type=int, default=50)
    ap.add_argument("--kernel-steps", type=int, default=200,
                    help="steps of the per-kernel CUDA-event pass behind the roofline")
    ap.add_argument("--serve-fill", type=int, default=16_000_000,
                    help="fill target (cells) of the extra saturated serving run")
    ap.add_argument("--serve-loads", type=float, nargs="+", default=[0.0, 0.3, 0.6, 0.9],
                    help="offered load as a fraction of the measured saturation rate (0 = all at once)")
    ap.add_argument("--cpu-steps", type=int, default=50,
                    help="time steps of the one-core CPU baseline sample (about 15 s of CPU work)")
    ap.add_argument("--ref-steps-cap", type=int, default=20)
    ap.add_argument("--no-c0", action="store_true", help="skip the 101^3 homogeneous-cube block")
    ap.add_argument("--c0-steps", type=int, default=400, help="timed steps of the 101^3 cube")
    ap.add_argument("--c0-cpu-steps", type=int, default=100,
                    help="steps of the 101^3 one-core reference CPU samples (about 1-3 s each)")
    ap.add_argument("--c0-only", action="store_true", help="print only the 101^3 block (profiling runs)")
    ap.add_argument("--c0-schedule", type=int, default=-1,
                    help="schedule of the 101^3 FP32 shot (0-4); -1 = built-in choice")
    ap.add_argument("--c0-chunk", type=int, default=0, help="z-chunk planes with --c0-schedule")
    ap.add_argument("--c0-variant", type=int, default=-1,
                    help="kernel variant of the 101^3 FP32 shot (an index of ela3d_gb300.variants()); -1 = built-in")
    ap.add_argument("--full", nargs="+", default=[], choices=["batched", "uneven", "serve"],
                    help="instead of the default line: the named batched, uneven and serving configurations at "
                         "their full sizes (64 shots x 2000 steps; 48 grids to t = 2 s; 2000 requests of 2 s)")
    ap.add_argument("--full-serve-count", type=int, default=2000)
    ap.add_argument("--full-serve-loads", type=float, nargs="+", default=[0.0, 0.8],
                    help="offered loads of the full serving stream (0 = all submitted at once)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank, world, local = dist_env()
    if args.full:
        if rank == 0:
            run_full(args)
        return
    if args.c0_only:
        if rank == 0:
            import ela3d_gb300 as E

            E.select_device(local)
            print(json.dumps({"metric": METRIC, "c0": homogeneous_101(args)}), flush=True)
        return
    if args.impl == "reference":
        run_reference(args, rank, world, local)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
