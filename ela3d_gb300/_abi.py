"""ctypes binding of libela3d.so (include/ela3d.h).

There is no fallback: if the CUDA library is missing or cannot be loaded,
``load_library`` raises.  The library is built in-tree by
``ela3d_gb300._build.build_library`` (``__graft_entry__.build()`` runs it).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .params import CParams, FP64, ShotParams

_LIB = None
LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "libela3d.so")

# (name, restype, argtypes) of every entry point declared in include/ela3d.h
_c = ctypes
_P = _c.c_void_p
# ela3d_request_callback: (ticket, status, user)
REQUEST_CALLBACK = _c.CFUNCTYPE(None, _c.c_uint64, _c.c_int, _c.c_void_p)

SIGNATURES = [
    ("ela3d_version", _c.c_char_p, []),
    ("ela3d_status_string", _c.c_char_p, [_c.c_int]),
    ("ela3d_last_error", _c.c_char_p, []),
    ("ela3d_params_default", _c.c_int, [_c.POINTER(CParams)]),
    ("ela3d_plan_create", _c.c_int, [_c.POINTER(CParams), _P, _P, _P, _c.POINTER(_P)]),
    ("ela3d_run", _c.c_int, [_P, _c.c_int32]),
    ("ela3d_enqueue", _c.c_int, [_P, _c.c_int32]),
    ("ela3d_sync", _c.c_int, [_P]),
    ("ela3d_get_seismograms", _c.c_int, [_P, _P]),
    ("ela3d_get_seismograms_f64", _c.c_int, [_P, _P]),
    ("ela3d_get_field", _c.c_int, [_P, _c.c_int32, _P]),
    ("ela3d_get_source_trace", _c.c_int, [_P, _P]),
    ("ela3d_checkpoint_size", _c.c_int, [_P, _c.POINTER(_c.c_int64)]),
    ("ela3d_checkpoint_save", _c.c_int, [_P, _P, _c.c_int64]),
    ("ela3d_checkpoint_load", _c.c_int, [_P, _P, _c.c_int64]),
    ("ela3d_get_source_trace_f64", _c.c_int, [_P, _P]),
    ("ela3d_get_field_f64", _c.c_int, [_P, _c.c_int32, _P]),
    ("ela3d_energy", _c.c_int, [_P, _c.POINTER(_c.c_double)]),
    ("ela3d_energy_noalloc", _c.c_int, [_P, _P, _P, _P, _c.c_int32, _c.c_int32, _c.c_int32, _c.c_int32,
                                         _c.c_double, _c.c_double, _c.c_double, _P, _P]),
    ("ela3d_plan_info_get", _c.c_int, [_P, _P]),
    ("ela3d_set_kernel_timing", _c.c_int, [_P, _c.c_int32]),
    ("ela3d_get_kernel_timing", _c.c_int, [_P, _c.POINTER(_c.c_double), _c.POINTER(_c.c_double),
                                           _c.POINTER(_c.c_int64), _c.POINTER(_c.c_int64)]),
    ("ela3d_get_flow_timing", _c.c_int, [_P, _c.POINTER(_c.c_double), _c.POINTER(_c.c_int64),
                                         _c.POINTER(_c.c_int64)]),
    ("ela3d_flow_schedule_build", _c.c_int, [_c.c_int32] * 9 + [_c.POINTER(_c.c_int32), _P]),
    ("ela3d_plan_destroy", _c.c_int, [_P]),
    ("ela3d_plan_inject_timeout", _c.c_int, [_P, _c.c_int32]),
    ("ela3d_plan_poison_padding", _c.c_int, [_P, _c.c_double]),
    ("ela3d_plan_get_profiles", _c.c_int, [_P, _c.c_int32, _c.c_void_p]),
    ("ela3d_plan_check_guards", _c.c_int, [_P]),
    ("ela3d_select_device", _c.c_int, [_c.c_int32]),
    ("ela3d_host_alloc", _c.c_int, [_c.c_size_t, _c.POINTER(_P)]),
    ("ela3d_builtin_tuning", _c.c_int, [_c.POINTER(CParams), _P]),
    ("ela3d_host_free", _c.c_int, [_P]),
    ("ela3d_run_timed", _c.c_int, [_P, _c.c_int32, _c.POINTER(_c.c_double)]),
    ("ela3d_slab_extent", _c.c_int, [_P, _P, _c.c_int32, _c.POINTER(_c.c_int32), _c.POINTER(_c.c_int32)]),
    ("ela3d_schedule_build", _c.c_int, [_c.c_int32] * 8 + [_c.POINTER(_c.c_int32), _c.POINTER(_c.c_int32), _P, _P]),
    ("ela3d_batch_create", _c.c_int, [_c.c_int32, _P, _P, _P, _P, _P, _c.POINTER(_P)]),
    ("ela3d_batch_run", _c.c_int, [_P, _c.c_int32]),
    ("ela3d_batch_run_timed", _c.c_int, [_P, _c.c_int32, _c.POINTER(_c.c_double)]),
    ("ela3d_batch_get_seismograms", _c.c_int, [_P, _c.c_int32, _P]),
    ("ela3d_batch_get_field", _c.c_int, [_P, _c.c_int32, _c.c_int32, _P]),
    ("ela3d_batch_get_source_trace", _c.c_int, [_P, _c.c_int32, _P]),
    ("ela3d_batch_info", _c.c_int, [_P, _c.c_int32, _P]),
    ("ela3d_batch_destroy", _c.c_int, [_P]),
    ("ela3d_server_config_default", _c.c_int, [_P]),
    ("ela3d_server_create", _c.c_int, [_P, _c.POINTER(_P)]),
    ("ela3d_server_submit", _c.c_int, [_P, _c.POINTER(CParams), _P, _P, _P, _c.POINTER(_c.c_uint64)]),
    ("ela3d_server_poll", _c.c_int, [_P, _c.c_uint64, _c.POINTER(_c.c_int32), _c.POINTER(_c.c_int32)]),
    ("ela3d_server_read", _c.c_int, [_P, _c.c_uint64, _c.c_int32, _c.c_int32, _P]),
    ("ela3d_server_wait", _c.c_int, [_P, _c.c_uint64, _c.c_int32]),
    ("ela3d_server_cancel", _c.c_int, [_P, _c.c_uint64]),
    ("ela3d_server_release", _c.c_int, [_P, _c.c_uint64]),
    ("ela3d_server_on_done", _c.c_int, [_P, _c.c_uint64, REQUEST_CALLBACK, _c.c_void_p]),
    ("ela3d_server_stats_get", _c.c_int, [_P, _P]),
    ("ela3d_server_destroy", _c.c_int, [_P]),
    ("ela3d_autotune", _c.c_int, [_c.c_int32, _P, _P, _P, _P, _c.c_int32, _P, _c.POINTER(_c.c_double),
                                   _c.POINTER(_c.c_int32)]),
    ("ela3d_plan_create_model", _c.c_int, [_c.POINTER(CParams), _P, _P, _c.POINTER(_P)]),
    ("ela3d_model_generate", _c.c_int, [_P, _c.c_int32, _c.c_int32, _c.c_int32, _P, _P, _P]),
    ("ela3d_server_submit_model", _c.c_int, [_P, _c.POINTER(CParams), _P, _c.POINTER(_c.c_uint64)]),
    ("ela3d_variant_count", _c.c_int32, []),
    ("ela3d_variant_get", _c.c_int, [_c.c_int32, _P]),
    ("ela3d_plan_create_tuned", _c.c_int, [_c.POINTER(CParams), _P, _P, _P, _P, _c.POINTER(_P)]),
]


class PlanInfo(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
                ("pitch_x", ctypes.c_int32), ("step", ctypes.c_int32), ("nsamp", ctypes.c_int32),
                ("nrec", ctypes.c_int32), ("precision", ctypes.c_int32), ("device_bytes", ctypes.c_int64),
                ("slab_lo", ctypes.c_int32 * 3), ("slab_hi", ctypes.c_int32 * 3)]


class VariantInfo(ctypes.Structure):
    _fields_ = [("fp64", ctypes.c_int32), ("tile_x", ctypes.c_int32), ("tile_y", ctypes.c_int32),
                ("stages", ctypes.c_int32), ("threads", ctypes.c_int32), ("stress_smem", ctypes.c_int32),
                ("velocity_smem", ctypes.c_int32), ("loads", ctypes.c_int32),
                ("velocity_stages", ctypes.c_int32)]


class Tuning(ctypes.Structure):
    """ela3d_tuning; -1 / 0 fields leave the choice to the library."""
    _fields_ = [("variant", ctypes.c_int32), ("schedule", ctypes.c_int32), ("chunk", ctypes.c_int32),
                ("blocks_per_sm", ctypes.c_int32), ("prefetch", ctypes.c_int32), ("lag", ctypes.c_int32)]

    def __init__(self, variant: int = -1, schedule: int = -1, chunk: int = 0, blocks_per_sm: int = -1,
                 prefetch: int = -1, lag: int = -1):
        super().__init__(variant, schedule, chunk, blocks_per_sm, prefetch, lag)

    def as_dict(self) -> dict:
        return {"variant": self.variant, "schedule": self.schedule, "chunk": self.chunk, "prefetch": self.prefetch,
                "lag": self.lag}


# the dataflow kernel (many steps per cooperative launch): steps in
# sequence, or overlapping
SCHEDULE_FLOW, SCHEDULE_FLOW_OVERLAP = 3, 4


def flow_schedule(nx, ny, nz, tile_x, tile_y, chunk, gap, overlap, nsteps):
    """The dataflow work list of one shot (ela3d_flow_schedule_build):
    items [n, 6] of (kind, step, chunk, tile, k0, k1) in launch order."""
    lib = load_library()
    n = ctypes.c_int32()
    args = (nx, ny, nz, tile_x, tile_y, chunk, gap, 1 if overlap else 0, nsteps, ctypes.byref(n))
    _check(lib.ela3d_flow_schedule_build(*args, None), "ela3d_flow_schedule_build")
    items = np.zeros((n.value, 6), np.int32)
    _check(lib.ela3d_flow_schedule_build(*args, items.ctypes.data), "ela3d_flow_schedule_build")
    return items


def variants() -> list[VariantInfo]:
    lib = load_library()
    out = []
    for i in range(lib.ela3d_variant_count()):
        v = VariantInfo()
        _check(lib.ela3d_variant_get(i, ctypes.byref(v)), "ela3d_variant_get")
        out.append(v)
    return out


def slab_extent(a_full, a_half) -> tuple[int, int]:
    lib = load_library()
    a = np.ascontiguousarray(a_full, np.float64)
    b = np.ascontiguousarray(a_half, np.float64)
    lo, hi = ctypes.c_int32(), ctypes.c_int32()
    _check(lib.ela3d_slab_extent(a.ctypes.data, b.ctypes.data, a.size, ctypes.byref(lo), ctypes.byref(hi)),
           "ela3d_slab_extent")
    return lo.value, hi.value


def schedule(nx, ny, nz, tile_x, tile_y, kind, chunk, max_blocks):
    """Returns (items [n, 3] of (tile, k0, k1), block_first [nblocks + 1])."""
    lib = load_library()
    ni, nb = ctypes.c_int32(), ctypes.c_int32()
    _check(lib.ela3d_schedule_build(nx, ny, nz, tile_x, tile_y, kind, chunk, max_blocks, ctypes.byref(ni),
                                    ctypes.byref(nb), None, None), "ela3d_schedule_build")
    items = np.zeros((ni.value, 3), np.int32)
    first = np.zeros(nb.value + 1, np.int32)
    _check(lib.ela3d_schedule_build(nx, ny, nz, tile_x, tile_y, kind, chunk, max_blocks, ctypes.byref(ni),
                                    ctypes.byref(nb), items.ctypes.data, first.ctypes.data), "ela3d_schedule_build")
    return items, first


class ModelSpec(ctypes.Structure):
    """ctypes mirror of ela3d_model_spec."""
    _fields_ = [("kind", ctypes.c_int32), ("nlayers", ctypes.c_int32), ("cp", ctypes.c_double * 8),
                ("cs_ratio", ctypes.c_double * 8), ("depth", ctypes.c_double * 8), ("dome_amp", ctypes.c_double),
                ("dome_sigma", ctypes.c_double), ("dome_xc", ctypes.c_double), ("dome_yc", ctypes.c_double),
                ("rho_coef", ctypes.c_double), ("rho_pow", ctypes.c_double), ("perturb", ctypes.c_double),
                ("seed", ctypes.c_uint64), ("cp0", ctypes.c_double), ("cs0", ctypes.c_double),
                ("rho0", ctypes.c_double)]

    @classmethod
    def from_dict(cls, d: dict) -> "ModelSpec":
        m = cls()
        for k, v in d.items():
            if k in ("cp", "cs_ratio", "depth"):
                arr = getattr(m, k)
                for i, x in enumerate(v):
                    arr[i] = float(x)
            else:
                setattr(m, k, v)
        return m


def generate_model(spec: dict, nx: int, ny: int, nz: int):
    """Runs the device model generator and returns (cp, cs, rho) [nz, ny, nx]."""
    lib = load_library()
    out = [np.empty((nz, ny, nx), np.float32) for _ in range(3)]
    m = ModelSpec.from_dict(spec)
    _check(lib.ela3d_model_generate(ctypes.byref(m), nx, ny, nz, out[0].ctypes.data, out[1].ctypes.data,
                                    out[2].ctypes.data), "ela3d_model_generate")
    return tuple(out)


class Ela3dError(RuntimeError):
    def __init__(self, status: int, where: str):
        lib = _LIB
        msg = lib.ela3d_status_string(status).decode() if lib else str(status)
        detail = lib.ela3d_last_error().decode() if lib else ""
        super().__init__(f"{where}: {msg} ({detail})")
        self.status = status


def load_library(path: str | None = None) -> ctypes.CDLL:
    global _LIB
    if _LIB is not None:
        return _LIB
    path = path or os.environ.get("ELA3D_LIB", LIB_PATH)
    if not os.path.exists(path):
        raise RuntimeError(f"libela3d.so not built ({path}); run __graft_entry__.build()")
    lib = ctypes.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def builtin_tuning(p) -> "Tuning":
    """The built-in kernel choice for a single shot with parameters p
    (ela3d_builtin_tuning; host only)."""
    c, _rec = p.to_c()
    t = Tuning()
    _check(load_library().ela3d_builtin_tuning(ctypes.byref(c), ctypes.addressof(t)), "ela3d_builtin_tuning")
    return t


def select_device(ordinal: int) -> None:
    _check(load_library().ela3d_select_device(ordinal), "ela3d_select_device")


class _HostBuffer:
    """Owner of one page-locked allocation; freed when the last array view
    of it is collected."""

    def __init__(self, nbytes: int):
        self._lib = load_library()
        self.ptr = ctypes.c_void_p()
        _check(self._lib.ela3d_host_alloc(nbytes, ctypes.byref(self.ptr)), "ela3d_host_alloc")
        self.nbytes = nbytes

    def __del__(self):
        if getattr(self, "ptr", None) and self.ptr.value:
            self._lib.ela3d_host_free(self.ptr)
            self.ptr = ctypes.c_void_p()


def pinned_empty(shape, dtype=np.float32) -> np.ndarray:
    """A numpy array in page-locked host memory (ela3d_host_alloc): model
    arrays and read-back buffers in it copy at the link's full rate."""
    dtype = np.dtype(dtype)
    count = int(np.prod(shape)) if np.ndim(shape) else int(shape)
    owner = _HostBuffer(max(1, count * dtype.itemsize))
    raw = (ctypes.c_char * owner.nbytes).from_address(owner.ptr.value)
    arr = np.frombuffer(raw, dtype=dtype, count=count).reshape(shape)
    arr.flags.writeable = True
    # the ctypes buffer keeps the owner alive as long as any view exists
    raw._owner = owner
    return arr


def pinned_copy(a: np.ndarray, dtype=None) -> np.ndarray:
    """A page-locked copy of a."""
    a = np.asarray(a, dtype=dtype)
    out = pinned_empty(a.shape, a.dtype)
    out[...] = a
    return out


def _check(st: int, where: str) -> None:
    if st != 0:
        raise Ela3dError(st, where)


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


class Plan:
    """One shot resident on the GPU (ela3d_plan_create / ela3d_run / ...)."""

    def __init__(self, params: ShotParams, cp: np.ndarray, cs: np.ndarray, rho: np.ndarray,
                 variant: int = -1, schedule: int = -1, chunk: int = 0, blocks_per_sm: int = -1,
                 prefetch: int = -1, lag: int = -1):
        lib = load_library()
        self._lib = lib
        self.params = params
        n = params.cells
        models = [np.ascontiguousarray(a, dtype=np.float32).reshape(-1) for a in (cp, cs, rho)]
        if any(m.size != n for m in models):
            raise ValueError("model arrays must hold nx*ny*nz float32 values")
        c, rec = params.to_c()
        h = ctypes.c_void_p()
        t = Tuning(variant, schedule, chunk, blocks_per_sm, prefetch, lag)
        _check(lib.ela3d_plan_create_tuned(ctypes.byref(c), _ptr(models[0]), _ptr(models[1]), _ptr(models[2]),
                                           ctypes.byref(t), ctypes.byref(h)), "ela3d_plan_create")
        self._h = h

    @classmethod
    def from_model(cls, params: ShotParams, spec: dict, variant: int = -1, schedule: int = -1,
                   chunk: int = 0, prefetch: int = -1, lag: int = -1) -> "Plan":
        """A plan whose model is generated on the device (ela3d_plan_create_model)."""
        self = cls.__new__(cls)
        lib = load_library()
        self._lib = lib
        self.params = params
        c, rec = params.to_c()
        m = ModelSpec.from_dict(spec)
        t = Tuning(variant, schedule, chunk, -1, prefetch, lag)
        h = ctypes.c_void_p()
        _check(lib.ela3d_plan_create_model(ctypes.byref(c), ctypes.byref(m), ctypes.byref(t), ctypes.byref(h)),
               "ela3d_plan_create_model")
        self._h = h
        return self

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def run(self, nsteps: int) -> None:
        _check(self._lib.ela3d_run(self._h, nsteps), "ela3d_run")

    def run_timed(self, nsteps: int) -> float:
        """Runs nsteps and returns their device time in ms (CUDA events on
        the plan's stream)."""
        ms = ctypes.c_double()
        _check(self._lib.ela3d_run_timed(self._h, nsteps, ctypes.byref(ms)), "ela3d_run_timed")
        return ms.value

    def enqueue(self, nsteps: int) -> None:
        _check(self._lib.ela3d_enqueue(self._h, nsteps), "ela3d_enqueue")

    def sync(self) -> None:
        _check(self._lib.ela3d_sync(self._h), "ela3d_sync")

    def seismograms(self, fp64: bool = False, out: np.ndarray | None = None) -> np.ndarray:
        """[nrec, 3, nsamp] receiver traces; `out` (C-contiguous, of that
        shape and float32 / float64) receives them instead of a new array."""
        p = self.params
        dt = np.float64 if fp64 else np.float32
        if out is None:
            out = np.zeros((p.nrec, 3, p.nsamp), dt)
        elif out.shape != (p.nrec, 3, p.nsamp) or out.dtype != dt or not out.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous [nrec, 3, nsamp] array of the requested precision")
        if out.size:
            fn = self._lib.ela3d_get_seismograms_f64 if fp64 else self._lib.ela3d_get_seismograms
            _check(fn(self._h, _ptr(out)), "ela3d_get_seismograms")
        return out

    def checkpoint(self) -> np.ndarray:
        """The plan's complete state (ela3d_checkpoint_save) as a uint8 array."""
        n = ctypes.c_int64()
        _check(self._lib.ela3d_checkpoint_size(self._h, ctypes.byref(n)), "ela3d_checkpoint_size")
        buf = np.empty(n.value, np.uint8)
        _check(self._lib.ela3d_checkpoint_save(self._h, _ptr(buf), n.value), "ela3d_checkpoint_save")
        return buf

    def restore(self, buf: np.ndarray) -> None:
        """Continue from a checkpoint of a plan with the same parameters."""
        buf = np.ascontiguousarray(buf, np.uint8)
        _check(self._lib.ela3d_checkpoint_load(self._h, _ptr(buf), buf.size), "ela3d_checkpoint_load")

    def source_trace(self, fp64: bool = False) -> np.ndarray:
        """[3, nstep + 1]: the source cell's injected components after each
        step's injection (sxx syy szz explosive, vx vy vz force)."""
        out = np.zeros((3, self.params.nstep + 1), np.float64 if fp64 else np.float32)
        fn = self._lib.ela3d_get_source_trace_f64 if fp64 else self._lib.ela3d_get_source_trace
        _check(fn(self._h, _ptr(out)), "ela3d_get_source_trace")
        return out

    def field(self, comp: int, fp64: bool = False) -> np.ndarray:
        p = self.params
        out = np.empty((p.nz, p.ny, p.nx), np.float64 if fp64 else np.float32)
        fn = self._lib.ela3d_get_field_f64 if fp64 else self._lib.ela3d_get_field
        _check(fn(self._h, comp, _ptr(out)), "ela3d_get_field")
        return out

    def energy(self) -> float:
        e = ctypes.c_double()
        _check(self._lib.ela3d_energy(self._h, ctypes.byref(e)), "ela3d_energy")
        return e.value

    def info(self) -> PlanInfo:
        i = PlanInfo()
        _check(self._lib.ela3d_plan_info_get(self._h, ctypes.byref(i)), "ela3d_plan_info_get")
        return i

    def set_kernel_timing(self, on: bool) -> None:
        _check(self._lib.ela3d_set_kernel_timing(self._h, 1 if on else 0), "ela3d_set_kernel_timing")

    def flow_timing(self) -> tuple[float, int, int]:
        """(ms, launches, steps) of the dataflow launches timed since
        set_kernel_timing(True) (ela3d_get_flow_timing)."""
        ms, nl, ns = ctypes.c_double(), ctypes.c_int64(), ctypes.c_int64()
        _check(self._lib.ela3d_get_flow_timing(self._h, ctypes.byref(ms), ctypes.byref(nl), ctypes.byref(ns)),
               "ela3d_get_flow_timing")
        return ms.value, nl.value, ns.value

    def kernel_timing(self) -> tuple[float, float, int, int]:
        a, b = ctypes.c_double(), ctypes.c_double()
        na, nb = ctypes.c_int64(), ctypes.c_int64()
        _check(self._lib.ela3d_get_kernel_timing(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(na),
                                                 ctypes.byref(nb)), "ela3d_get_kernel_timing")
        return a.value, b.value, na.value, nb.value

    def profiles(self, axis: int) -> dict:
        """The C-PML profiles of one axis as the kernels read them
        (ela3d_plan_get_profiles): a, b, K, a_half, b_half, K_half."""
        n = (self.params.nx, self.params.ny, self.params.nz)[axis]
        out = np.zeros(6 * n, np.float64)
        _check(self._lib.ela3d_plan_get_profiles(self._h, axis, out.ctypes.data), "ela3d_plan_get_profiles")
        v = out.reshape(6, n)
        return {"a": v[0], "b": v[1], "K": 1.0 / v[2], "a_half": v[3], "b_half": v[4], "K_half": 1.0 / v[5]}

    def poison_padding(self, value: float = float("nan")) -> None:
        """Test hook: `value` into every padding column of the fields and
        memory variables (ela3d_plan_poison_padding)."""
        _check(self._lib.ela3d_plan_poison_padding(self._h, value), "ela3d_plan_poison_padding")

    def check_guards(self) -> None:
        """Raises Ela3dError (ELA3D_ERR_CORRUPT) if a write ran past a device
        array (guard zones are on when ELA3D_GUARD_ZONES was set at creation)."""
        _check(self._lib.ela3d_plan_check_guards(self._h), "ela3d_plan_check_guards")

    def inject_timeout(self, launches: int) -> None:
        """Test hook: the next `launches` kernel launches withhold their loads
        so their bounded waits expire (ELA3D_ERR_TIMEOUT at the next sync)."""
        _check(self._lib.ela3d_plan_inject_timeout(self._h, launches), "ela3d_plan_inject_timeout")

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.ela3d_plan_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def is_fp64(p: ShotParams) -> bool:
    return p.precision == FP64


class Batch:
    """Many shots advanced together (ela3d_batch_*).  `shots` is a list of
    (ShotParams, cp, cs, rho); passing the same model arrays for several
    shots stores that model once on the device."""

    def __init__(self, shots, variant: int = -1, schedule: int = -1, chunk: int = 0, blocks_per_sm: int = -1,
                 prefetch: int = -1, lag: int = -1):
        lib = load_library()
        self._lib = lib
        self.params = [s[0] for s in shots]
        n = len(shots)
        structs = (CParams * n)()
        keep = []
        ptrs = {k: (ctypes.c_void_p * n)() for k in ("cp", "cs", "rho")}
        seen = {}
        for i, (p, cp, cs, rho) in enumerate(shots):
            c, rec = p.to_c()
            structs[i] = c
            keep.append(rec)
            for key, arr in (("cp", cp), ("cs", cs), ("rho", rho)):
                m = seen.get(id(arr))
                if m is None:
                    m = np.ascontiguousarray(arr, dtype=np.float32).reshape(-1)
                    if m.size != p.cells:
                        raise ValueError("model arrays must hold nx*ny*nz float32 values")
                    seen[id(arr)] = m
                    keep.append(m)
                ptrs[key][i] = m.ctypes.data
        t = Tuning(variant, schedule, chunk, blocks_per_sm, prefetch, lag)
        h = ctypes.c_void_p()
        _check(lib.ela3d_batch_create(n, structs, ptrs["cp"], ptrs["cs"], ptrs["rho"], ctypes.byref(t),
                                      ctypes.byref(h)), "ela3d_batch_create")
        self._h = h

    def run(self, nsteps: int) -> None:
        _check(self._lib.ela3d_batch_run(self._h, nsteps), "ela3d_batch_run")

    def run_timed(self, nsteps: int) -> float:
        ms = ctypes.c_double()
        _check(self._lib.ela3d_batch_run_timed(self._h, nsteps, ctypes.byref(ms)), "ela3d_batch_run_timed")
        return ms.value

    def seismograms(self, shot: int) -> np.ndarray:
        p = self.params[shot]
        out = np.zeros((p.nrec, 3, p.nsamp), np.float32)
        if out.size:
            _check(self._lib.ela3d_batch_get_seismograms(self._h, shot, _ptr(out)), "ela3d_batch_get_seismograms")
        return out

    def source_trace(self, shot: int) -> np.ndarray:
        out = np.zeros((3, self.params[shot].nstep + 1), np.float32)
        _check(self._lib.ela3d_batch_get_source_trace(self._h, shot, _ptr(out)), "ela3d_batch_get_source_trace")
        return out

    def field(self, shot: int, comp: int) -> np.ndarray:
        p = self.params[shot]
        out = np.empty((p.nz, p.ny, p.nx), np.float32)
        _check(self._lib.ela3d_batch_get_field(self._h, shot, comp, _ptr(out)), "ela3d_batch_get_field")
        return out

    def info(self, shot: int) -> PlanInfo:
        i = PlanInfo()
        _check(self._lib.ela3d_batch_info(self._h, shot, ctypes.byref(i)), "ela3d_batch_info")
        return i

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.ela3d_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_int64), ("max_active", ctypes.c_int32),
                ("steps_per_round", ctypes.c_int32), ("precision", ctypes.c_int32), ("fill_cells", ctypes.c_int32),
                ("tune", Tuning)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_int64), ("completed", ctypes.c_int64), ("failed", ctypes.c_int64),
                ("cancelled", ctypes.c_int64), ("queued", ctypes.c_int64), ("running", ctypes.c_int64),
                ("rounds", ctypes.c_int64), ("cell_updates", ctypes.c_double), ("busy_seconds", ctypes.c_double),
                ("wall_seconds", ctypes.c_double), ("latency_p50_s", ctypes.c_double),
                ("latency_p99_s", ctypes.c_double), ("latency_max_s", ctypes.c_double),
                ("device_bytes_in_use", ctypes.c_int64), ("device_bytes_budget", ctypes.c_int64)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED, REQ_CANCELLED = range(5)


class Server:
    """Continuous-batching request loop (ela3d_server_*)."""

    def __init__(self, hbm_budget_bytes: int = 0, max_active: int = 0, steps_per_round: int = 50,
                 precision: int = 0, variant: int = -1, schedule: int = -1, chunk: int = 0, prefetch: int = -1,
                 fill_cells: int = 0, lag: int = -1):
        lib = load_library()
        self._lib = lib
        cfg = ServerConfig()
        _check(lib.ela3d_server_config_default(ctypes.byref(cfg)), "ela3d_server_config_default")
        cfg.hbm_budget_bytes = hbm_budget_bytes
        cfg.max_active = max_active
        cfg.steps_per_round = steps_per_round
        cfg.precision = precision
        cfg.fill_cells = fill_cells
        cfg.tune = Tuning(variant, schedule, chunk, -1, prefetch, lag)
        h = ctypes.c_void_p()
        _check(lib.ela3d_server_create(ctypes.byref(cfg), ctypes.byref(h)), "ela3d_server_create")
        self._h = h
        self._params = {}
        self._callbacks = {}

    def submit(self, params: ShotParams, cp, cs, rho) -> int:
        c, rec = params.to_c()
        m = [np.ascontiguousarray(a, dtype=np.float32).reshape(-1) for a in (cp, cs, rho)]
        if any(x.size != params.cells for x in m):
            raise ValueError("model arrays must hold nx*ny*nz float32 values")
        t = ctypes.c_uint64()
        _check(self._lib.ela3d_server_submit(self._h, ctypes.byref(c), m[0].ctypes.data, m[1].ctypes.data,
                                             m[2].ctypes.data, ctypes.byref(t)), "ela3d_server_submit")
        self._params[t.value] = params
        return t.value

    def submit_model(self, params: ShotParams, spec: dict) -> int:
        """Queues a request whose model is generated on the device at admission."""
        c, rec = params.to_c()
        m = ModelSpec.from_dict(spec)
        t = ctypes.c_uint64()
        _check(self._lib.ela3d_server_submit_model(self._h, ctypes.byref(c), ctypes.byref(m), ctypes.byref(t)),
               "ela3d_server_submit_model")
        self._params[t.value] = params
        return t.value

    def poll(self, ticket: int) -> tuple[int, int]:
        st, ready = ctypes.c_int32(), ctypes.c_int32()
        rc = self._lib.ela3d_server_poll(self._h, ticket, ctypes.byref(st), ctypes.byref(ready))
        if rc not in (0,) and st.value != REQ_FAILED:
            _check(rc, "ela3d_server_poll")
        return st.value, ready.value

    def read(self, ticket: int, first: int = 0, count: int | None = None) -> np.ndarray:
        p = self._params[ticket]
        count = p.nsamp - first if count is None else count
        out = np.zeros((p.nrec, 3, count), np.float32)
        if out.size:
            _check(self._lib.ela3d_server_read(self._h, ticket, first, count, out.ctypes.data), "ela3d_server_read")
        return out

    def wait(self, ticket: int, timeout_ms: int = -1) -> None:
        _check(self._lib.ela3d_server_wait(self._h, ticket, timeout_ms), "ela3d_server_wait")

    def cancel(self, ticket: int) -> None:
        _check(self._lib.ela3d_server_cancel(self._h, ticket), "ela3d_server_cancel")

    def on_done(self, ticket: int, fn) -> None:
        """fn(ticket, status) once the request ends (status 0: done); called
        on the server's worker thread, or at once if it has already ended."""
        cb = REQUEST_CALLBACK(lambda t, st, _user: fn(int(t), int(st)))
        self._callbacks[ticket] = cb   # kept alive until the server is closed
        _check(self._lib.ela3d_server_on_done(self._h, ticket, cb, None), "ela3d_server_on_done")

    def release(self, ticket: int) -> None:
        _check(self._lib.ela3d_server_release(self._h, ticket), "ela3d_server_release")
        self._params.pop(ticket, None)

    def stats(self) -> dict:
        s = ServerStats()
        _check(self._lib.ela3d_server_stats_get(self._h, ctypes.byref(s)), "ela3d_server_stats_get")
        return s.as_dict()

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.ela3d_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune(shots, steps: int = 10) -> tuple[Tuning, float, int]:
    """Runs the library's autotuner on a list of (ShotParams, cp, cs, rho);
    returns (best tuning, its ms for `steps` steps, candidates timed)."""
    lib = load_library()
    n = len(shots)
    structs = (CParams * n)()
    keep = []
    ptrs = {k: (ctypes.c_void_p * n)() for k in ("cp", "cs", "rho")}
    seen = {}
    for i, (p, cp, cs, rho) in enumerate(shots):
        c, rec = p.to_c()
        structs[i] = c
        keep.append(rec)
        for key, arr in (("cp", cp), ("cs", cs), ("rho", rho)):
            m = seen.get(id(arr))
            if m is None:
                m = np.ascontiguousarray(arr, dtype=np.float32).reshape(-1)
                seen[id(arr)] = m
                keep.append(m)
            ptrs[key][i] = m.ctypes.data
    best = Tuning()
    ms = ctypes.c_double()
    cand = ctypes.c_int32()
    _check(lib.ela3d_autotune(n, structs, ptrs["cp"], ptrs["cs"], ptrs["rho"], steps, ctypes.byref(best),
                              ctypes.byref(ms), ctypes.byref(cand)), "ela3d_autotune")
    return best, ms.value, cand.value
