"""The C ABI library: loads without a GPU, exports every declared entry
point, its structs match the Python mirror, and argument errors come back as
status codes before any device is touched."""
import ctypes
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ela3d.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(ela3d_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(built):
    from ela3d_gb300 import _abi

    lib = _abi.load_library()
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    bound = {s[0] for s in _abi.SIGNATURES}
    assert set(names) == bound, set(names) ^ bound


def test_header_compiles_as_c_and_struct_layout_matches(built):
    from ela3d_gb300 import _abi, params

    prog = r"""
#include <stdio.h>
#include <stddef.h>
#include "ela3d.h"
#define F(s, m) printf(#s "." #m " %zu\n", offsetof(s, m));
int main(void) {
  printf("ela3d_params %zu\n", sizeof(ela3d_params));
  printf("ela3d_plan_info %zu\n", sizeof(ela3d_plan_info));
  printf("ela3d_tuning %zu\n", sizeof(ela3d_tuning));
  printf("ela3d_variant_info %zu\n", sizeof(ela3d_variant_info));
  F(ela3d_params, dx) F(ela3d_params, npml) F(ela3d_params, npower) F(ela3d_params, stf)
  F(ela3d_params, src_w) F(ela3d_params, rec) F(ela3d_params, nrec) F(ela3d_params, energy_every)
  F(ela3d_plan_info, device_bytes) F(ela3d_plan_info, slab_hi)
  return 0;
}
"""
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        open(c, "w").write(prog)
        subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), c, "-o", exe],
                       check=True)
        out = dict(line.split() for line in subprocess.run([exe], capture_output=True, text=True,
                                                           check=True).stdout.splitlines())
    assert int(out["ela3d_params"]) == ctypes.sizeof(params.CParams)
    assert int(out["ela3d_plan_info"]) == ctypes.sizeof(_abi.PlanInfo)
    assert int(out["ela3d_tuning"]) == ctypes.sizeof(_abi.Tuning)
    assert int(out["ela3d_variant_info"]) == ctypes.sizeof(_abi.VariantInfo)
    for key, val in out.items():
        if "." in key:
            s, m = key.split(".")
            cls = {"ela3d_params": params.CParams, "ela3d_plan_info": _abi.PlanInfo}[s]
            assert getattr(cls, m).offset == int(val), key


def test_header_compiles_as_cpp():
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.cpp")
        open(c, "w").write('#include "ela3d.h"\nint main() { ela3d_params p; return ela3d_params_default(&p); }\n')
        subprocess.run(["g++", "-fsyntax-only", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), c],
                       check=True)


def test_params_default_is_reference_main(built):
    from ela3d_gb300 import _abi, params

    lib = _abi.load_library()
    c = params.CParams()
    assert lib.ela3d_params_default(ctypes.byref(c)) == 0
    # seismicCPML_3d_isotropic_simpelmodel.cpp:20-78
    assert (c.nx, c.ny, c.nz, c.nstep, c.npml, c.sampgat, c.it_output) == (500, 500, 500, 1000, 10, 2, 200)
    assert (c.dx, c.dt, c.f0, c.factor, c.vpml, c.rcoef) == (10.0, 1e-3, 35.0, 1e7, 3000.0, 1e-3)
    assert (c.src_i, c.src_j, c.src_k) == (249, 249, 10)
    assert c.stf == params.STF_GAUSS_DERIV and c.src_kind == params.SRC_EXPLOSIVE


def test_status_strings(built):
    from ela3d_gb300 import _abi

    lib = _abi.load_library()
    for s in range(0, 12):
        assert lib.ela3d_status_string(s).decode() not in ("", "unknown status")
    assert lib.ela3d_status_string(99).decode() == "unknown status"
    assert lib.ela3d_version().decode().startswith("ela3d-gb300")


BAD = {
    "tiny_grid": {"nx": 2},
    "negative_dt": {"dt": -1e-3},
    "source_outside": {"src": (200, 5, 5)},
    "receiver_outside": {"rec": np.array([[1, 1, 1], [0, 0, 999]], np.int32)},
    "sampgat_zero": {"sampgat": 0},
    "bad_precision": {"precision": 7},
    "bad_pml_mode": {"pml_mode": 3},
    "bad_rcoef": {"rcoef": 1.5},
}


@pytest.mark.parametrize("name", sorted(BAD))
def test_invalid_arguments_rejected_before_device(built, name):
    from ela3d_gb300 import Ela3dError, Plan, ShotParams, media

    p = ShotParams(nx=20, ny=20, nz=20, nstep=10, npml=4, src=(10, 10, 10),
                   rec=np.array([[5, 5, 5]], np.int32)).with_(**BAD[name])
    n = max(p.nx, 1) * p.ny * p.nz
    m = np.ones(n, np.float32)
    with pytest.raises(Ela3dError) as e:
        Plan(p, m * 3000, m * 1700, m * 2000)
    assert e.value.status == 1, e.value  # ELA3D_ERR_INVALID_ARG


def _fp64_variant():
    import ela3d_gb300

    return next(i for i, v in enumerate(ela3d_gb300.variants()) if v.fp64)


BAD_TUNING = {
    "no_such_variant": lambda: {"variant": 10_000},
    "variant_of_other_precision": lambda: {"variant": _fp64_variant()},
    "schedule_kind": lambda: {"schedule": 5},
    "negative_chunk": lambda: {"chunk": -2},
    "dataflow_chunk_of_one_plane": lambda: {"schedule": 3, "chunk": 1},
    "overlapping_dataflow_chunk_of_one_plane": lambda: {"schedule": 4, "chunk": 1},
    "negative_lag": lambda: {"schedule": 3, "lag": -2},
}


@pytest.mark.parametrize("name", sorted(BAD_TUNING))
def test_invalid_tuning_rejected_before_device(built, name):
    """Tuning fields are checked with the parameters, before any device work
    (plans, generated-model plans, batches, servers)."""
    from ela3d_gb300 import Batch, Ela3dError, Plan, Server, ShotParams

    p = ShotParams(nx=20, ny=20, nz=20, nstep=10, npml=4, src=(10, 10, 10))
    m = np.ones(p.cells, np.float32)
    tune = BAD_TUNING[name]()
    for make in (lambda: Plan(p, m * 3000, m * 1700, m * 2000, **tune),
                 lambda: Plan.from_model(p, {"kind": 0, "cp0": 3000.0, "cs0": 1700.0, "rho0": 2000.0}, **tune),
                 lambda: Batch([(p, m * 3000, m * 1700, m * 2000)], **tune),
                 lambda: Server(**tune)):
        with pytest.raises(Ela3dError) as e:
            make()
        assert e.value.status == 1, e.value  # ELA3D_ERR_INVALID_ARG


def test_variants_listed(built):
    import ela3d_gb300

    vs = ela3d_gb300.variants()
    assert any(v.fp64 == 0 for v in vs) and any(v.fp64 == 1 for v in vs)
    for v in vs:
        assert v.tile_x % (4 if not v.fp64 else 2) == 0
        assert v.threads % 32 == 0 and v.stages >= 3
        assert v.stress_smem <= 227 * 1024 and v.velocity_smem <= 227 * 1024


def test_plan_without_gpu_fails_loudly(built):
    """On a machine without a CUDA device the product raises; there is no CPU
    path to fall back on."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from ela3d_gb300 import Ela3dError, Plan, ShotParams

    p = ShotParams(nx=16, ny=16, nz=16, nstep=4, npml=2, src=(8, 8, 8))
    m = np.ones(p.cells, np.float32)
    with pytest.raises(Ela3dError):
        Plan(p, m * 3000, m * 1700, m * 2000)


def test_model_spec_layout_matches_header(built):
    import ctypes as C
    from ela3d_gb300._abi import ModelSpec

    prog = r'''
#include <stdio.h>
#include <stddef.h>
#include "ela3d.h"
int main(void) { printf("%zu %zu %zu\n", sizeof(ela3d_model_spec), offsetof(ela3d_model_spec, seed),
                        offsetof(ela3d_model_spec, rho0)); return 0; }
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "m.c")
        open(c, "w").write(prog)
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", os.path.join(d, "m")], check=True)
        size, seed, rho0 = (int(v) for v in subprocess.run([os.path.join(d, "m")], capture_output=True, text=True,
                                                            check=True).stdout.split())
    assert size == C.sizeof(ModelSpec) and seed == ModelSpec.seed.offset and rho0 == ModelSpec.rho0.offset
