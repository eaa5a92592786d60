"""ela3d_energy_noalloc through the C ABI: the energy of caller-owned device
arrays, computed without any device allocation inside the library, must
match the plan-based ela3d_energy on the same state, call after call."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# the plan's monitor scales by 1/(1/dx) rounded through float32, this entry
# point by dx itself: they agree to a few 1e-8 relative
TOL = 1e-6


def _case():
    from ela3d_gb300 import ShotParams, media

    nx, ny, nz = 40, 36, 30
    cp, cs, rho = media.anticline_layers(nx, ny, nz, depths=(8, 15, 22, 60), amp=3, sigma=8, seed=2)
    p = ShotParams(nx=nx, ny=ny, nz=nz, nstep=80, dt=1e-3, npml=5, f0=25.0, t0=0.05, src=(20, 18, 12))
    return p, cp, cs, rho


def _on_device(a, p, pitch):
    import torch

    t = torch.zeros((p.nz, p.ny, pitch), dtype=torch.float32, device="cuda")
    t[:, :, : p.nx] = torch.from_numpy(np.ascontiguousarray(a, np.float32).reshape(p.nz, p.ny, p.nx)).cuda()
    return t


def _call(lib, fields, model, p, pitch, nz, out_ptr):
    ptrs = (ctypes.c_void_p * 9)(*[t.data_ptr() for t in fields])
    return lib.ela3d_energy_noalloc(ptrs, ctypes.c_void_p(model[0].data_ptr()), ctypes.c_void_p(model[1].data_ptr()),
                                    ctypes.c_void_p(model[2].data_ptr()), p.nx, p.ny, nz, pitch, p.dx, p.dy, p.dz,
                                    ctypes.c_void_p(out_ptr), None)


@pytest.mark.parametrize("pad", [0, 8])
def test_noalloc_energy_matches_plan_energy_twice(built, pad):
    torch = pytest.importorskip("torch")
    from ela3d_gb300 import Plan
    from ela3d_gb300._abi import load_library

    lib = load_library()
    p, cp, cs, rho = _case()
    pitch = p.nx + pad
    with Plan(p, cp, cs, rho) as plan:
        plan.run(p.nstep)
        e_plan = plan.energy()
        fields = [_on_device(plan.field(c), p, pitch) for c in range(9)]
    model = [_on_device(a, p, pitch) for a in (cp, cs, rho)]
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    for call in range(2):   # two calls in a row, each into its own slot
        st = _call(lib, fields, model, p, pitch, p.nz, out.data_ptr() + 8 * call)
        assert st == 0, lib.ela3d_last_error().decode()
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    assert e_plan > 0 and got[0] > 0
    assert got[0] == got[1]
    assert abs(got[0] - e_plan) <= TOL * e_plan, (got[0], e_plan)


def test_noalloc_energy_rejects_sizes_beyond_its_scratch(built):
    torch = pytest.importorskip("torch")
    from ela3d_gb300._abi import load_library

    lib = load_library()
    p, cp, cs, rho = _case()
    fields = [_on_device(np.zeros(p.cells, np.float32), p, p.nx) for _ in range(9)]
    model = [_on_device(a, p, p.nx) for a in (cp, cs, rho)]
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    # argument checks happen on the host, before any device work
    assert _call(lib, fields, model, p, p.nx, 16385, out.data_ptr()) == 1
    assert "16384" in lib.ela3d_last_error().decode()
    assert _call(lib, fields, model, p, p.nx - 1, p.nz, out.data_ptr()) == 1
