"""ela3d_energy_noalloc through the C ABI: the energy of caller-owned device
arrays, computed without any device allocation inside the library, must
match the plan-based ela3d_energy on the same state and an independent
NumPy FP64 evaluation of the same arrays, call after call, and must leave
the device's free memory unchanged."""
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


def _numpy_energy(fields, cp, cs, rho, p):
    """Kinetic plus strain energy in FP64, written independently of the
    library: strains from Hooke's law in Young's modulus E and Poisson's
    ratio nu, energy density 1/2 rho |v|^2 + 1/2 sigma_ij eps_ij."""
    f = [np.asarray(a, np.float64).reshape(p.nz, p.ny, p.nx) for a in fields]
    cp, cs, rho = (np.asarray(a, np.float64).reshape(p.nz, p.ny, p.nx) for a in (cp, cs, rho))
    vx, vy, vz, sxx, syy, szz, sxy, sxz, syz = f
    mu = rho * cs ** 2
    lam = rho * cp ** 2 - 2.0 * mu
    E = mu * (3.0 * lam + 2.0 * mu) / (lam + mu)
    nu = lam / (2.0 * (lam + mu))
    exx = (sxx - nu * (syy + szz)) / E
    eyy = (syy - nu * (sxx + szz)) / E
    ezz = (szz - nu * (sxx + syy)) / E
    w = 0.5 * (sxx * exx + syy * eyy + szz * ezz) + (sxy ** 2 + sxz ** 2 + syz ** 2) / (2.0 * mu)
    kin = 0.5 * rho * (vx ** 2 + vy ** 2 + vz ** 2)
    return float((kin + w).sum() * p.dx * p.dy * p.dz)


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
        host = [plan.field(c) for c in range(9)]
    fields = [_on_device(a, p, pitch) for a in host]
    model = [_on_device(a, p, pitch) for a in (cp, cs, rho)]
    e_np = _numpy_energy(host, cp, cs, rho, p)
    out = torch.zeros(6, dtype=torch.float64, device="cuda")
    for call in range(2):   # two calls in a row, each into its own slot
        st = _call(lib, fields, model, p, pitch, p.nz, out.data_ptr() + 8 * call)
        assert st == 0, lib.ela3d_last_error().decode()
    torch.cuda.synchronize()
    # it allocates nothing: after those calls (the first one on this device
    # loads the kernels), more calls leave the device's free memory as it was
    free0 = torch.cuda.mem_get_info()[0]
    for call in range(2, 6):
        assert _call(lib, fields, model, p, pitch, p.nz, out.data_ptr() + 8 * call) == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    got = out.cpu().numpy()
    assert e_plan > 0 and got[0] > 0
    assert np.all(got == got[0])
    assert abs(got[0] - e_plan) <= TOL * e_plan, (got[0], e_plan)
    assert abs(got[0] - e_np) <= 1e-9 * e_np, (got[0], e_np)


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
