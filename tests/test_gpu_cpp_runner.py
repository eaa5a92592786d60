"""The C++ runner ela3d_run (csrc/ela3d_run.cpp, host code on the C ABI): on
the same parameter file it writes the same reference-format files as the
Python runner, byte for byte -- receiver text, snapshots and source trace,
in FP32 and FP64 -- and rejects a bad file with exit status 1."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _params(tmp_path):
    from ela3d_gb300 import refio
    from test_refio import case

    p, cp, cs, rho = case()
    refio.write_model(str(tmp_path / "m"), cp, cs, rho)
    path = tmp_path / "params.txt"
    path.write_text("\n".join([
        f"nx {p.nx}", f"ny {p.ny}", f"nz {p.nz}", "dx 10", f"dt {p.dt!r}", f"nstep {p.nstep}",
        f"sampgat {p.sampgat}", "it_output 10", "ngatx 4", "ngaty 2", f"npml {p.npml}", f"f0 {p.f0!r}",
        f"t0 {p.t0!r}", "src %d %d %d" % p.src, f"model {tmp_path / 'm'}", "rec 3 4 5", "rec 9 8 7"]) + "\n")
    return p, str(path)


@pytest.mark.parametrize("fp64", [False, True], ids=["fp32", "fp64"])
def test_cpp_runner_writes_the_python_runners_files(built, tmp_path, fp64):
    from ela3d_gb300 import cli
    from ela3d_gb300._build import RUNNER

    p, params = _params(tmp_path)
    py_dir, cc_dir = str(tmp_path / "py"), str(tmp_path / "cc")
    cli.run(params, py_dir, fp64=fp64)
    os.makedirs(cc_dir)
    r = subprocess.run([RUNNER, params, "--outdir", cc_dir] + (["--fp64"] if fp64 else []), capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    names = [f"rechorv{c}.txt" for c in "xyz"] + [f"recsrc{c}.txt" for c in "xyz"]
    names += ["%s%05i.bin" % (c, it) for c in ("vx", "vy", "vz") for it in (10, 20)]
    for name in names:
        a = open(os.path.join(py_dir, name), "rb").read()
        b = open(os.path.join(cc_dir, name), "rb").read()
        assert len(a) > 0 and a == b, name
    seis_py = np.load(os.path.join(py_dir, "seis.npy"))
    seis_cc = np.fromfile(os.path.join(cc_dir, "seis.bin"), np.float32).reshape(seis_py.shape)
    assert np.array_equal(seis_py.astype(np.float32), seis_cc) and np.any(seis_cc)


def test_cpp_runner_rejects_bad_input(built, tmp_path):
    from ela3d_gb300._build import RUNNER

    bad = tmp_path / "bad.txt"
    bad.write_text("nx 20\nny 20\nnz 20\nnpml 4\nsrc 50 10 10\n")   # source outside the grid
    r = subprocess.run([RUNNER, str(bad), "--outdir", str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 1 and "ela3d_plan_create" in r.stderr
    r = subprocess.run([RUNNER, str(tmp_path / "missing.txt")], capture_output=True, text=True)
    assert r.returncode == 1 and "cannot open" in r.stderr
