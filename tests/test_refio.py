"""The reference program's file formats (CPU).  The oracle reproduces the
reference bit for bit, so its traces and fields written through
ela3d_gb300.refio must equal, byte for byte, the files the reference
program writes itself (rechorv?.txt receiver text, v?%05i.bin snapshots)."""
import os

import numpy as np
import pytest


def case():
    from ela3d_gb300 import ShotParams, media

    nx, ny, nz = 24, 22, 20
    p = ShotParams(nx=nx, ny=ny, nz=nz, nstep=20, dt=1e-3, npml=3, f0=30.0, t0=0.04, src=(11, 10, 8),
                   sampgat=2)
    cp, cs, rho = media.anticline_layers(nx, ny, nz, depths=(5, 10, 15, 40), amp=2, sigma=6, seed=5)
    return p, cp, cs, rho


@pytest.mark.parametrize("ngatx,ngaty", [(4, 2), (1, 1), (24, 16)])
def test_receiver_text_and_snapshots_byte_identical(tmp_path, ngatx, ngaty):
    import oracle
    from ela3d_gb300 import refio

    if oracle.reference_binary(False) is None:
        pytest.skip("reference program not built in this checkout (oracle/_ref)")
    p, cp, cs, rho = case()
    wd = str(tmp_path / "ref")
    os.makedirs(wd)
    oracle.run_reference(p, cp, cs, rho, workdir=wd, ngatx=ngatx, ngaty=ngaty, it_output=10)
    cells, slots = refio.gather_layout(p.nx, p.ny, p.npml, ngatx, ngaty, p.src[2])
    seis, fields = oracle.run(p.with_(rec=cells), cp, cs, rho)
    out = str(tmp_path / "ours")
    os.makedirs(out)
    refio.write_rechor(out, seis, slots)
    for name in ("rechorvx.txt", "rechorvy.txt", "rechorvz.txt"):
        assert open(os.path.join(out, name), "rb").read() == open(os.path.join(wd, name), "rb").read(), name
    refio.write_snapshots(out, 20, fields[0], fields[1], fields[2])
    _, f10 = oracle.run(p, cp, cs, rho, nsteps=10)
    refio.write_snapshots(out, 10, f10[0], f10[1], f10[2])
    for it in (10, 20):
        for c in ("vx", "vy", "vz"):
            name = "%s%05i.bin" % (c, it)
            assert open(os.path.join(out, name), "rb").read() == open(os.path.join(wd, name), "rb").read(), name


def test_snapshot_index_covers_every_cell():
    from ela3d_gb300.refio import snapshot_index

    for nx, ny, nz in ((5, 4, 3), (24, 22, 20)):
        idx = snapshot_index(nx, ny, nz)
        assert idx.size == (nx + 1) * (ny + 1) * (nz + 1)
        live = idx[idx >= 0]
        assert set(live.tolist()) == set(range(nx * ny * nz))


def test_model_files_roundtrip(tmp_path):
    from ela3d_gb300 import refio
    from ela3d_gb300.media import anticline_layers

    cp, cs, rho = anticline_layers(9, 7, 5, depths=(1, 2, 3, 4), amp=1, sigma=2, seed=1)
    prefix = str(tmp_path / "model")
    refio.write_model(prefix, cp, cs, rho)
    assert os.path.getsize(prefix + "cp.bin") == 9 * 7 * 5 * 4
    a, b, c = refio.read_model(prefix, 9, 7, 5)
    assert np.array_equal(a, cp) and np.array_equal(b, cs) and np.array_equal(c, rho)


def test_too_many_receivers_rejected_like_the_reference():
    from ela3d_gb300.refio import gather_layout

    with pytest.raises(ValueError):
        gather_layout(20, 20, 10, 4, 2, 5)   # ylen = (20 - 20) / 2 = 0


def test_recsrc_text_matches_cpp_iostream(tmp_path):
    """recsrc?.txt values are printed by `fout << double << " "`
    (elatic_3d_unified_cuda_memory.cu:1205-1223); pinned against g++."""
    import shutil
    import subprocess

    from ela3d_gb300 import refio

    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    vals = np.array([0.0, 1.5, -2.25e-7, 123456789.0, 3.14159265358979, 1e-300, -0.0, 7.0e5, 1234567.0,
                     0.000123456789, -98765.4321], np.float64)
    src = tmp_path / "w.cpp"
    src.write_text('#include <fstream>\n#include <cstdlib>\nint main(int c, char **v) {\n'
                   '  std::ofstream f(v[1]);\n  for (int i = 2; i < c; ++i) f << std::strtod(v[i], 0) << " ";\n}\n')
    exe = tmp_path / "w"
    subprocess.run(["g++", "-O1", str(src), "-o", str(exe)], check=True)
    out = tmp_path / "recsrcx.txt"
    subprocess.run([str(exe), str(out)] + [repr(float(v)) for v in vals], check=True)
    assert refio.recsrc_text(vals) == out.read_text()
    paths = refio.write_recsrc(str(tmp_path), np.stack([vals, vals * 2, vals * 3]))
    assert [os.path.basename(q) for q in paths] == ["recsrcx.txt", "recsrcy.txt", "recsrcz.txt"]
    assert open(paths[0]).read() == out.read_text()
