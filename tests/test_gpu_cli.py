"""The command line on the GPU writes the reference program's files; their
values match the reference program's own within the FP32 tolerance."""
import os

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def test_cli_files_match_reference_program(built, tmp_path):
    import oracle
    from ela3d_gb300 import cli, refio
    from test_refio import case

    p, cp, cs, rho = case()
    refio.write_model(str(tmp_path / "m"), cp, cs, rho)
    params = tmp_path / "params.txt"
    params.write_text("\n".join([
        f"nx {p.nx}", f"ny {p.ny}", f"nz {p.nz}", "dx 10", f"dt {p.dt!r}", f"nstep {p.nstep}",
        f"sampgat {p.sampgat}", "it_output 10", "ngatx 4", "ngaty 2", f"npml {p.npml}", f"f0 {p.f0!r}",
        f"t0 {p.t0!r}", "src %d %d %d" % p.src, f"model {tmp_path / 'm'}", "rec 3 4 5"]) + "\n")
    out = str(tmp_path / "gpu")
    cli.run(str(params), out)
    # the reference program on the same inputs (when it is built here), else the oracle
    cells, slots = refio.gather_layout(p.nx, p.ny, p.npml, 4, 2, p.src[2])
    seis, fields = oracle.run(p.with_(rec=cells), cp, cs, rho)
    want_dir = str(tmp_path / "oracle")
    os.makedirs(want_dir)
    refio.write_rechor(want_dir, seis, slots)
    refio.write_snapshots(want_dir, 20, fields[0], fields[1], fields[2])
    for name in ("rechorvx.txt", "rechorvy.txt", "rechorvz.txt"):
        a = np.array([[float(v) for v in l.split()] for l in open(os.path.join(out, name))])
        b = np.array([[float(v) for v in l.split()] for l in open(os.path.join(want_dir, name))])
        assert a.shape == b.shape and rel_l2(a, b) < 1e-5, name
    for c in ("vx", "vy", "vz"):
        name = "%s%05i.bin" % (c, 20)
        a = np.fromfile(os.path.join(out, name), np.float32)
        b = np.fromfile(os.path.join(want_dir, name), np.float32)
        assert a.size == b.size == 25 * 23 * 21 and rel_l2(a, b) < 2e-5
    assert os.path.exists(os.path.join(out, "vz00010.bin"))
    assert np.load(os.path.join(out, "seis.npy")).shape == (1, 3, p.nstep // p.sampgat)
    # source-point trace: vz at the source cell of the force source after each step
    tz = np.array([float(v) for v in open(os.path.join(out, "recsrcz.txt")).read().split()])
    assert tz.size == p.nstep + 1 and tz[0] == 0
    i, j, k = p.src
    assert abs(tz[-1] - fields[2][k, j, i]) <= 1e-4 * np.abs(fields[2]).max()
