"""The two runners' parameter files on the host (no GPU): both read the same
keys, reject an unknown key (a misspelt one would otherwise fall back to its
default silently), and the C++ runner exits 1 on bad input before any device
work."""
import os
import re
import subprocess

import pytest

from conftest import ROOT


def _runner():
    from ela3d_gb300._build import RUNNER

    return RUNNER


def test_both_runners_read_the_same_keys(built):
    from ela3d_gb300 import cli

    src = open(os.path.join(ROOT, "ela3d_gb300", "csrc", "ela3d_run.cpp")).read()
    block = re.search(r"kKeys\[\] = \{(.*?)\};", src, re.S).group(1)
    assert tuple(re.findall(r'"([a-z0-9_]+)"', block)) == cli.KEYS


def test_python_runner_rejects_unknown_keys_and_reads_energy_every(built, tmp_path):
    from ela3d_gb300 import cli

    good = tmp_path / "good.txt"
    good.write_text("nx 40\nny 30\nnz 20\nnstep 5\nsrc 20 15 10\nenergy_every 7\n# a comment\nrec 1 2 3\n")
    p, extra = cli.parse_params(str(good))
    assert (p.nx, p.ny, p.nz, p.nstep, p.energy_every) == (40, 30, 20, 5, 7) and p.nrec == 1
    bad = tmp_path / "bad.txt"
    bad.write_text("nx 40\nnsetp 5\n")
    with pytest.raises(ValueError, match="nsetp"):
        cli.parse_params(str(bad))


@pytest.mark.parametrize("text,args,message", [
    (None, [], "usage"),
    (None, ["/nonexistent/params.txt"], "cannot open"),
    ("nx 40\nny 30\nnz 20\nnsetp 5\n", None, "unknown key nsetp"),
    ("nx 2\nny 30\nnz 20\nsrc 1 1 1\n", None, "at least 3 cells"),
    ("nx 40\nny 30\nnz 20\nsrc 50 1 1\n", None, "source outside the grid"),
    ("nx 40\nny 30\nnz 20\nsrc 5 5 5\nmodel /nonexistent/m\n", None, "cannot open"),
])
def test_cpp_runner_bad_input_exits_1(built, tmp_path, text, args, message):
    if args is None:
        path = tmp_path / "params.txt"
        path.write_text(text)
        args = [str(path), "--outdir", str(tmp_path / "out")]
    r = subprocess.run([_runner()] + args, capture_output=True, text=True, timeout=120)
    assert r.returncode == 1, (r.returncode, r.stderr)
    assert message in r.stderr
