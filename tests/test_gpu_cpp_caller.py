"""A C++ caller of the C ABI, as a maintainer of the reference would write
it in place of main(): compiled with g++ against include/ela3d.h, linked to
the in-tree libela3d.so, run on the GPU.  Its seismograms must equal the
same shot run through the Python mirror bit for bit (same kernels, same
tuning), and a checkpoint written by the C++ program must resume in Python."""
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <cstdio>
#include <vector>
#include "ela3d.h"

#define TRY(call) do { ela3d_status s_ = (call); if (s_ != ELA3D_OK) { \
    std::fprintf(stderr, "%s: %s (%s)\n", #call, ela3d_status_string(s_), ela3d_last_error()); return 1; } } while (0)

int main(int argc, char **argv) {
    ela3d_params p;
    TRY(ela3d_params_default(&p));               // the reference's literals
    p.nx = 48; p.ny = 40; p.nz = 36;             // NIMX, NIMY, NIMZ
    p.nstep = 120; p.npml = 6; p.sampgat = 2;    // NSTEP, NPOINTS_PML, sampgat
    p.f0 = 25; p.t0 = 1.2 / 25;
    p.src_i = 24; p.src_j = 20; p.src_k = 12;    // 0-based ISOURCE-1 ...
    std::vector<int32_t> rec;
    for (int i = 4; i < 44; i += 4) { rec.push_back(i); rec.push_back(20); rec.push_back(14); }
    p.rec = rec.data(); p.nrec = (int32_t)(rec.size() / 3);
    const size_t n = (size_t)p.nx * p.ny * p.nz;
    std::vector<float> cp(n), cs(n), rho(n);
    for (size_t q = 0; q < n; ++q) {             // two layers, like a model*.bin fill
        const bool deep = q / ((size_t)p.nx * p.ny) >= 18;
        cp[q] = deep ? 3600.f : 3000.f; cs[q] = cp[q] / 1.73f; rho[q] = deep ? 2500.f : 2200.f;
    }
    ela3d_plan *plan = nullptr;
    TRY(ela3d_plan_create(&p, cp.data(), cs.data(), rho.data(), &plan));
    TRY(ela3d_run(plan, 60));                    // the it loop, resumable
    int64_t bytes = 0;
    TRY(ela3d_checkpoint_size(plan, &bytes));
    std::vector<unsigned char> ck((size_t)bytes);
    TRY(ela3d_checkpoint_save(plan, ck.data(), bytes));
    TRY(ela3d_run(plan, p.nstep - 60));
    std::vector<float> seis((size_t)p.nrec * 3 * (p.nstep / p.sampgat));
    TRY(ela3d_get_seismograms(plan, seis.data()));
    TRY(ela3d_plan_destroy(plan));
    FILE *f = std::fopen(argv[1], "wb");
    std::fwrite(seis.data(), sizeof(float), seis.size(), f);
    std::fclose(f);
    f = std::fopen(argv[2], "wb");
    std::fwrite(ck.data(), 1, ck.size(), f);
    std::fclose(f);
    return 0;
}
"""


def test_cpp_caller_matches_python_and_checkpoint_resumes(built, tmp_path):
    from ela3d_gb300 import Plan
    from ela3d_gb300._build import LIB, OUT
    from ela3d_gb300.params import reference_defaults

    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    src = tmp_path / "main.cpp"
    exe = tmp_path / "main"
    src.write_text(PROGRAM)
    subprocess.run(["g++", "-O2", "-std=c++17", str(src), "-I", os.path.join(ROOT, "include"), "-L", OUT,
                    "-lela3d", f"-Wl,-rpath,{OUT}", "-o", str(exe)], check=True)
    seis_path, ck_path = tmp_path / "seis.bin", tmp_path / "ck.bin"
    r = subprocess.run([str(exe), str(seis_path), str(ck_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert os.path.exists(LIB)

    nx, ny, nz = 48, 40, 36
    rec = np.array([[i, 20, 14] for i in range(4, 44, 4)], np.int32)
    p = reference_defaults().with_(nx=nx, ny=ny, nz=nz, nstep=120, npml=6, sampgat=2, f0=25.0, t0=1.2 / 25,
                                   src=(24, 20, 12), rec=rec, it_output=0)
    deep = (np.arange(nz) >= 18)[:, None, None] & np.ones((nz, ny, nx), bool)
    cp = np.where(deep, 3600.0, 3000.0).astype(np.float32)
    cs = (cp / np.float32(1.73)).astype(np.float32)
    rho = np.where(deep, 2500.0, 2200.0).astype(np.float32)
    want_shape = (len(rec), 3, p.nstep // p.sampgat)
    got = np.fromfile(seis_path, np.float32).reshape(want_shape)
    with Plan(p, cp, cs, rho) as plan:
        plan.run(p.nstep)
        mine = plan.seismograms()
    assert np.any(mine != 0)
    assert np.array_equal(got, mine)
    with Plan(p, cp, cs, rho) as resumed:       # the C++ program's checkpoint, in Python
        resumed.restore(np.fromfile(ck_path, np.uint8))
        assert resumed.info().step == 60
        resumed.run(p.nstep - 60)
        assert np.array_equal(resumed.seismograms(), mine)
