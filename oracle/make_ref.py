"""Build the reference CPU program as a parity oracle.  TEST INFRASTRUCTURE.

Reads the unmodified reference source
``seismicCPML_3d_isotropic_simpelmodel.cpp`` from the reference checkout,
applies a mechanical parameter patch, and writes the result plus binaries
into ``oracle/_ref/`` (git-ignored; nothing from the reference is committed).

The patch only turns hard-coded literals into fields of ``g_cfg``
(oracle/ref_harness.h) and adds hooks; the time-loop arithmetic is left as
written.  Changes, each asserted to match exactly the expected number of
times so that a different reference fails loudly:

- main() reads a config file; NIMX/NIMY/NIMZ, NSTEP, DELTATT, sampgat,
  IT_OUTPUT, DELTAX, f0, t0, factor, NPOINTS_PML, source position, angle,
  NPOWER, K_MAX_PML, ALPHA_MAX_PML, Rcoef and vpml come from it (:20-153);
- every full-grid malloc becomes a calloc with one extra z-plane, so the
  read of plane NIMZ+1 by the sigma_xz/sigma_yz loop (:450,:477) sees zeros;
- the model is loaded from binary files after the constant fill (:45-59);
- the source time function may be the Ricker (elatic_3d_unified_cuda_memory.cu:441)
  and the injection a force into velocity
  (seismicCPML_3d_isotropic_cudazerocopy.cu:451-453), selected by config;
- per-step console output is removed;
- receivers are recorded from the velocity after the update, before the
  source, exactly where the program gathers its plane (:592-604);
- optional "clean" switch fixes the a_x_half assignment (:223), the zmin
  half-node abscissa (:331) and the z normalisation, and clamps alpha at 0 on
  y and z as on x (:217-218), for checking the textbook C-PML variant;
- a float64 variant replaces ``float`` by ``double`` and the f-suffixed
  libm calls by their double versions.

It also builds the reference's FP32 GPU program
``seismicCPML_3d_isotropic_cudazerocopy.cu`` (all arrays in device memory,
five stencil kernels per step with 10x10x10-thread blocks) as a timing
baseline, with a patch that changes no kernel: the grid edge, step count and
warm-up come from the command line (:488-491,:521); blocks become 8x8x8
threads so that a 256-cell edge is covered exactly (:1361-1369; with 10 the
last 6 cells of each axis would never be updated); the per-step receiver text
and the snapshot files are switched off by a flag (:1385,:1423); the time
after the warm-up steps and the launch status are printed after the loop.
Its kernels' indices were checked by reading for cubic grids whose edge is a
multiple of 8: every neighbour access stays inside the arrays.

And the reference's FP64 GPU program ``elatic_3d_unified_cuda_memory.cu``
(all arrays in managed memory, seven kernels per step with 5x5x5-thread
blocks), with a patch that changes no kernel and no launch shape: grid edge,
steps and warm-up from the command line (:499-501,:530), the per-step
receiver text, the snapshots and the initial model dump switched off by the
same flag (:583-591,:1110,:1154), its thirty managed grid arrays prefetched
to the GPU before the loop (first touched by the host, they would otherwise
migrate page by page inside the timed steps), and the same timing line.  Its
kernels' indices were checked by reading: every neighbour access is guarded
by the update ranges; for an edge divisible by 5 the blocks cover the grid
exactly.

Usage: python oracle/make_ref.py [--ref DIR] [--no-build]
(DIR defaults to ELA3D_REFERENCE_DIR, else a ``reference`` directory beside
this repository.)
"""
from __future__ import annotations

import argparse
import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REF_NAME = "seismicCPML_3d_isotropic_simpelmodel.cpp"
GPU_REF_NAME = "seismicCPML_3d_isotropic_cudazerocopy.cu"


def reference_dir() -> str | None:
    """The reference checkout: ``ELA3D_REFERENCE_DIR`` when set, else a
    ``reference`` directory beside this repository; None when neither holds
    the reference source."""
    cands = [os.environ.get("ELA3D_REFERENCE_DIR"),
             os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")]
    for c in cands:
        if c and os.path.exists(os.path.join(c, REF_NAME)):
            return c
    return None


def _sub(src: str, old: str, new: str, count: int = 1) -> str:
    n = src.count(old)
    if n != count:
        raise RuntimeError(f"patch anchor matched {n} times (expected {count}): {old!r}")
    return src.replace(old, new)


def patch(src: str) -> str:
    s = src.replace("\r\n", "\n")
    s = _sub(s, '#include "conio.h"', '#include "conio.h"\n#include "ref_harness.h"')
    s = _sub(s, "int main(void) {", "int main(int argc, char **argv) {\n\tref_load_cfg(argc, argv);")
    for name, field in (("NIMX = 500;", "NIMX = g_cfg.nx;"), ("NIMY = 500;", "NIMY = g_cfg.ny;"),
                        ("NIMZ = 500;", "NIMZ = g_cfg.nz;")):
        s = _sub(s, name, field)
    s = _sub(s, "int Ngatx = 100;", "int Ngatx = g_cfg.ngatx;")
    s = _sub(s, "int Ngaty = 5;", "int Ngaty = g_cfg.ngaty;")
    s = _sub(s, "int NSTEP = 1000;", "int NSTEP = g_cfg.nstep;")
    s = _sub(s, "float DELTATT = 1e-3;", "float DELTATT = g_cfg.dt;")
    s = _sub(s, "int sampgat = 2;", "int sampgat = g_cfg.sampgat;")
    s = _sub(s, "int IT_OUTPUT = 200;", "int IT_OUTPUT = g_cfg.it_output;")
    s = _sub(s, "DELTAX = 10;", "DELTAX = g_cfg.dx;")
    s = _sub(s, "(float*)malloc(sizeof(float)*(DIMX*DIMY*DIMZ))",
             "(float*)calloc(1, sizeof(float)*(DIMX*DIMY*(DIMZ+1)))", count=30)
    s = _sub(s, "\tfloat f0, t0, factor;",
             "\tref_load_model(ccp, ccs, crho, NIMX, NIMY, NIMZ);\n\tfloat f0, t0, factor;")
    s = _sub(s, "f0 = 35;", "f0 = g_cfg.f0;")
    s = _sub(s, "t0 = 1.2 / f0;", "t0 = g_cfg.t0;")
    s = _sub(s, "factor = 1e+7;", "factor = g_cfg.factor;")
    s = _sub(s, "int NPOINTS_PML = 10;", "int NPOINTS_PML = g_cfg.npml;")
    s = _sub(s, "ISOURCEE = DIMX / 2;", "ISOURCEE = g_cfg.src_i + 1;")
    s = _sub(s, "JSOURCEE = DIMY / 2;", "JSOURCEE = g_cfg.src_j + 1;")
    s = _sub(s, "KSOURCEE = 11;", "KSOURCEE = g_cfg.src_k + 1;")
    s = _sub(s, "float ANGLE_FORCEE = 0;", "float ANGLE_FORCEE = g_cfg.angle;")
    s = _sub(s, "float NPOWER = 2;", "float NPOWER = g_cfg.npower;")
    s = _sub(s, "float K_MAX_PML = 1;", "float K_MAX_PML = g_cfg.k_max;")
    s = _sub(s, "float ALPHA_MAX_PML = 2 * PI*(f0 / 2);",
             "float ALPHA_MAX_PML = 2 * PI*(f0 / 2);\n\tif (g_cfg.alpha_max >= 0) ALPHA_MAX_PML = g_cfg.alpha_max;")
    s = _sub(s, "Rcoef = 0.001;", "Rcoef = g_cfg.rcoef;")
    s = _sub(s, "float vpml = 3000;", "float vpml = g_cfg.vpml;")
    # optional textbook fixes (off unless the config says clean 1)
    s = _sub(s, "{ calpha_x_half[i] = cd_x_half[i] * (cb_x_half[i] - 1.0)",
             "{ (g_cfg.clean ? ca_x_half[i] : calpha_x_half[i]) = cd_x_half[i] * (cb_x_half[i] - 1.0)")
    head, zsec = s.split("//-----------------PML Z", 1)
    zsec, tail = zsec.split("float *gatvx", 1)
    zsec = _sub(zsec, "abscissa_in_PML = yoriginbottom - (yval + DELTAY / 2.0);",
                "abscissa_in_PML = g_cfg.clean ? (zoriginbottom - (zval + DELTAZ / 2.0)) : "
                "(yoriginbottom - (yval + DELTAY / 2.0));")
    zsec = _sub(zsec, "abscissa_normalized = abscissa_in_PML / thickness_PML_y;",
                "abscissa_normalized = abscissa_in_PML / (g_cfg.clean ? thickness_PML_z : thickness_PML_y);",
                count=3)
    zsec = _sub(zsec, "\t\tcb_z[i] = expf(",
                "\t\tif (g_cfg.clean) { if (calpha_z[i] < 0.0) calpha_z[i] = 0.0;"
                " if (calpha_z_half[i] < 0.0) calpha_z_half[i] = 0.0; }\n\t\tcb_z[i] = expf(")
    s = head + "//-----------------PML Z" + zsec + "float *gatvx" + tail
    s = _sub(s, "\t\tcb_y[i] = expf(",
             "\t\tif (g_cfg.clean) { if (calpha_y[i] < 0.0) calpha_y[i] = 0.0;"
             " if (calpha_y_half[i] < 0.0) calpha_y_half[i] = 0.0; }\n\t\tcb_y[i] = expf(")
    # time loop hooks
    s = _sub(s, "for (int it = 1; it <= NSTEP; it++) {",
             "for (int it = 1; it <= NSTEP; it++) {\n\t\tref_step_hook(it);")
    s = _sub(s, "}//end it", "}//end it\n\tref_step_hook(NSTEP + 1);")
    s = _sub(s, "\t\t//addsource", "\t\tref_record(it, cvx, cvy, cvz, NIMX, NIMY);\n\t\t//addsource")
    s = _sub(s, "cout << endl << lesource;", "")
    s = _sub(s, "cout << endl << it;", "")
    s = _sub(s, 'cout << endl << xlen << " " << ylen;', "")
    s = _sub(s, "float source_term = -factor * 2.0*a*(t - t0)*expf(-a*powf((t - t0), 2));",
             "float source_term = (g_cfg.stf == 1) ? (float)(-factor * 2.0*a*(t - t0)*expf(-a*powf((t - t0), 2)))"
             " : (g_cfg.stf == 2) ? (float)(factor * expf(-a*powf((t - t0), 2)))"
             " : (float)(factor*(1.0 - 2.0*a*powf((t - t0), 2))*expf(-a*powf(t - t0, 2)));")
    s = _sub(s, "\t\tcsigmaxx[lesource] = csigmaxx[lesource] + force_x*DELTATT * lambdaplus2mu;",
             "\t\tif (g_cfg.src_kind == 1) {\n"
             "\t\tcsigmaxx[lesource] = csigmaxx[lesource] + force_x*DELTATT * lambdaplus2mu;")
    s = _sub(s, "\t\tcsigmazz[lesource] = csigmazz[lesource] + force_y*DELTATT * lambdaplus2mu;",
             "\t\tcsigmazz[lesource] = csigmazz[lesource] + force_y*DELTATT * lambdaplus2mu;\n"
             "\t\t} else {\n"
             "\t\tif (g_cfg.w[0] != 0.0) { float fsrc = (float)g_cfg.w[0] * source_term;"
             " cvx[lesource] = cvx[lesource] + fsrc*DELTATT / ((crho[lesource] + crho[lesource - 1]) / 2); }\n"
             "\t\tif (g_cfg.w[1] != 0.0) { float fsrc = (float)g_cfg.w[1] * source_term;"
             " cvy[lesource] = cvy[lesource] + fsrc*DELTATT / ((crho[lesource] + crho[lesource + NIMX]) / 2); }\n"
             "\t\tif (g_cfg.w[2] != 0.0) { float fsrc = (float)g_cfg.w[2] * source_term;"
             " cvz[lesource] = cvz[lesource] + fsrc*DELTATT / ((crho[lesource] + crho[lesource + NIMX * NIMY]) / 2); }\n"
             "\t\t}")
    s = _sub(s, "\tfree(cvx); ",
             "\tref_finish(cvx, cvy, cvz, csigmaxx, csigmayy, csigmazz, csigmaxy, csigmaxz, csigmayz,"
             " NIMX, NIMY, NIMZ);\n\tfree(cvx); ")
    return s


def patch_gpu(src: str) -> str:
    """The FP32 GPU program, made runnable at a given size without file I/O
    in the timed loop (kernels untouched)."""
    s = src.replace("\r\n", "\n")
    s = _sub(s, "#include <iomanip>", "#include <iomanip>\n#include <chrono>")
    s = _sub(s, "int main(void) {", "int main(int argc, char **argv) {\n"
             "\tconst int ref_n = argc > 1 ? atoi(argv[1]) : 200;\n"
             "\tconst int ref_warm = argc > 3 ? atoi(argv[3]) : 0;\n"
             "\tconst int ref_io = argc > 4 ? atoi(argv[4]) : 1;")
    s = _sub(s, "\tNIMX = 200;\n\tNIMY = 200;\n\tNIMZ = 200;", "\tNIMX = ref_n;\n\tNIMY = ref_n;\n\tNIMZ = ref_n;")
    s = _sub(s, "int NSTEP = 200;", "int NSTEP = argc > 2 ? atoi(argv[2]) : 200;")
    for ax in "xyz":
        s = _sub(s, f"threads.{ax} = 10;", f"threads.{ax} = 8;")
    s = _sub(s, "\tfor (int it = 1; it <= NSTEP; it++) {",
             "\tstd::chrono::steady_clock::time_point ref_t0 = std::chrono::steady_clock::now();\n"
             "\tfor (int it = 1; it <= NSTEP; it++) {\n"
             "\t\tif (it == ref_warm + 1) { cudaDeviceSynchronize(); ref_t0 = std::chrono::steady_clock::now(); }")
    s = _sub(s, "if (fmod(it, sampgat) == 0) {", "if (ref_io && fmod(it, sampgat) == 0) {")
    s = _sub(s, "if (fmod(it, IT_OUTPUT) == 0){", "if (ref_io && fmod(it, IT_OUTPUT) == 0){")
    s = _sub(s, "\tfree(tempvz); free(tempvy); free(tempvx);",
             "\t{\n\t\tcudaError_t ref_e = cudaDeviceSynchronize();\n"
             "\t\tif (ref_e == cudaSuccess) ref_e = cudaGetLastError();\n"
             "\t\tconst double ref_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - ref_t0).count();\n"
             "\t\tprintf(\"ELA3D_REF_GPU n %d steps %d seconds %.9f status %d\\n\", NIMX, NSTEP - ref_warm, ref_s,"
             " (int)ref_e);\n\t}\n"
             "\tfree(tempvz); free(tempvy); free(tempvx);")
    return s


GPU64_REF_NAME = "elatic_3d_unified_cuda_memory.cu"
# the managed grid arrays of the FP64 GPU program (prefetched to the device
# before its time loop, so that the loop times its kernels and not page
# migration)
_GPU64_ARRAYS = ("cp", "cs", "rho", "vx", "vy", "vz", "sigmaxx", "sigmaxy", "sigmayy", "sigmazz", "sigmaxz",
                 "sigmayz", "memory_dvx_dx", "memory_dvx_dy", "memory_dvx_dz", "memory_dvy_dx", "memory_dvy_dy",
                 "memory_dvy_dz", "memory_dvz_dx", "memory_dvz_dy", "memory_dvz_dz", "memory_dsigmaxx_dx",
                 "memory_dsigmayy_dy", "memory_dsigmazz_dz", "memory_dsigmaxy_dx", "memory_dsigmaxy_dy",
                 "memory_dsigmaxz_dx", "memory_dsigmaxz_dz", "memory_dsigmayz_dy", "memory_dsigmayz_dz")


def patch_gpu64(src: str) -> str:
    """The FP64 GPU program (managed memory, 5x5x5-thread blocks), made
    runnable at a given size without file I/O in the timed loop; kernels and
    launch shapes untouched.  Its managed grid arrays, first touched by the
    host, are prefetched to the GPU before the loop."""
    s = src.replace("\r\n", "\n")
    s = _sub(s, "#include <iomanip>", "#include <iomanip>\n#include <chrono>")
    s = _sub(s, "int main(void) {", "int main(int argc, char **argv) {\n"
             "\tconst int ref_n = argc > 1 ? atoi(argv[1]) : 373;\n"
             "\tconst int ref_warm = argc > 3 ? atoi(argv[3]) : 0;\n"
             "\tconst int ref_io = argc > 4 ? atoi(argv[4]) : 1;")
    s = _sub(s, "\tNIMX = 373;\n\tNIMY = 373;\n\tNIMZ = 373;", "\tNIMX = ref_n;\n\tNIMY = ref_n;\n\tNIMZ = ref_n;")
    s = _sub(s, "int NSTEP = 200;", "int NSTEP = argc > 2 ? atoi(argv[2]) : 200;")
    s = _sub(s, "foutt.write((char *)&rho[ijk], sizeof rho[ijk]);",
             "if (ref_io) foutt.write((char *)&rho[ijk], sizeof rho[ijk]);")
    arrays = ", ".join(_GPU64_ARRAYS)
    s = _sub(s, "\tdim3 threads;\n",
             "\t{\n\t\tint ref_dev = 0;\n\t\tHANDLE_ERROR(cudaGetDevice(&ref_dev));\n"
             "\t\tcudaMemLocation ref_loc;\n\t\tref_loc.type = cudaMemLocationTypeDevice;\n"
             "\t\tref_loc.id = ref_dev;\n"
             f"\t\tdouble *ref_arrays[] = {{{arrays}}};\n"
             "\t\tfor (double *ref_a : ref_arrays)\n"
             "\t\t\tHANDLE_ERROR(cudaMemPrefetchAsync(ref_a, sizeof(double)*NIMX*NIMY*NIMZ, ref_loc, 0, 0));\n"
             "\t\tHANDLE_ERROR(cudaDeviceSynchronize());\n\t}\n"
             "\tdim3 threads;\n")
    s = _sub(s, "\tfor (int it = 1; it <= NSTEP; it++){",
             "\tstd::chrono::steady_clock::time_point ref_t0 = std::chrono::steady_clock::now();\n"
             "\tfor (int it = 1; it <= NSTEP; it++){\n"
             "\t\tif (it == ref_warm + 1) { cudaDeviceSynchronize(); ref_t0 = std::chrono::steady_clock::now(); }")
    s = _sub(s, "if (fmod(it, sampgat) == 0) {", "if (ref_io && fmod(it, sampgat) == 0) {")
    s = _sub(s, "if (fmod(it, IT_OUTPUT) == 0){", "if (ref_io && fmod(it, IT_OUTPUT) == 0){")
    s = _sub(s, "\tchar nmfilesx[20], nmfilesy[20], nmfilesz[20];",
             "\t{\n\t\tcudaError_t ref_e = cudaDeviceSynchronize();\n"
             "\t\tif (ref_e == cudaSuccess) ref_e = cudaGetLastError();\n"
             "\t\tconst double ref_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - ref_t0).count();\n"
             "\t\tprintf(\"ELA3D_REF_GPU n %d steps %d seconds %.9f status %d\\n\", NIMX, NSTEP - ref_warm, ref_s,"
             " (int)ref_e);\n\t}\n"
             "\tif (!ref_io) return 0;\n"
             "\tchar nmfilesx[20], nmfilesy[20], nmfilesz[20];")
    return s


def gpu_compiler_cmd(src: str, exe: str) -> list[str]:
    # 512-thread blocks: at most 128 registers a thread (the kernels' launches
    # are not error-checked by the program, so the cap keeps every launch valid)
    return ["nvcc", "-O3", "-gencode", "arch=compute_103a,code=sm_103a", "-maxrregcount=128", "-w",
            "-Dsprintf_s=sprintf", "-I", OUT, src, "-o", exe]


def to_f64(s: str) -> str:
    s = re.sub(r"\bfloat\b", "double", s)
    for f in ("expf", "powf", "logf", "sinf", "cosf"):
        s = re.sub(r"\b%s\(" % f, f[:-1] + "(", s)
    return s


def compiler_cmd(src: str, exe: str) -> list[str]:
    return ["g++", "-O3", "-ffp-contract=off", "-w", "-Dsprintf_s=sprintf",
            "-I", OUT, "-I", HERE, src, "-o", exe]


def _write_if_changed(path: str, text: str) -> None:
    """Leaves an identical file alone, so that its binary is not rebuilt."""
    if os.path.exists(path):
        with open(path, "r") as f:
            if f.read() == text:
                return
    with open(path, "w") as f:
        f.write(text)


def generate(ref_dir: str) -> None:
    with open(os.path.join(ref_dir, REF_NAME), "r", encoding="latin-1") as f:
        src = f.read()
    os.makedirs(OUT, exist_ok=True)
    p32 = patch(src)
    _write_if_changed(os.path.join(OUT, "ref_f32.cpp"), p32)
    _write_if_changed(os.path.join(OUT, "ref_f64.cpp"), to_f64(p32))
    _write_if_changed(os.path.join(OUT, "conio.h"), "/* empty stand-in for the Windows console header */\n")
    gpu = os.path.join(ref_dir, GPU_REF_NAME)
    if os.path.exists(gpu):
        with open(gpu, "r", encoding="latin-1") as f:
            g = patch_gpu(f.read())
        _write_if_changed(os.path.join(OUT, "ref_gpu_f32.cu"), g)
    gpu64 = os.path.join(ref_dir, GPU64_REF_NAME)
    if os.path.exists(gpu64):
        with open(gpu64, "r", encoding="latin-1") as f:
            g = patch_gpu64(f.read())
        _write_if_changed(os.path.join(OUT, "ref_gpu_f64.cu"), g)


def build() -> list[str]:
    """Compile whatever patched sources exist in oracle/_ref (no reference read)."""
    built = []
    procs = []
    for v in ("f32", "f64"):
        src = os.path.join(OUT, f"ref_{v}.cpp")
        if not os.path.exists(src):
            continue
        exe = os.path.join(OUT, f"ref_{v}")
        procs.append((exe, subprocess.Popen(compiler_cmd(src, exe))))
    for name in ("ref_gpu_f32", "ref_gpu_f64"):
        gsrc = os.path.join(OUT, name + ".cu")
        if os.path.exists(gsrc) and shutil.which("nvcc"):
            exe = os.path.join(OUT, name)
            procs.append((exe, subprocess.Popen(gpu_compiler_cmd(gsrc, exe))))
    for exe, p in procs:
        if p.wait() != 0:
            raise RuntimeError(f"building {exe} failed")
        built.append(exe)
    return built


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None)
    ap.add_argument("--no-build", action="store_true")
    a = ap.parse_args()
    ref = a.ref or reference_dir()
    if ref and os.path.exists(os.path.join(ref, REF_NAME)):
        generate(ref)
    elif not os.path.exists(os.path.join(OUT, "ref_f32.cpp")):
        print("reference source not found and no patched copy present", file=sys.stderr)
        return 1
    if not a.no_build:
        for exe in build():
            print(exe)
    return 0


if __name__ == "__main__":
    sys.exit(main())
