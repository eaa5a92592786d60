"""The reference program's files: receiver text, snapshots, model input.

- ``gather_layout``: which cells the receiver text lines of
  seismicCPML_3d_isotropic_simpelmodel.cpp hold.  The program copies plane
  KSOURCE+1 (1-based; one below the source) of vx, vy, vz into a buffer
  indexed i + j*NIMX for 1-based i, j (:593-602) and, every sampgat steps,
  prints the buffer entries kk = i + j*NIMX for i = 0, xlen, ... < DIMX and
  j = 0, ylen, ... < DIMY with xlen = NIMX / Ngatx and
  ylen = (NIMY - 2 NPOINTS_PML) / Ngaty (:629-670).  Entry kk is 1-based cell
  ((kk-1) % NIMX + 1, (kk-1) / NIMX) when that row index is in [1, NIMY];
  other entries are never written and stay 0.
- ``rechor_text``: one file's content, values printed as C++ iostream does
  by default (6 significant digits, ``%g``), each followed by a space, one
  line per sample.
- ``snapshot_bytes``: a v?%05i.bin file (:685-722): DIMX*DIMY*DIMZ values
  read at address ii + jj*NIMX + kk*NIMX*NIMY, which with the program's
  1-based cells maps each address to a cell or to never-written zeros.
- ``recsrc_text`` / ``write_recsrc``: recsrcx.txt, recsrcy.txt, recsrcz.txt
  of the FP64 GPU program (elatic_3d_unified_cuda_memory.cu:1202-1223): the
  NSTEP+1 source-point values of one component, each followed by a space,
  no newline; index 0 is the never-written 0.
- ``read_model`` / ``write_model``: modelcp.bin, modelcs.bin, modelrh.bin,
  raw float32 (float64 in elatic_3d_unified_cuda_memory.cu), x fastest, read
  in (k, j, i) order (seismicCPML_3d_isotropic_cudazerocopy.cu:544-595).
"""
from __future__ import annotations

import os

import numpy as np


def gather_layout(nx: int, ny: int, npml: int, ngatx: int, ngaty: int, src_k: int):
    """Returns (cells, slots): `cells` the distinct live receiver cells
    (i, j, k) 0-based, `slots` for every printed value in order the index
    into `cells` or -1 for a never-written (zero) entry."""
    xlen = nx // ngatx
    ylen = (ny - 2 * npml) // ngaty
    if xlen <= 0 or ylen <= 0:
        raise ValueError("more receivers than grid cells (the reference program stops here, :631-634)")
    k = src_k + 1  # plane KSOURCE+1 (1-based) = src_k + 1 (0-based)
    cells, index, slots = [], {}, []
    for j in range(0, ny + 1, ylen):
        for i in range(0, nx + 1, xlen):
            kk = i + j * nx
            i1 = (kk - 1) % nx + 1 if kk >= 1 else 0
            j1 = (kk - 1) // nx if kk >= 1 else 0
            if kk >= 1 and 1 <= j1 <= ny:
                c = (i1 - 1, j1 - 1, k)
                if c not in index:
                    index[c] = len(cells)
                    cells.append(c)
                slots.append(index[c])
            else:
                slots.append(-1)
    return np.array(cells, np.int32).reshape(-1, 3), np.array(slots, np.int64)


def _fmt(v: float) -> str:
    return "%g" % float(v)


def rechor_text(seis_comp: np.ndarray, slots: np.ndarray) -> str:
    """seis_comp [ncells, nsamp] of one component -> the file content."""
    lines = []
    for s in range(seis_comp.shape[1]):
        vals = [(_fmt(seis_comp[q, s]) if q >= 0 else "0") for q in slots]
        lines.append(" ".join(vals) + " \n")
    return "".join(lines)


def write_rechor(outdir: str, seis: np.ndarray, slots: np.ndarray, append: bool = False) -> list[str]:
    """Writes rechorvx.txt, rechorvy.txt, rechorvz.txt from seismograms
    [ncells, 3, nsamp] of the gather_layout cells."""
    paths = []
    for c, name in enumerate(("rechorvx.txt", "rechorvy.txt", "rechorvz.txt")):
        path = os.path.join(outdir, name)
        with open(path, "a" if append else "w") as f:
            f.write(rechor_text(seis[:, c, :], slots))
        paths.append(path)
    return paths


def recsrc_text(trace_comp: np.ndarray) -> str:
    """One component of the source trace [nstep + 1] -> the file content."""
    return "".join(_fmt(v) + " " for v in np.asarray(trace_comp).reshape(-1))


def write_recsrc(outdir: str, trace: np.ndarray) -> list[str]:
    """trace [3, nstep + 1] -> recsrcx.txt, recsrcy.txt, recsrcz.txt."""
    paths = []
    for c, name in enumerate(("recsrcx.txt", "recsrcy.txt", "recsrcz.txt")):
        path = os.path.join(outdir, name)
        with open(path, "w") as f:
            f.write(recsrc_text(trace[c]))
        paths.append(path)
    return paths


def snapshot_index(nx: int, ny: int, nz: int) -> np.ndarray:
    """For every value of a snapshot file, the compact cell index
    k*ny*nx + j*nx + i, or -1 where the program prints never-written zeros."""
    ii = np.arange(nx + 1, dtype=np.int64)
    jj = np.arange(ny + 1, dtype=np.int64)
    kk = np.arange(nz + 1, dtype=np.int64)
    addr = (ii[None, None, :] + jj[None, :, None] * nx + kk[:, None, None] * nx * ny).reshape(-1)
    out = np.full(addr.shape, -1, np.int64)
    ok = addr >= 1
    a = addr[ok] - 1
    i1 = a % nx + 1
    q = a // nx
    j1 = q % ny
    k1 = q // ny
    wrap = j1 == 0        # row 0 of plane k is row NIMY of plane k-1
    j1 = np.where(wrap, ny, j1)
    k1 = np.where(wrap, k1 - 1, k1)
    live = (k1 >= 1) & (k1 <= nz)
    idx = np.where(live, (k1 - 1) * ny * nx + (j1 - 1) * nx + (i1 - 1), -1)
    out[ok] = idx
    return out


def snapshot_bytes(field: np.ndarray, dtype=np.float32) -> bytes:
    """field [nz, ny, nx] -> the bytes of the program's v?%05i.bin file."""
    nz, ny, nx = field.shape
    idx = snapshot_index(nx, ny, nz)
    flat = np.ascontiguousarray(field, dtype=dtype).reshape(-1)
    vals = np.where(idx >= 0, flat[np.maximum(idx, 0)], 0).astype(dtype)
    return vals.tobytes()


def write_snapshots(outdir: str, it: int, vx: np.ndarray, vy: np.ndarray, vz: np.ndarray, dtype=np.float32):
    for name, f in (("vz", vz), ("vy", vy), ("vx", vx)):
        with open(os.path.join(outdir, "%s%05i.bin" % (name, it)), "wb") as fh:
            fh.write(snapshot_bytes(f, dtype))


def read_model(prefix: str, nx: int, ny: int, nz: int, dtype=np.float32):
    """(cp, cs, rho) [nz, ny, nx] from <prefix>cp.bin, cs.bin, rh.bin."""
    out = []
    for name in ("cp", "cs", "rh"):
        a = np.fromfile(f"{prefix}{name}.bin", dtype=dtype, count=nx * ny * nz)
        if a.size != nx * ny * nz:
            raise ValueError(f"short model file {prefix}{name}.bin")
        out.append(a.reshape(nz, ny, nx).astype(np.float32))
    return tuple(out)


def write_model(prefix: str, cp, cs, rho, dtype=np.float32) -> None:
    for name, a in (("cp", cp), ("cs", cs), ("rh", rho)):
        np.ascontiguousarray(a, dtype=dtype).tofile(f"{prefix}{name}.bin")
