"""Algorithmic bytes and rates of the time loop.

One cell-update is one full time step (stress + velocity half-steps) of one
cell; every step counts all nx*ny*nz cells, PML included.  Algorithmic
bytes per cell-update (W = size of the real type):
  stress half-step: read v x3, sigma x6, model x3, write sigma x6 = 18 W;
  velocity half-step: read sigma x6, v x3, rho, write v x3        = 13 W;
  each PML direction a cell lies in adds 3 memory variables read and
  written per half-step = 6 W per half-step (12 W per step).
The fraction of cells in the PML of axis d is 2 npml / n_d, so the averages
are 124 + 48 sum_d 2 npml / n_d bytes in FP32: 152.5 B for the 101^3 cube
with 10 PML cells, 142 B for 256^3 with 16.
"""
from __future__ import annotations


def pml_directions(nx: int, ny: int, nz: int, npml: int) -> float:
    return sum(min(1.0, 2.0 * npml / n) for n in (nx, ny, nz))


def bytes_per_cell(nx: int, ny: int, nz: int, npml: int, word: int = 4) -> dict:
    d = pml_directions(nx, ny, nz, npml)
    stress = word * (18 + 6 * d)
    velocity = word * (13 + 6 * d)
    return {"stress": stress, "velocity": velocity, "step": stress + velocity}


def gcells_per_s(cells: int, steps: int, seconds: float) -> float:
    return cells * steps / seconds / 1e9
