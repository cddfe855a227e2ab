"""Snapshot output in the reference's layout (src/Output/output.f90:7-352).

`output()` of the reference writes, per particle Type, one legacy ASCII VTK
file `Type_<type>_<index>.vtk` with the points (cast to FP32), the scalars
Mass, Density, Pressure, InternalEnergy, Type, State, Boundary,
SmoothingLength and DivDistance, the vectors U and Displacement, the Stress
tensor, von Mises for solids and, when rates are given, the Acceleration.
Particles of Type 0 are filed with Type 4 when that exists, else with
Type 5 (output.f90:38-52).  `SnapshotWriter` gathers the fields from the
device on the caller's thread and formats and writes the files on a worker
thread, so the next steps can run meanwhile.
"""
from __future__ import annotations

import concurrent.futures as cf
from pathlib import Path

import numpy as np

FIELDS = ("X", "V", "MASS", "RHO", "P", "E", "H", "TYPE", "DIVX", "DISP", "STRESS", "DVDT")


def von_mises(stress: np.ndarray, dim: int) -> np.ndarray:
    """von Mises stress of column-major Dim x Dim tensors (output.f90:354-377)."""
    s = stress.reshape(-1, dim, dim)  # s[:, col, row]
    if dim == 1:
        return np.abs(s[:, 0, 0])
    if dim == 2:
        s11, s22, s12 = s[:, 0, 0], s[:, 1, 1], s[:, 1, 0]
        return np.sqrt((s11 + s22) ** 2 - 3 * (s11 * s22) + 3 * s12 ** 2)
    s11, s22, s33 = s[:, 0, 0], s[:, 1, 1], s[:, 2, 2]
    s12, s13, s23 = s[:, 1, 0], s[:, 2, 0], s[:, 2, 1]
    return np.sqrt((s11 + s22 + s33) ** 2 - 3 * (s22 * s33 + s33 * s11 + s11 * s22)
                   + 3 * (s12 ** 2 + s13 ** 2 + s23 ** 2))


def type_groups(types: np.ndarray) -> dict[int, np.ndarray]:
    """Indices per Type, with Type 0 filed under 4 (or 5) as the reference does."""
    t = np.asarray(types).astype(np.int64)
    groups = {int(v): np.flatnonzero(t == v) for v in np.unique(t)}
    if 0 in groups:
        zero = groups.pop(0)
        key = 4 if 4 in groups else 5
        groups[key] = np.concatenate([groups.get(key, np.zeros(0, np.int64)), zero])
    return dict(sorted(groups.items()))


def _rows(a: np.ndarray) -> str:
    a = np.asarray(a, dtype=np.float32).astype(np.float64)
    if a.ndim == 1:
        a = a[:, None]
    return "\n".join("   ".join(f"{v: .16E}" for v in row) for row in a) + "\n"


def _pad(a: np.ndarray, width: int) -> np.ndarray:
    a = np.asarray(a, dtype=np.float64)
    a = a.reshape(len(a), -1)
    if a.shape[1] < width:
        a = np.concatenate([a, np.zeros((len(a), width - a.shape[1]))], 1)
    return a


def write_vtk(path: Path, f: dict, idx: np.ndarray, dim: int, state=None, boundary=None) -> None:
    n = len(idx)
    t = f["TYPE"][idx]
    lines = ["# vtk DataFile Version 3.0", "paraview_vtk_output", "ASCII", "DATASET UNSTRUCTURED_GRID",
             f"POINTS {n} float"]
    out = "\n".join(lines) + "\n" + _rows(_pad(f["X"][idx], 3)) + f"POINT_DATA {n}\n"

    def scalar(name, vals, kind="float"):
        nonlocal out
        out += f"SCALARS {name} {kind} 1\nLOOKUP_TABLE DEFAULT\n"
        if kind == "int":
            out += "\n".join(str(int(v)) for v in vals) + "\n"
        else:
            out += _rows(vals)

    scalar("Mass", f["MASS"][idx])
    scalar("Density", f["RHO"][idx])
    scalar("Pressure", f["P"][idx])
    scalar("InternalEnergy", f["E"][idx])
    scalar("Type", t, "int")
    scalar("State", np.zeros(n) if state is None else np.asarray(state)[idx], "int")
    scalar("Boundary", np.zeros(n) if boundary is None else np.asarray(boundary)[idx], "int")
    scalar("SmoothingLength", f["H"][idx])
    scalar("DivDistance", f["DIVX"][idx])
    out += "VECTORS U float\n" + _rows(_pad(f["V"][idx], 3))
    out += "VECTORS Displacement float\n" + _rows(_pad(f["DISP"][idx], 3))
    out += "TENSORS Stress float\n" + _rows(_pad(f["STRESS"][idx], 9))
    if n and t[0] > 100:
        scalar("vonMises", von_mises(f["STRESS"][idx], dim))
    if "DVDT" in f:
        out += "VECTORS Acceleration float\n" + _rows(_pad(f["DVDT"][idx], 3))
    path.write_text(out)


class SnapshotWriter:
    """Writes `Type_<type>_<index>.vtk` files of a solver's state on a worker
    thread.  `snapshot()` gathers on the caller's thread (the device state
    must not change while it is read) and returns at once."""

    def __init__(self, out_dir: str | Path, dim: int, state=None, boundary=None, with_walls: bool = True):
        self.dir = Path(out_dir)
        self.dir.mkdir(parents=True, exist_ok=True)
        self.dim = dim
        self.state, self.boundary = state, boundary
        self.with_walls = with_walls
        self.pool = cf.ThreadPoolExecutor(max_workers=1)
        self.pending: list[cf.Future] = []

    def snapshot(self, solver, index: int, n_real: int | None = None) -> None:
        f = {k: solver.field(k) for k in FIELDS}
        n = len(f["TYPE"]) if self.with_walls or n_real is None else n_real
        self.pending.append(self.pool.submit(self._write, f, index, n))

    def _write(self, f: dict, index: int, n: int) -> list[Path]:
        out = []
        for typ, idx in type_groups(f["TYPE"][:n]).items():
            p = self.dir / f"Type_{typ}_{index}.vtk"
            write_vtk(p, f, idx, self.dim, self.state, self.boundary)
            out.append(p)
        return out

    def close(self) -> list[Path]:
        files = [p for fut in self.pending for p in fut.result()]
        self.pool.shutdown()
        return files
