"""Snapshot output in the reference's layout (src/Output/output.f90:7-352).

`output()` of the reference writes, per particle Type, one legacy ASCII VTK
file `Type_<type>_<index>.vtk` with the points (cast to FP32), the scalars
Mass, Density, Pressure, InternalEnergy, Type, State, Boundary,
SmoothingLength and DivDistance, the vectors U and Displacement, the Stress
tensor, von Mises for solids and, when rates are given, the Acceleration;
and one text file `Type_<type>_<index>.dat` with a row per particle (its
index in the whole set, then the fields of the Particle type's formatted
write, SPH.f90:55-90, and von Mises for solids).  Particles of Type 0 are
filed with Type 4 when that exists, else with Type 5 (output.f90:38-52).
The VTK files can also be written in the legacy BINARY form (big-endian
FP32 / int32), several times smaller and faster to write.  `SnapshotWriter`
gathers the fields from the device on the caller's thread and formats and
writes the files on a worker thread, so the next steps can run meanwhile.
"""
from __future__ import annotations

import concurrent.futures as cf
from pathlib import Path

import numpy as np

FIELDS = ("X", "V", "MASS", "RHO", "P", "E", "C", "H", "VISC", "TYPE", "DIVX", "DISP", "STRESS", "DVDT")


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


def _vtk_sections(f: dict, idx: np.ndarray, dim: int, state=None, boundary=None):
    """(header line, values, kind) of write_vtk's data sections in the
    reference's order (output.f90:233-352)."""
    n = len(idx)
    t = f["TYPE"][idx]
    out = [(f"POINTS {n} float", _pad(f["X"][idx], 3), "float")]
    sc = lambda name, v, kind="float": (f"SCALARS {name} {kind} 1\nLOOKUP_TABLE DEFAULT", v, kind)
    out.append((f"POINT_DATA {n}", None, None))
    out += [sc("Mass", f["MASS"][idx]), sc("Density", f["RHO"][idx]), sc("Pressure", f["P"][idx]),
            sc("InternalEnergy", f["E"][idx]), sc("Type", t, "int"),
            sc("State", np.zeros(n) if state is None else np.asarray(state)[idx], "int"),
            sc("Boundary", np.zeros(n) if boundary is None else np.asarray(boundary)[idx], "int"),
            sc("SmoothingLength", f["H"][idx]), sc("DivDistance", f["DIVX"][idx]),
            ("VECTORS U float", _pad(f["V"][idx], 3), "float"),
            ("VECTORS Displacement float", _pad(f["DISP"][idx], 3), "float"),
            ("TENSORS Stress float", _pad(f["STRESS"][idx], 9), "float")]
    if n and t[0] > 100:
        out.append(sc("vonMises", von_mises(f["STRESS"][idx], dim)))
    if "DVDT" in f:
        out.append(("VECTORS Acceleration float", _pad(f["DVDT"][idx], 3), "float"))
    return out


def write_vtk(path: Path, f: dict, idx: np.ndarray, dim: int, state=None, boundary=None,
              binary: bool = False) -> None:
    """One Type's legacy VTK file: ASCII as the reference writes it, or
    BINARY (big-endian FP32 and int32 arrays, the same sections)."""
    head = ["# vtk DataFile Version 3.0", "paraview_vtk_output", "BINARY" if binary else "ASCII",
            "DATASET UNSTRUCTURED_GRID"]
    if not binary:
        out = "\n".join(head) + "\n"
        for line, vals, kind in _vtk_sections(f, idx, dim, state, boundary):
            out += line + "\n"
            if vals is None:
                continue
            if kind == "int":
                out += "\n".join(str(int(v)) for v in vals) + "\n"
            else:
                out += _rows(vals)
        path.write_text(out)
        return
    parts = [("\n".join(head) + "\n").encode()]
    for line, vals, kind in _vtk_sections(f, idx, dim, state, boundary):
        parts.append((line + "\n").encode())
        if vals is None:
            continue
        dt = ">i4" if kind == "int" else ">f4"
        parts.append(np.ascontiguousarray(np.asarray(vals).astype(np.float64).astype(dt)).tobytes())
        parts.append(b"\n")
    path.write_bytes(b"".join(parts))


def es(v: float, d: int = 7, e: int = 0) -> str:
    """Fortran ES0.dEe without the field width: one digit before the point, d
    after, an exponent of e digits (e = 0: as many as needed)."""
    if not np.isfinite(v):
        return "NaN" if np.isnan(v) else ("Infinity" if v > 0 else "-Infinity")
    m, x = f"{v:.{d}E}".split("E")
    k = int(x)
    digits = str(abs(k)) if e == 0 else str(abs(k)).rjust(e, "0")
    return f"{m}E{'-' if k < 0 else '+'}{digits}"


def dat_header(dim: int, solid: bool) -> str:
    """The column line of write_file (output.f90:95-213), format (3(A8), *(A17))."""
    ax = "XYZ"[:dim]
    cols = ["Index", "Type", "State", *ax, *"UVW"[:dim], "Mass", "Density", "Pressure", "InternalEnergy",
            "SoundSpeed", "SmoothingLength", "Viscosity", "DivDistance",
            *[f"Displacement_{a}" for a in ax], *[f"Stress{a}{b}" for a in ax for b in ax]]
    if dim == 1:
        cols[3:5] = ["X", "V"]
    if solid:
        cols.append("vonMises")
    return "".join(c.rjust(8)[-8:] if k < 3 else c.rjust(17)[:17] for k, c in enumerate(cols))


def write_dat(path: Path, f: dict, idx: np.ndarray, dim: int, state=None) -> None:
    """One Type's text file as write_file writes it: per row the particle's
    1-based index in the whole set (I8), then Type and State (2(I8)), 2X, the
    scalars, vectors and stress of the Particle write (SPH.f90:84-90), each
    ES15.7E0 followed by 2X, and for solids von Mises as ES24.16E3."""
    n = len(idx)
    t = f["TYPE"][idx].astype(np.int64)
    solid = bool(n and t[0] > 100)
    st = np.zeros(n, np.int64) if state is None else np.asarray(state)[idx].astype(np.int64)
    vec = lambda k: np.asarray(f[k][idx], np.float64).reshape(n, -1)[:, :dim]
    cols = [vec("X"), vec("V"), vec("MASS"), vec("RHO"), vec("P"), vec("E"), vec("C"), vec("H"),
            vec("VISC"), vec("DIVX"), vec("DISP")]
    # ((Stress(i, j), j = 1, dim), i = 1, dim): column-major storage s[j*dim + i]
    S = np.asarray(f["STRESS"][idx], np.float64).reshape(n, dim, dim)   # S[:, j, i]
    cols.append(S.transpose(0, 2, 1).reshape(n, dim * dim))
    vals = np.concatenate(cols, 1)
    vm = von_mises(f["STRESS"][idx], dim) if solid else None
    lines = [dat_header(dim, solid)]
    for r in range(n):
        row = f"{int(idx[r]) + 1:8d}{int(t[r]):8d}{int(st[r]):8d}  "
        row += "  ".join(es(v).rjust(15) for v in vals[r])
        if solid:
            row += "  " + es(vm[r], 16, 3).rjust(24)
        lines.append(row)
    path.write_text("\n".join(lines) + "\n")


class SnapshotWriter:
    """Writes `Type_<type>_<index>.vtk` files of a solver's state (and the
    `.dat` files into `dat_dir` when given) on a worker thread.  `snapshot()`
    gathers on the caller's thread (the device state must not change while
    it is read) and returns at once."""

    def __init__(self, out_dir: str | Path, dim: int, state=None, boundary=None, with_walls: bool = True,
                 dat_dir: str | Path | None = None, binary: bool = False):
        self.dir = Path(out_dir)
        self.dir.mkdir(parents=True, exist_ok=True)
        self.dat_dir = Path(dat_dir) if dat_dir is not None else None
        if self.dat_dir is not None:
            self.dat_dir.mkdir(parents=True, exist_ok=True)
        self.dim = dim
        self.state, self.boundary = state, boundary
        self.with_walls = with_walls
        self.binary = binary
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
            write_vtk(p, f, idx, self.dim, self.state, self.boundary, self.binary)
            out.append(p)
            if self.dat_dir is not None:
                q = self.dat_dir / f"Type_{typ}_{index}.dat"
                write_dat(q, f, idx, self.dim, self.state)
                out.append(q)
        return out

    def close(self) -> list[Path]:
        files = [p for fut in self.pending for p in fut.result()]
        self.pool.shutdown()
        return files
