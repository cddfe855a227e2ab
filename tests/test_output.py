"""Snapshot files (output.f90:7-352) on the CPU: the `.dat` rows of the
Particle type's formatted write read back to the written precision, the
Fortran ES edit forms, and the BINARY legacy VTK carrying the same arrays as
the ASCII one."""
import numpy as np
import pytest

from mysph_gb300 import output as O


def _fields(n=6, dim=2, seed=3):
    rng = np.random.default_rng(seed)
    d2 = dim * dim
    return {"X": rng.normal(size=(n, dim)), "V": rng.normal(size=(n, dim)), "MASS": rng.uniform(1, 2, n),
            "RHO": rng.uniform(990, 1010, n), "P": rng.normal(size=n) * 1e4, "E": rng.uniform(0, 1, n),
            "C": np.full(n, 62.6), "H": np.full(n, 0.024), "VISC": np.full(n, 1e-3),
            "TYPE": np.array([2, 2, 102, 102, -2, 0][:n], dtype=float), "DIVX": rng.normal(size=n),
            "DISP": rng.normal(size=(n, dim)) * 1e-3, "STRESS": rng.normal(size=(n, d2)) * 1e5,
            "DVDT": rng.normal(size=(n, dim))}


def test_es_edit_forms():
    assert O.es(1234.5678) == "1.2345678E+3"
    assert O.es(-0.000123) == "-1.2300000E-4"
    assert O.es(0.0) == "0.0000000E+0"
    assert O.es(1.0, 16, 3) == "1.0000000000000000E+000"
    assert O.es(0.25, 16, 3) == "2.5000000000000000E-001"


@pytest.mark.parametrize("dim", [2, 3])
def test_dat_rows_read_back(tmp_path, dim):
    f = _fields(dim=dim)
    state = np.array([0, 1, 0, 0, 0, 0])
    groups = O.type_groups(f["TYPE"])
    for typ, idx in groups.items():
        p = tmp_path / f"Type_{typ}_0.dat"
        O.write_dat(p, f, idx, dim, state)
        lines = p.read_text().splitlines()
        head = lines[0]
        assert head[:24] == "   Index    Type   State"
        ncol = 3 + 2 * dim + 8 + dim + dim * dim + (1 if typ > 100 else 0)
        assert len(head) == 24 + 17 * (ncol - 3)
        a = np.loadtxt(p, skiprows=1, ndmin=2)
        assert a.shape == (len(idx), ncol)
        assert np.array_equal(a[:, 0], idx + 1)                 # 1-based index in the whole set
        assert np.array_equal(a[:, 1], f["TYPE"][idx])
        assert np.array_equal(a[:, 2], state[idx])
        want = np.concatenate([f["X"][idx], f["V"][idx], f["MASS"][idx, None], f["RHO"][idx, None],
                               f["P"][idx, None], f["E"][idx, None], f["C"][idx, None], f["H"][idx, None],
                               f["VISC"][idx, None], f["DIVX"][idx, None], f["DISP"][idx],
                               # ((Stress(i, j), j = 1, dim), i = 1, dim)
                               f["STRESS"][idx].reshape(-1, dim, dim).transpose(0, 2, 1).reshape(-1, dim * dim)],
                              1)
        np.testing.assert_allclose(a[:, 3:3 + want.shape[1]], want, rtol=6e-8, atol=0)
        if typ > 100:
            np.testing.assert_allclose(a[:, -1], O.von_mises(f["STRESS"][idx], dim), rtol=1e-15)
            assert lines[1].endswith(O.es(O.von_mises(f["STRESS"][idx[:1]], dim)[0], 16, 3).rjust(24))


def _read_binary_vtk(data: bytes, sections):
    """Split a BINARY legacy VTK into its arrays using the known sections."""
    pos = data.index(b"DATASET UNSTRUCTURED_GRID\n") + len(b"DATASET UNSTRUCTURED_GRID\n")
    out = []
    for line, vals, kind in sections:
        hdr = (line + "\n").encode()
        assert data[pos:pos + len(hdr)] == hdr
        pos += len(hdr)
        if vals is None:
            continue
        cnt = np.asarray(vals).size
        dt = ">i4" if kind == "int" else ">f4"
        out.append(np.frombuffer(data, dt, cnt, pos).reshape(np.asarray(vals).shape))
        pos += 4 * cnt + 1
    assert pos == len(data)
    return out


def test_binary_vtk_matches_ascii(tmp_path):
    f = _fields(n=6, dim=3)
    idx = np.array([2, 3])     # the solids: von Mises included
    O.write_vtk(tmp_path / "a.vtk", f, idx, 3)
    O.write_vtk(tmp_path / "b.vtk", f, idx, 3, binary=True)
    secs = O._vtk_sections(f, idx, 3)
    arrays = _read_binary_vtk((tmp_path / "b.vtk").read_bytes(), secs)
    txt = (tmp_path / "a.vtk").read_text()
    assert "ASCII" in txt.splitlines()[2]
    k = 0
    for line, vals, kind in secs:
        if vals is None:
            continue
        want = np.asarray(vals).astype(np.float32) if kind == "float" else np.asarray(vals).astype(np.int32)
        assert np.array_equal(arrays[k], want), line
        k += 1


def test_snapshot_writer_writes_dat_and_vtk(tmp_path):
    class Fake:
        def __init__(self, f):
            self.f = f

        def field(self, k):
            return self.f[k]

    f = _fields()
    w = O.SnapshotWriter(tmp_path / "vtk", 2, dat_dir=tmp_path / "dat", binary=True)
    w.snapshot(Fake(f), 7)
    files = sorted(p.relative_to(tmp_path).as_posix() for p in w.close())
    assert files == sorted([f"{d}/Type_{t}_7.{d}" for t in (-2, 2, 5, 102) for d in ("dat", "vtk")])
