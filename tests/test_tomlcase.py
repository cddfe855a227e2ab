"""sph.toml front-end (getValueFromToml.f90:80-185): keys, defaults, the
switch-to-flag mapping and the rejection of options the GPU path lacks."""
from pathlib import Path

import pytest

from mysph_gb300 import cases
from mysph_gb300 import params as P
from mysph_gb300 import tomlcase as T

GOLD = Path(__file__).parent / "golden" / "toml"


def test_defaults_of_the_reference():
    cfg = T.parse("name = 'x'\n[Parameter]\nDIM = 3\n")
    assert cfg.dim == 3 and cfg.maxn == 5000 and cfg.kpair == 20
    assert cfg.pa_sph == 2 and cfg.nnps == 1 and cfg.skf == 1 and cfg.sle == 0
    assert cfg.print_interval == 100 and cfg.save_interval == 500 and cfg.max_time_step == 1000
    assert cfg.delta_t == P.f32(5e-4)        # dble(5e-4) is a single-precision literal
    assert cfg.sum_density and cfg.print_statistics and not cfg.gravity
    assert cfg.nick == "unknown"


def test_dam_break_file():
    cfg = T.parse(GOLD / "dam_break.toml")
    assert cfg.nick == "dam_break" and cfg.dim == 2 and cfg.delta_t == 1e-3
    assert cfg.ex_force  # forced on by dummyParticle / gravity
    assert cfg.nthreads == 4 and cfg.write_dp_vtk is False
    f = T.flags(cfg)
    assert f == (P.F_VISCOSITY | P.F_GRAVITY | P.F_EXT_FORCE | P.F_ARTI_VISC | P.F_DUMMY)
    case = T.build_case(cfg)
    ref = cases.reference_dam_break(dt=1e-3)
    assert case.n_real == ref.n_real and case.n_wall == ref.n_wall
    assert case.params.flags == f and case.params.dt == 1e-3
    assert (case.x == ref.x).all()


def test_unsupported_options_are_rejected():
    cfg = T.parse(GOLD / "shifting.toml")
    assert T.unsupported(cfg) == ["shifting"]
    with pytest.raises(T.UnsupportedOption):
        T.build_case(cfg)
    with pytest.warns(UserWarning):
        case = T.build_case(cfg, allow_unsupported=True)
    assert case.params.flags & P.F_SUM_DENSITY     # summationDensity defaults to true


def test_kernel_correction_maps_to_flag():
    cfg = T.parse(GOLD / "can_beam_kgc.toml")
    assert T.unsupported(cfg) == []
    case = T.build_case(cfg)
    assert case.params.flags & P.F_KERNEL_CORRECTION and case.params.dt == 2e-6
    assert (case.type[: case.n_real] > 100).all()


def test_bad_inputs():
    with pytest.raises(ValueError):
        T.parse("[Parameter]\nSPH = 2\n")                 # DIM missing
    with pytest.raises(ValueError):
        T.parse("[Parameter]\nDIM = 2\ngravity = 1\n")     # not a boolean
    with pytest.raises(ValueError):
        T.build_case(T.parse("nick = 'nope'\n[Parameter]\nDIM = 2\n"))
    cfg = T.parse("nick = 'dam_break'\n[Parameter]\nDIM = 2\nSLE = 3\n")
    assert T.unsupported(cfg) == ["SLE = 3"]


@pytest.mark.gpu
def test_toml_run_equals_direct_solver(gpu):
    from mysph_gb300.solver import GpuSolver
    import numpy as np
    lines = []
    r = T.run(GOLD / "dam_break.toml", out=lines.append)
    assert len(lines) == 3 and r["steps"] == 30
    case = T.build_case(T.parse(GOLD / "dam_break.toml"))
    with GpuSolver(case) as s:
        s.advance(30)
        for k in ("X", "V", "RHO"):
            assert np.array_equal(r["fields"][k], s.field(k)[: case.n_real]), k


def test_vtk_writer_layout(tmp_path):
    import numpy as np
    from mysph_gb300 import output as O
    n, dim = 5, 2
    f = {"X": np.arange(n * dim, dtype=float).reshape(n, dim), "V": np.ones((n, dim)),
         "MASS": np.full(n, 2.0), "RHO": np.full(n, 1000.0), "P": np.zeros(n), "E": np.zeros(n),
         "H": np.full(n, 0.1), "TYPE": np.array([2, 2, 0, -2, 102], dtype=float), "DIVX": np.zeros(n),
         "DISP": np.zeros((n, dim)), "STRESS": np.tile([1.0, 0.0, 0.0, -1.0], (n, 1)),
         "DVDT": np.zeros((n, dim))}
    groups = O.type_groups(f["TYPE"])
    assert list(groups) == [-2, 2, 5, 102]        # Type 0 filed under 5 (no Type 4)
    O.write_vtk(tmp_path / "t.vtk", f, groups[102], dim)
    txt = (tmp_path / "t.vtk").read_text().splitlines()
    assert txt[3] == "DATASET UNSTRUCTURED_GRID" and txt[4] == "POINTS 1 float"
    assert "SCALARS vonMises float 1" in txt and "TENSORS Stress float" in txt
    vm = O.von_mises(np.array([1.0, 0.0, 0.0, -1.0]), 2)
    assert vm[0] == pytest.approx(np.sqrt(3.0))


@pytest.mark.gpu
def test_toml_run_writes_snapshots(gpu, tmp_path):
    r = T.run(GOLD / "dam_break.toml", steps=20, out=None, out_dir=tmp_path)
    names = sorted(p.name for p in r["files"])
    # saveInterval 50 > 20 steps: the step-0 snapshot of the fluid (Type 2) only
    assert names == ["Type_2_0.vtk"]


def test_scheme_options():
    """SPH = 1 / 3 run on the GPU path; SPH = 4 has no internal-force form in
    the reference and is rejected."""
    for sph, bad in ((1, []), (3, []), (4, ["SPH = 4"])):
        cfg = T.parse(f"nick = 'dam_break'\n[Parameter]\nDIM = 2\nSPH = {sph}\n")
        assert T.unsupported(cfg) == bad
    case = T.build_case(T.parse("nick = 'dam_break'\n[Parameter]\nDIM = 2\nSPH = 3\n"))
    assert case.params.pa_sph == 3


def test_can_beam_3d_file():
    cfg = T.parse(GOLD / "can_beam_3d_kgc.toml")
    assert cfg.nick == "can_beam_3d" and cfg.dim == 3 and cfg.kernel_correction
    case = T.build_case(cfg)
    assert (case.n_real, case.n_wall, case.dim) == (9045, 0, 3)
    assert case.params.flags & P.F_KERNEL_CORRECTION
    assert int(case.boundary.sum()) == 5 * 9          # the clamped first layer
    assert case.params.dt == 2e-6                     # a TOML float, read as a double


@pytest.mark.gpu
def test_can_beam_3d_run_matches_oracle(gpu):
    """The 3-D cantilever project with kernel correction, run from its
    sph.toml on the GPU, against the oracle over the same steps."""
    import numpy as np
    from oracle.oracle import Oracle
    from tests.conftest import rel_l2
    from tests.helpers import bggs_band_covers
    r = T.run(GOLD / "can_beam_3d_kgc.toml", out=None)
    case = T.build_case(T.parse(GOLD / "can_beam_3d_kgc.toml"))
    # the reference's grid band falls short of 2h on this thin beam: the oracle
    # takes the exact r < 2h sets the GPU implements
    assert not bggs_band_covers(case)
    o = Oracle(case, covering_band=True)
    o.advance(r["steps"])
    for k in ("X", "V", "RHO", "P"):
        assert rel_l2(r["fields"][k], o.field(k)[: case.n_real]) <= 1e-8, k


def test_water_impact_file():
    """The nick's generator reproduces the reference's particle count (its
    project file's maxN is exactly the real + dummy total)."""
    cfg = T.parse(GOLD / "water_impact.toml")
    case = T.build_case(cfg)
    assert case.n_real + case.n_wall == cfg.maxn == 20582
    solid = case.type[: case.n_real] == 103
    assert solid.sum() == 240 and int(case.boundary[: case.n_real].sum()) == 6
    assert case.params.flags & P.F_GRAVITY_SKIP_SOLIDS


@pytest.mark.gpu
def test_water_impact_run_matches_oracle(gpu):
    from oracle.oracle import Oracle
    from tests.conftest import rel_l2
    from tests.helpers import bggs_band_covers
    r = T.run(GOLD / "water_impact.toml", out=None)
    case = T.build_case(T.parse(GOLD / "water_impact.toml"))
    assert bggs_band_covers(case)
    o = Oracle(case)
    o.advance(r["steps"])
    for k in ("X", "V", "RHO", "P"):
        assert rel_l2(r["fields"][k], o.field(k)[: case.n_real]) <= 1e-8, k


@pytest.mark.parametrize("maker,total", [
    (cases.reference_can_beam, 505),       # data/cantileverBeam/sph.toml: maxN = 505
    (cases.reference_can_beam_3d, 9045),   # data/cantileverBeam3D/sph.toml: maxN = 9045
    (cases.reference_water_impact, 20582), # data/waterImpact/sph.toml: maxN = 20582
])
def test_reference_generators_match_project_sizes(maker, total):
    """Known answers from the reference's own project files: where a project
    sizes maxN to exactly its particles (real + dummy), the generator of its
    nick produces that many."""
    c = maker()
    assert c.n_real + c.n_wall == total


def test_artificial_heat_maps_to_its_flag():
    """artificialHeat is implemented (FP64): it maps to SPH_F_ARTI_HEAT and is
    no longer an unsupported option."""
    cfg = T.parse("nick = 'dam_break'\n[Parameter]\nDIM = 2\nartificialHeat = true\n")
    assert cfg.arti_heat and T.unsupported(cfg) == []
    assert T.flags(cfg) & P.F_ARTI_HEAT
