"""Shared helpers of the test suite (case perturbation, neighbour sets)."""
from __future__ import annotations

import numpy as np

from mysph_gb300.cases import Case


def perturb(case: Case, seed: int = 1, v_amp: float = 0.0, x_frac: float = 0.0) -> Case:
    """Random velocity noise (m/s) and position jitter (fraction of dx) on the
    real particles, so that every pair branch (AV, strain, guard band) runs."""
    rng = np.random.default_rng(seed)
    c = Case(**{k: getattr(case, k) for k in case.__dataclass_fields__})
    c.x = case.x.copy()
    c.v = case.v.copy()
    dx = case.meta.get("dx", 1.0)
    nr = case.n_real
    if x_frac:
        c.x[:nr] += rng.uniform(-x_frac, x_frac, size=(nr, case.dim)) * dx
    if v_amp:
        c.v[:nr] += rng.normal(0.0, v_amp, size=(nr, case.dim))
        c.v[case.boundary == 1] = case.v[case.boundary == 1]
    return c


def csr_sets(off, lst):
    return [frozenset(lst[off[i]:off[i + 1]].tolist()) for i in range(len(off) - 1)]


def brute_force_sets(case: Case, scale_k: int = 2):
    """O(N^2) FP64 enumeration: j != i, State_j != -1, sqrt(sum dx^2) < scale_k h_i,
    dx and the sum formed as the reference forms them (asymmetricSearch.f90:227-237).
    Returns 1-based index sets and the pairs within 4 ulp of the cut-off."""
    x = case.x
    n, nr = case.n, case.n_real
    ok_src = case.state != -1
    sets, ties = [], []
    for i in range(nr):
        if case.state[i] == -1:
            sets.append(frozenset())
            continue
        d = x[i][None, :] - x
        dr = d[:, 0] * d[:, 0]
        for a in range(1, case.dim):
            dr = dr + d[:, a] * d[:, a]
        r = np.sqrt(dr)
        cut = case.h[i] * scale_k
        m = (r < cut) & ok_src
        m[i] = False
        sets.append(frozenset((np.flatnonzero(m) + 1).tolist()))
        near = np.flatnonzero(np.abs(r - cut) <= 4 * np.spacing(cut))
        ties.extend((i, int(j)) for j in near if j != i)
    return sets, ties


def bggs_band_covers(case: Case, scale_k: int = 2) -> bool:
    """Whether the reference's background grid search scans at least
    scale_k*h around every target.  BGGS scans int(h/cell)+1 cells per axis
    (asymmetricSearch.f90:209-217), which covers h but not 2h when the cell
    is in [h, 2h); its grid is the particles' bounding box grown by GMR-1 =
    0.2 (single-precision 1.2) per side with about 3 particles per cell
    (asymmetricSearch.f90:61-131)."""
    gmr = float(np.float32(1.2))
    x = case.x
    n, dim = case.n, case.dim
    mx, mn = x.max(0), x.min(0)
    delta = mx - mn
    hi = mx + (gmr - 1) * delta
    lo = mn - (gmr - 1) * delta
    if dim == 2:
        c1 = min(int(((n * delta[0]) / (delta[1] * 3)) ** 0.5) + 1, 1000)
        cn = [c1, min(int(c1 * delta[1] / delta[0]) + 1, 1000)]
    else:
        c1 = min(int(((n * delta[0] * delta[0]) / (delta[1] * delta[2] * 3)) ** (1 / 3)) + 1, 1000)
        cn = [c1, min(int(c1 * delta[1] / delta[0]) + 1, 1000), min(int(c1 * delta[2] / delta[0]) + 1, 1000)]
    ext = hi - lo
    for hh in np.unique(case.h[: case.n_real]):
        for a in range(dim):
            band = int(hh / ext[a] * cn[a]) + 1
            if band * ext[a] / cn[a] < scale_k * hh:
                return False
    return True


def fsi_block_3d(seed: int = 57) -> Case:
    """The 3-D dam break at dx = 3 cm with the half of the water column
    nearest x = 0 turned into a linear-elastic solid (Type 102): fluid-solid
    pairs in 3-D, and solid stress rows read by fluid and solid targets."""
    from mysph_gb300 import cases
    from mysph_gb300 import params as P
    c = perturb(cases.dam_break_3d(dx=0.03), seed=seed, v_amp=0.2, x_frac=0.1)
    nr = c.n_real
    solid = c.x[:nr, 0] < np.median(c.x[:nr, 0])
    c.type = c.type.copy()
    c.type[:nr][solid] = 102
    c.shear = np.zeros((c.n, 9))
    c.params = c.params.copy()
    c.params.add_material(**P.linear_solid(102, 1000.0, P.f32(2e7), P.f32(4.27e6)))
    cs = (P.f32(2e7) / 1000.0) ** 0.5          # solid sound speed, and a time step for it
    c.c = c.c.copy()
    c.c[:nr][solid] = cs
    c.params.dt = 0.2 * float(c.h[0]) / cs
    return c



def plastic_block(dim: int = 2, type_id: int = 101, seed: int = 61, n: int = 14,
                  dx: float = 1e-3) -> Case:
    """A perturbed block of an elastic-plastic solid with no walls.

    Type 101 is the reference's Mie-Grueneisen armco iron (eos.f90:180-215,
    yield stress 6e8); type 104 its linear-EOS aluminium (eos.f90:228-236,
    yield stress 3e8).  The density straddles rho0, so both branches of the
    Hugoniot curve run; the internal energy is non-zero, so the Grueneisen
    term counts; the initial deviatoric stress exceeds the yield surface for
    most particles, so the radial return (timeIntegration.f90:145-167) caps it
    in the first step, while a fifth of the particles start below it.  One
    edge is clamped (Boundary = 1).  Viscosity (the strain and rotation
    rates), the solid artificial viscosity, gravity and, in 2-D, the
    artificial stress are on."""
    from mysph_gb300 import params as P
    rng = np.random.default_rng(seed)
    prm = P.base_params(dim, 1.0)
    prm.flags = P.F_VISCOSITY | P.F_ARTI_VISC | P.F_GRAVITY | P.F_EXT_FORCE
    if dim == 2:
        prm.flags |= P.F_ARTI_STRESS
        prm.as_dp = dx
    P.reference_materials(prm, 50.0)
    m = prm.material(type_id)
    rho0 = m.rho0
    if type_id == 101:
        cs = m.mg_cs * 1.3
    else:
        cs = (m.K / rho0) ** 0.5
    h = 1.2 * dx
    prm.dt = 0.2 * h / cs
    axes = [np.arange(n)] * dim
    g = (np.stack(np.meshgrid(*axes, indexing="ij"), -1).reshape(-1, dim) + 0.5) * dx
    g = g - g.mean(0)
    N = len(g)
    x = g + rng.uniform(-0.1, 0.1, size=(N, dim)) * dx
    v = rng.normal(0.0, 2.0, size=(N, dim))
    rho = rho0 * (1.0 + rng.normal(0.0, 1e-3, size=N))
    e = rng.uniform(0.0, 2e3, size=N)
    S = np.zeros((N, dim, dim))
    amp = 2.5 * m.sigma_y / np.sqrt(3.0)
    for a in range(dim):
        for b in range(a, dim):
            S[:, a, b] = rng.normal(0.0, amp / dim, size=N)
            S[:, b, a] = S[:, a, b]
    S -= np.trace(S, axis1=1, axis2=2)[:, None, None] / dim * np.eye(dim)[None]
    S[rng.random(N) < 0.2] *= 0.05
    shear = S.transpose(0, 2, 1).reshape(N, dim * dim)   # column-major per particle
    bnd = (g[:, 0] < g[:, 0].min() + 1.5 * dx).astype(np.int32)
    v[bnd == 1] = 0.0
    return Case(f"plastic{dim}d_{type_id}", prm, N, 0, x, v, np.full(N, rho0 * dx ** dim), rho,
                np.zeros(N), e, np.full(N, cs), np.full(N, h), np.full(N, type_id, np.int32),
                np.zeros(N, np.int32), bnd, shear, dict(dx=dx))


def two_fluid_dam_break(seed: int = 62) -> Case:
    """The 2-D dam break at dx = 4 cm with the upper half of the column a
    second fluid (Type 3, a lighter Tait fluid): the multiphase penalty of
    externalForce.f90:126-141 acts across the interface, with the
    reference's constants (factor 1e5, exponents 6 and 4).  The time step is
    cut to 1e-6 s so that the penalty's large accelerations move particles by
    far less than dx over a 20-step comparison."""
    from mysph_gb300 import cases
    from mysph_gb300 import params as P
    c = perturb(cases.dam_break_2d(dx=0.04), seed=seed, v_amp=0.2, x_frac=0.1)
    nr = c.n_real
    upper = c.x[:nr, 1] > np.median(c.x[:nr, 1])
    c.type = c.type.copy()
    c.type[:nr][upper] = 3
    c.rho, c.mass = c.rho.copy(), c.mass.copy()
    c.rho[:nr][upper] *= 0.9
    c.mass[:nr][upper] *= 0.9
    c.params = c.params.copy()
    c0 = c.params.material(2).c0
    c.params.add_material(**dict(P.water(c0, rho0=900.0), type=3))
    c.params.flags |= P.F_EXT_FORCE
    c.params.dt = 1e-6
    return c


def with_heat(case: Case, seed: int = 63, e_max: float = 50.0) -> Case:
    """The case with the artificial heat on (artificialHeat.f90:6-56) and a
    random internal energy in [0, e_max] on its real particles, so that the
    conduction term e_i - e_j is not zero."""
    from mysph_gb300 import params as P
    rng = np.random.default_rng(seed)
    c = Case(**{k: getattr(case, k) for k in case.__dataclass_fields__})
    c.e = case.e.copy()
    c.e[: case.n_real] = rng.uniform(0.0, e_max, case.n_real)
    c.params = case.params.copy()
    c.params.flags |= P.F_ARTI_HEAT
    return c
