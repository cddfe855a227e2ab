"""CPU checks of the oracle (oracle/sph_oracle.cpp) before it is trusted.

The reference ships no golden vectors for this path and cannot be compiled
here, so the oracle is pinned by known answers derived from the reference's
formulas and by properties: kernel normalisation (the partition-of-unity
sums printed by the reference's test/kernelTest.f90), EOS round trips,
brute-force neighbour sets, hydrostatic rest, momentum conservation, the J2
radial return and the Jaumann rate of a rigidly spinning patch.
"""
import math

import numpy as np
import pytest

from mysph_gb300 import cases
from mysph_gb300 import params as P
from oracle import oracle as O
from tests.conftest import rel_l2
from tests.helpers import bggs_band_covers, brute_force_sets, csr_sets, perturb


# ---- kernels (src/Numeric/kernel.f90) -------------------------------------
@pytest.mark.parametrize("dim", [1, 2, 3])
def test_cubic_known_values(dim):
    h = 0.7
    factor = {1: 1.0 / h, 2: 15.0 / (7.0 * math.pi * h * h), 3: 3.0 / (2.0 * math.pi * h ** 3)}[dim]
    w, dw = O.kernel(1, dim, 0.0, np.zeros(dim), h)
    assert w == pytest.approx(factor * 2.0 / 3.0, rel=1e-15)
    assert np.all(dw == 0)
    dx = np.zeros(dim)
    dx[0] = h  # q = 1: both branches meet
    w1, dw1 = O.kernel(1, dim, h, dx, h)
    assert w1 == pytest.approx(factor / 6.0, rel=1e-14)
    assert dw1[0] == pytest.approx(-0.5 * factor / h, rel=1e-14)
    dx[0] = 2.0 * h
    w2, dw2 = O.kernel(1, dim, 2.0 * h, dx, h)
    assert w2 == 0.0 and dw2[0] == 0.0


@pytest.mark.parametrize("skf", [1, 2, 3])
def test_partition_of_unity_1d(skf):
    """test/kernelTest.f90: sum W dx -> 1 and sum (x_i - x_m) dW/dx dx -> 1."""
    k = 40
    delta = 1.0 / k
    h = delta * 1.2
    x = delta * np.arange(-200, 201)
    s0 = s1 = 0.0
    for xi in x:
        dx = np.array([0.0 - xi])
        w, dw = O.kernel(skf, 1, abs(dx[0]), dx, h)
        s0 += w * delta
        s1 += (xi - 0.0) * dw[0] * delta
    assert s0 == pytest.approx(1.0, abs=2e-3)
    if skf == 1:  # the reference's test uses the cubic spline
        assert s1 == pytest.approx(1.0, abs=3e-2)  # first moment: lattice error at h = 1.2 dx


@pytest.mark.parametrize("dim", [2, 3])
def test_lattice_normalisation(dim):
    dx = 0.01
    h = 1.2 * dx
    r = np.arange(-3, 4)
    pts = np.stack(np.meshgrid(*([r] * dim), indexing="ij"), -1).reshape(-1, dim) * dx
    s = 0.0
    grad = np.zeros(dim)
    for p in pts:
        d = -p
        w, dw = O.kernel(1, dim, float(np.linalg.norm(d)), d, h)
        s += w * dx ** dim
        grad += dw * dx ** dim
    assert s == pytest.approx(1.0, abs=2e-2)
    assert np.abs(grad).max() < 1e-12 / dx  # symmetric lattice: zero net gradient


# ---- EOS (src/Physic/eos.f90) -----------------------------------------------
def test_tait_round_trip():
    prm = P.base_params(2, 1e-4)
    prm.add_material(**P.water(50.0))
    m = prm.materials[0]
    p_in = np.array([0.0, 1e3, 2.4e5])
    rho = cases.tait_density(p_in, 50.0)
    for pi, ri in zip(p_in, rho):
        p, _ = O.eos(m, False, ri)
        assert p == pytest.approx(pi, rel=1e-11, abs=1e-9)
    assert O.eos(m, False, 1000.0)[0] == 0.0


def test_solid_eos():
    prm = P.base_params(2, 1e-4)
    P.reference_materials(prm, 50.0)
    m102 = prm.material(102)
    p, _ = O.eos(m102, True, 1111.0)
    assert p == (P.f32(2e7) / 1100.0) * (1111.0 - 1100.0)
    m101 = prm.material(101)
    p0, _ = O.eos(m101, True, 7850.0, e=10.0)
    assert p0 == pytest.approx(m101.gamma * 7850.0 * 10.0, rel=1e-15)
    mu = 0.01
    p1, _ = O.eos(m101, True, 7850.0 * (1 + mu), e=0.0)
    c1 = 7850.0 * 3630.0 ** 2
    s = m101.mg_s
    ph = c1 * mu + c1 * (1 + 2 * (s - 1)) * mu ** 2 + c1 * (2 * (s - 1) + 3 * (s - 1) ** 2) * mu ** 3
    assert p1 == pytest.approx((1 - 0.5 * m101.gamma * mu) * ph, rel=1e-13)


# ---- NNPS -------------------------------------------------------------------
@pytest.mark.parametrize("maker", [
    lambda: perturb(cases.dam_break_2d(dx=0.04), seed=3, x_frac=0.3),
    lambda: perturb(cases.dam_break_3d(dx=0.03), seed=4, x_frac=0.3),
])
def test_bggs_equals_brute_force(maker):
    c = maker()
    assert bggs_band_covers(c)
    o = O.Oracle(c)
    o.bggs()
    off, lst = o.neighbors()
    got = csr_sets(off, lst)
    want, ties = brute_force_sets(c)
    assert not ties
    assert got == want


def test_bggs_band_deficit():
    """Where the reference's grid cell lies in [h, 2h) its band of
    int(h/cell)+1 cells misses some pairs with r < 2h: the oracle keeps that
    behaviour, so its sets are then subsets of the exact ones."""
    c = perturb(cases.dam_break_3d(dx=0.06), seed=4, x_frac=0.3)
    assert not bggs_band_covers(c)
    o = O.Oracle(c)
    o.bggs()
    got = csr_sets(*o.neighbors())
    want, _ = brute_force_sets(c)
    assert all(g <= w for g, w in zip(got, want))
    assert any(g != w for g, w in zip(got, want))


def test_bggs_lattice_counts():
    c = cases.dam_break_3d(dx=0.03)
    o = O.Oracle(c)
    o.bggs()
    off, _ = o.neighbors()
    n = np.diff(off)
    # interior lattice points: 56 neighbours within 2.4 dx in 3-D
    assert n.max() == 56
    c2 = cases.dam_break_2d(dx=0.05)
    o2 = O.Oracle(c2)
    o2.bggs()
    assert np.diff(o2.neighbors()[0]).max() == 20


def test_state_minus_one_skipped():
    c = cases.dam_break_2d(dx=0.1)
    c.state[5] = -1
    o = O.Oracle(c)
    o.bggs()
    off, lst = o.neighbors()
    assert off[6] - off[5] == 0
    assert 6 not in set(lst.tolist())


# ---- physics properties ------------------------------------------------------
def test_hydrostatic_start():
    c = cases.dam_break_2d(dx=0.04)
    o = O.Oracle(c)
    o.rates()
    drho = o.field("DRHODT")[: c.n_real]
    assert np.all(drho == 0.0)  # v = 0 everywhere at t = 0
    a = o.field("DVDT")[: c.n_real]
    x = c.x[: c.n_real]
    interior = (x[:, 0] > 0.2) & (x[:, 0] < 0.6) & (x[:, 1] > 0.2) & (x[:, 1] < 1.6)
    # pressure gradient balances gravity in the interior of the column
    assert abs(a[interior, 1].mean()) < 0.05 * 9.81
    assert np.abs(a[interior, 0]).mean() < 0.05 * 9.81


def test_momentum_conservation_closed_box():
    """No walls, no gravity: internal + AV pair forces are antisymmetric."""
    c = cases.dam_break_2d(dx=0.05, width=1.0, height=1.0)
    c = perturb(c.subset_real(np.ones(c.n_real, bool)), seed=5, v_amp=0.5, x_frac=0.2)
    keep = np.arange(c.n_real)
    c2 = cases.Case(c.name, c.params.copy(), c.n_real, 0, c.x[keep], c.v[keep], c.mass[keep],
                    c.rho[keep], c.p[keep], c.e[keep], c.c[keep], c.h[keep], c.type[keep],
                    c.state[keep], c.boundary[keep], None, dict(c.meta))
    c2.params.flags = P.F_VISCOSITY | P.F_ARTI_VISC
    o = O.Oracle(c2)
    o.rates()
    a = o.field("DVDT")[: c2.n_real]
    mom = (c2.mass[:, None] * a).sum(0)
    scale = (c2.mass[:, None] * np.abs(a)).sum(0)
    assert np.all(np.abs(mom) < 1e-11 * scale)


def _solid_patch(n=12, dx=1e-3, omega=0.0, shear=None, type_id=102):
    prm = P.base_params(2, 1e-7)
    prm.flags = P.F_VISCOSITY
    P.reference_materials(prm, 50.0)
    g = (np.stack(np.meshgrid(np.arange(n), np.arange(n), indexing="ij"), -1).reshape(-1, 2) + 0.5) * dx
    g -= g.mean(0)
    N = len(g)
    v = np.zeros_like(g)
    v[:, 0] = -omega * g[:, 1]
    v[:, 1] = omega * g[:, 0]
    rho0 = prm.material(type_id).rho0
    sh = np.zeros((N, 4)) if shear is None else np.tile(np.asarray(shear, float), (N, 1))
    return cases.Case("patch", prm, N, 0, g, v, np.full(N, rho0 * dx * dx), np.full(N, rho0),
                      np.zeros(N), np.zeros(N), np.full(N, 100.0), np.full(N, 1.2 * dx),
                      np.full(N, type_id, np.int32), np.zeros(N, np.int32), np.zeros(N, np.int32), sh)


def test_jaumann_rotation():
    """Rigid spin: strain rate ~ 0, dS/dt = S R^T + (S R^T)^T (internalForce.f90:164-173)."""
    om = 10.0
    S0 = np.array([1e5, 3e4, 3e4, -2e5])  # column-major (1,1),(2,1),(1,2),(2,2)
    c = _solid_patch(omega=om, shear=S0)
    o = O.Oracle(c)
    o.rates()
    ds = o.field("DSDT")
    x = c.x
    inner = np.all(np.abs(x) < 3e-3, axis=1)
    S = S0.reshape(2, 2).T  # S[a, b]
    Rm = o.field("ROT")[inner].mean(0).reshape(2, 2).T  # rdot[a, b]
    want = np.zeros((2, 2))
    for a in range(2):
        for b in range(2):
            want[a, b] = sum(S[a, k] * Rm[b, k] + S[b, k] * Rm[a, k] for k in range(2))
    got = ds[inner].mean(0).reshape(2, 2).T
    # the rotation rate is the SPH estimate of the spin (dv_y/dx - dv_x/dy)/2 = omega
    assert abs(Rm[1, 0]) == pytest.approx(om, rel=0.05)
    strain = o.field("STRAIN")[inner]
    assert np.abs(strain).max() < 1e-8 * om
    assert rel_l2(got, want) < 1e-9


def test_radial_return_caps_j2():
    sig_y = P.f32(6e8)
    c = _solid_patch(type_id=101, shear=[9e8, 0, 0, -9e8])
    c.rho[:] = 7850.0
    c.mass[:] = 7850.0 * 1e-6
    o = O.Oracle(c)
    o.step()
    sh = o.field("SHEAR")
    j2 = (sh ** 2).sum(1)
    assert np.all(j2 <= sig_y ** 2 / 3 * (1 + 1e-12))
    assert np.all(j2 >= sig_y ** 2 / 3 * (1 - 1e-9))


def test_courant_mean_carries_over():
    """aver_courant is not reset between steps (timeIntegration.f90:213-251)."""
    c = cases.dam_break_2d(dx=0.1)
    o = O.Oracle(c)
    o.advance(2)
    mx2, mean2 = o.advance(1)
    h = c.h[: c.n_real]
    cc = c.c[: c.n_real]
    dv = o.field("DIVV")[: c.n_real]
    xi = c.params.dt * (h * dv + cc + P.f32(1.2) * (cc + h * np.abs(dv))) / h
    assert mx2 == pytest.approx(xi.max(), rel=1e-12)
    o2 = O.Oracle(c)
    _, m1 = o2.advance(2)
    assert mean2 == pytest.approx((m1 + xi.sum()) / c.n_real, rel=1e-12)


# ---- summation density and XSPH (density.f90:10-80, correctVelocity.f90) --
def _uniform_rest(flags):
    c = cases.dam_break_2d(dx=0.05)
    c.params = c.params.copy()
    c.params.flags |= flags
    c.rho = np.full_like(c.rho, 1000.0)
    return c


def test_normalised_summation_keeps_uniform_density():
    """With every rho_j = rho0 and equal masses, the Shepard-normalised sum
    m W / (m/rho0 W) is rho0 for every particle, near walls included."""
    c = _uniform_rest(P.F_SUM_DENSITY | P.F_NORM_DENSITY)
    o = O.Oracle(c)
    o.rates()
    rho = o.field("RHO")[: c.n_real]
    assert np.max(np.abs(rho / 1000.0 - 1.0)) < 1e-13


def test_summation_density_matches_direct_sum():
    """Unnormalised: rho_i = m_i W(0) + sum_j m_j W_ij over the BGGS set."""
    c = perturb(_uniform_rest(P.F_SUM_DENSITY), seed=5, x_frac=0.2)
    o = O.Oracle(c)
    o.bggs()
    off, lst = o.neighbors()
    h = c.h
    w0 = O.kernel(1, 2, 0.0, np.zeros(2), float(h[0]))[0]
    want = np.empty(c.n_real)
    for i in range(c.n_real):
        s = c.mass[i] * w0
        for j in lst[off[i]:off[i + 1]] - 1:
            dx = c.x[i] - c.x[j]
            s += c.mass[j] * O.kernel(1, 2, float(np.sqrt(dx @ dx)), dx, float(h[i]))[0]
        want[i] = s
    o.rates()
    assert rel_l2(o.field("RHO")[: c.n_real], want) < 1e-14


def test_xsph_zero_for_uniform_velocity():
    c = _uniform_rest(P.F_AVER_VELOCITY)
    c.v[:] = np.array([0.7, -0.2])
    o = O.Oracle(c)
    o.rates()
    assert np.all(o.field("AVER")[: c.n_real] == 0.0)


def test_xsph_matches_direct_sum():
    """XSPH (correctVelocity.f90:7-44) on a perturbed field: the correction
    of each real particle is sum_j 2 eps m_j / (rho_i + rho_j) W_ij (v_j - v_i)
    over the BGGS set, zero where Boundary == 1."""
    c = perturb(_uniform_rest(P.F_AVER_VELOCITY), seed=7, v_amp=0.4, x_frac=0.2)
    rng = np.random.default_rng(8)
    c.rho = c.rho * (1.0 + 0.01 * rng.standard_normal(c.n))
    o = O.Oracle(c)
    o.bggs()
    off, lst = o.neighbors()
    eps = float(c.params.xsph_eps)
    want = np.zeros((c.n_real, 2))
    for i in range(c.n_real):
        if c.boundary is not None and c.boundary[i] == 1:
            continue
        for j in lst[off[i]:off[i + 1]] - 1:
            dx = c.x[i] - c.x[j]
            w = O.kernel(1, 2, float(np.sqrt(dx @ dx)), dx, float(c.h[i]))[0]
            want[i] += (2 * eps * c.mass[j] / (c.rho[i] + c.rho[j])) * w * (c.v[j] - c.v[i])
    o.rates()
    got = o.field("AVER")[: c.n_real]
    assert np.abs(want).max() > 0
    assert rel_l2(got, want) < 1e-13


def test_continuity_and_divergence_match_direct_sums():
    """con_density (density.f90:83-107) and divergence (divergence.f90:6-29)
    on a perturbed field: drho_i/dt = rho_i sum_j m_j / rho_j (v_i - v_j) . dW_ij,
    div v_i = sum_j m_j / rho_j (v_j - v_i) . dW_ij and
    div x_i = sum_j m_j / rho_j (x_j - x_i) . dW_ij, over the BGGS set."""
    c = perturb(_uniform_rest(0), seed=9, v_amp=0.4, x_frac=0.2)
    rng = np.random.default_rng(10)
    c.rho = c.rho * (1.0 + 0.01 * rng.standard_normal(c.n))
    o = O.Oracle(c)
    o.bggs()
    off, lst = o.neighbors()
    drho, divv, divx = np.zeros(c.n_real), np.zeros(c.n_real), np.zeros(c.n_real)
    for i in range(c.n_real):
        for j in lst[off[i]:off[i + 1]] - 1:
            dx = c.x[i] - c.x[j]
            dw = O.kernel(1, 2, float(np.sqrt(dx @ dx)), dx, float(c.h[i]))[1]
            vol = c.mass[j] / c.rho[j]
            drho[i] += vol * ((c.v[i] - c.v[j]) @ dw)
            divv[i] += vol * ((c.v[j] - c.v[i]) @ dw)
            divx[i] += vol * ((c.x[j] - c.x[i]) @ dw)
    drho *= c.rho[: c.n_real]
    o.rates()
    assert rel_l2(o.field("DRHODT")[: c.n_real], drho) < 1e-12
    assert rel_l2(o.field("DIVV")[: c.n_real], divv) < 1e-12
    assert rel_l2(o.field("DIVX")[: c.n_real], divx) < 1e-12


def test_artificial_viscosity_matches_direct_sum():
    """Monaghan AV (artificialViscosity.f90:7-114) on a perturbed fluid: for
    approaching pairs (dv . dx < 0), phi = hbar dv.dx / (r^2 + (psi hbar)^2),
    PI = (beta phi - alpha cbar) phi / rhobar, a_i -= m_j PI dW_ij and
    de_i += 1/2 m_j PI dv . dW_ij, over the BGGS set."""
    c = perturb(cases.dam_break_2d(dx=0.05), seed=11, v_amp=0.5, x_frac=0.2)
    c.params = c.params.copy()
    c.params.av_beta = 0.7          # both terms of PI
    o = O.Oracle(c)
    o.bggs()
    off, lst = o.neighbors()
    o.rates()
    cs, rho = o.field("C"), o.field("RHO")
    al, be, psi = c.params.av_alpha, c.params.av_beta, c.params.av_psi
    a_want, e_want = np.zeros((c.n_real, 2)), np.zeros(c.n_real)
    for i in range(c.n_real):
        for j in lst[off[i]:off[i + 1]] - 1:
            dx, dv = c.x[i] - c.x[j], c.v[i] - c.v[j]
            vr = dv @ dx
            if not vr < 0:
                continue
            r2 = dx @ dx
            dw = O.kernel(1, 2, float(np.sqrt(r2)), dx, float(c.h[i]))[1]
            hb, cb, rb = 0.5 * (c.h[i] + c.h[j]), 0.5 * (cs[i] + cs[j]), 0.5 * (rho[i] + rho[j])
            phi = hb * vr / (r2 + (psi * hb) ** 2)
            pi = (be * phi - al * cb) * phi / rb
            a_want[i] -= c.mass[j] * pi * dw
            e_want[i] += 0.5 * c.mass[j] * pi * (dv @ dw)
    assert np.abs(a_want).max() > 0
    assert rel_l2(o.field("AV_DVDT"), a_want) < 1e-12
    assert rel_l2(o.field("AV_DEDT"), e_want) < 1e-12


def test_internal_force_matches_direct_sum():
    """internal_force, SPH = 2 (internalForce.f90:228-275, 332-334), on a
    perturbed fluid: a_i,d = sum_j m_j [-(p_i/rho_i^2 + p_j/rho_j^2) dW_d
    + sum_e (eta_i eps_i,de / rho_i^2 + eta_j eps_j,de / rho_j^2) dW_e] and
    de_i = T ds/dt_i + 1/2 sum_j m_j (p_i/rho_i^2 + p_j/rho_j^2) (v_i - v_j) . dW,
    with p, eps (the reference's fluid strain rate), eta and T ds/dt taken
    from the oracle's own state."""
    c = perturb(cases.dam_break_2d(dx=0.05), seed=12, v_amp=0.5, x_frac=0.2)
    c.params = c.params.copy()
    c.params.material(2).eta = 50.0     # a viscous term of the pressure term's order
    o = O.Oracle(c)
    o.bggs()
    off, lst = o.neighbors()
    o.rates()
    p, rho, eta = o.field("P"), o.field("RHO"), o.field("VISC")
    eps = o.field("STRAIN").reshape(-1, 2, 2).transpose(0, 2, 1)   # eps[i][d][e]
    tds = o.field("TDSDT")
    a_want, e_want = np.zeros((c.n_real, 2)), np.zeros(c.n_real)
    for i in range(c.n_real):
        for j in lst[off[i]:off[i + 1]] - 1:
            dx = c.x[i] - c.x[j]
            dw = O.kernel(1, 2, float(np.sqrt(dx @ dx)), dx, float(c.h[i]))[1]
            pp = p[i] / rho[i] ** 2 + p[j] / rho[j] ** 2
            tv = eta[i] * eps[i] / rho[i] ** 2 + eta[j] * eps[j] / rho[j] ** 2
            a_want[i] += c.mass[j] * (-pp * dw + tv @ dw)
            e_want[i] += c.mass[j] * pp * ((c.v[i] - c.v[j]) @ dw)
    e_want = tds[: c.n_real] + 0.5 * e_want
    assert np.abs(eps[: c.n_real]).max() > 0 and np.abs(tds[: c.n_real]).max() > 0
    assert rel_l2(o.field("IN_DVDT"), a_want) < 1e-12
    assert rel_l2(o.field("IN_DEDT"), e_want) < 1e-12


def test_external_force_matches_direct_sum():
    """external_force (externalForce.f90:7-101) on a perturbed dam break:
    gravity on the last axis, plus for each fluid-wall pair of the BGGS set
    with r < r0 the repulsion f_s ((r0/r)^p1 - (r0/r)^p2) dx / r^2."""
    c = perturb(cases.dam_break_2d(dx=0.05), seed=13, v_amp=0.2, x_frac=0.35)
    o = O.Oracle(c)
    o.bggs()
    off, lst = o.neighbors()
    o.rates()
    prm = c.params
    want = np.zeros((c.n_real, 2))
    want[:, 1] = prm.gravity
    hits = 0
    for i in range(c.n_real):
        for j in lst[off[i]:off[i + 1]] - 1:
            if not (c.type[i] > 0 and c.type[j] < 0):
                continue
            dx = c.x[i] - c.x[j]
            r = float(np.sqrt(dx[0] * dx[0] + dx[1] * dx[1]))
            if r < prm.wall_r0:
                t = prm.wall_r0 / r
                want[i] += prm.wall_fs * (t ** prm.wall_p1 - t ** prm.wall_p2) / (r * r) * dx
                hits += 1
    assert hits > 0
    assert rel_l2(o.field("EX_DVDT"), want) < 1e-12


def test_fluid_strain_rate_matches_direct_sum():
    """The fluid strain rate of internal_force (internalForce.f90:56-77, with
    the reference's unsymmetrised off-diagonals): with dv = v_j - v_i and
    V_j = m_j / rho_j, eps_de = 2 sum_j V_j dv_d dW_e for d != e and
    eps_dd = 2 sum_j V_j dv_d dW_d - 2/3 sum_j V_j dv . dW."""
    c = perturb(cases.dam_break_2d(dx=0.05), seed=14, v_amp=0.5, x_frac=0.2)
    o = O.Oracle(c)
    o.bggs()
    off, lst = o.neighbors()
    o.rates()
    rho = o.field("RHO")
    want = np.zeros((c.n_real, 2, 2))
    for i in range(c.n_real):
        g = np.zeros((2, 2))
        for j in lst[off[i]:off[i + 1]] - 1:
            dx = c.x[i] - c.x[j]
            dw = O.kernel(1, 2, float(np.sqrt(dx @ dx)), dx, float(c.h[i]))[1]
            g += (c.mass[j] / rho[j]) * np.outer(c.v[j] - c.v[i], dw)
        want[i] = 2.0 * g - (2.0 / 3.0) * np.trace(g) * np.eye(2)
    got = o.field("STRAIN").reshape(-1, 2, 2).transpose(0, 2, 1)[: c.n_real]
    assert rel_l2(got, want) < 1e-12
    # the off-diagonals are not symmetrised (quirk of the reference)
    assert np.abs(got[:, 0, 1] - got[:, 1, 0]).max() > 1e-3 * np.abs(got).max()


def test_solid_internal_force_matches_direct_sum():
    """internal_force for solid targets (internalForce.f90:137-186, 256-263):
    sigma = S - p I, and a_i,d = sum_j m_j sum_e (sigma_i,de / rho_i^2 +
    sigma_j,de / rho_j^2) dW_e, on a perturbed cantilever with a random
    symmetric deviatoric stress and density."""
    c = perturb(cases.cantilever_2d(dx=2e-3, length=0.04, thickness=0.01), seed=15, v_amp=0.5, x_frac=0.15)
    rng = np.random.default_rng(16)
    nr = c.n_real
    s_xy, s_d = rng.standard_normal(nr) * 1e7, rng.standard_normal(nr) * 1e7
    c.shear = np.zeros((c.n, 4))
    c.shear[:nr] = np.stack([s_d, s_xy, s_xy, -s_d], axis=1)
    c.rho = c.rho * (1.0 + 1e-3 * rng.standard_normal(c.n))
    o = O.Oracle(c, covering_band=True)
    o.bggs()
    off, lst = o.neighbors()
    o.rates()
    rho = o.field("RHO")
    sig = o.field("STRESS").reshape(-1, 2, 2).transpose(0, 2, 1)   # sig[i][d][e]
    want = np.zeros((nr, 2))
    for i in range(nr):
        for j in lst[off[i]:off[i + 1]] - 1:
            dx = c.x[i] - c.x[j]
            dw = O.kernel(1, 2, float(np.sqrt(dx @ dx)), dx, float(c.h[i]))[1]
            want[i] += c.mass[j] * ((sig[i] / rho[i] ** 2 + sig[j] / rho[j] ** 2) @ dw)
    assert np.all(np.abs(c.type[:nr]) > 100)
    assert rel_l2(o.field("IN_DVDT"), want) < 1e-12


def test_jaumann_rate_matches_direct_formula():
    """The solid stress rate (internalForce.f90:82-95, 137-180): with the
    velocity gradient G = sum_j V_j (v_j - v_i) (x) dW, eps = (G + G^T)/2,
    R = (G - G^T)/2 and epsbar = eps - tr(eps)/3 I (a third even in 2-D),
    dS/dt = 2 G_mod epsbar + S R^T + (S R^T)^T, on a perturbed cantilever with
    a random symmetric S."""
    c = perturb(cases.cantilever_2d(dx=2e-3, length=0.04, thickness=0.01), seed=17, v_amp=0.5, x_frac=0.15)
    rng = np.random.default_rng(18)
    nr = c.n_real
    s_xy, s_d = rng.standard_normal(nr) * 1e7, rng.standard_normal(nr) * 1e7
    c.shear = np.zeros((c.n, 4))
    c.shear[:nr] = np.stack([s_d, s_xy, s_xy, -s_d], axis=1)
    o = O.Oracle(c, covering_band=True)
    o.bggs()
    off, lst = o.neighbors()
    o.rates()
    rho = o.field("RHO")
    gmod = c.params.material(int(c.type[0])).eta
    want = np.zeros((nr, 2, 2))
    for i in range(nr):
        g = np.zeros((2, 2))
        for j in lst[off[i]:off[i + 1]] - 1:
            dx = c.x[i] - c.x[j]
            dw = O.kernel(1, 2, float(np.sqrt(dx @ dx)), dx, float(c.h[i]))[1]
            g += (c.mass[j] / rho[j]) * np.outer(c.v[j] - c.v[i], dw)
        eps, rot = 0.5 * (g + g.T), 0.5 * (g - g.T)
        epsbar = eps - (np.trace(eps) / 3.0) * np.eye(2)
        S = c.shear[i].reshape(2, 2).T
        srt = S @ rot.T
        want[i] = 2.0 * gmod * epsbar + srt + srt.T
    got = o.field("DSDT").reshape(-1, 2, 2).transpose(0, 2, 1)[:nr]
    assert rel_l2(got, want) < 1e-12


# ---- kernel gradient correction (kernelGradientCorrection.f90:8-51) --------
def _kgc(c):
    c.params = c.params.copy()
    c.params.flags |= P.F_KERNEL_CORRECTION
    return c


def test_kgc_makes_position_divergence_exact():
    """With the corrected gradients sum_j V_j (x_j - x_i) (x) dW'_ij is the
    identity for every solid target, so div x = dim exactly, boundary
    particles included."""
    c = _kgc(perturb(cases.cantilever_2d(dx=2e-3, length=0.04, thickness=0.01), seed=3, x_frac=0.15))
    o = O.Oracle(c, covering_band=True)
    o.rates()
    divx = o.field("DIVX")[: c.n_real]
    assert np.max(np.abs(divx - 2.0)) < 1e-12
    # without the correction the boundary rows are far from 2
    c2 = perturb(cases.cantilever_2d(dx=2e-3, length=0.04, thickness=0.01), seed=3, x_frac=0.15)
    o2 = O.Oracle(c2, covering_band=True)
    o2.rates()
    assert np.max(np.abs(o2.field("DIVX")[: c2.n_real] - 2.0)) > 0.1


def test_mcpe_pivoting_solves():
    """The pivoted elimination on a 3x3 system gives the exact solution."""
    c = _kgc(perturb(cases.dam_break_3d(dx=0.03), seed=4, x_frac=0.1))
    c.type[: c.n_real] = 102          # treat the block as a solid so A is built
    c.params.flags &= ~(P.F_GRAVITY | P.F_DUMMY | P.F_EXT_FORCE)
    o = O.Oracle(c)
    o.rates()
    divx = o.field("DIVX")[: c.n_real]
    # targets whose neighbours are all solid (the walls are Type -2: excluded from A
    # but still summed by divergence) -> check interior ones only
    x = c.x[: c.n_real]
    lo, hi = x.min(0) + 0.08, x.max(0) - 0.08   # farther than 2h = 0.072 from the walls
    inner = np.all((x > lo) & (x < hi), axis=1)
    assert inner.sum() > 10
    assert np.max(np.abs(divx[inner] - 3.0)) < 1e-12


# ---- momentum forms SPH = 1 / 3 (internalForce.f90:194-329, density.f90:110-148)
def _closed_box(pa_sph, seed=5):
    c = cases.dam_break_2d(dx=0.05, width=1.0, height=1.0)
    c = perturb(c.subset_real(np.ones(c.n_real, bool)), seed=seed, v_amp=0.5, x_frac=0.2)
    keep = np.arange(c.n_real)
    c2 = cases.Case(c.name, c.params.copy(), c.n_real, 0, c.x[keep], c.v[keep], c.mass[keep],
                    c.rho[keep], c.p[keep], c.e[keep], c.c[keep], c.h[keep], c.type[keep],
                    c.state[keep], c.boundary[keep], None, dict(c.meta))
    c2.params.flags = P.F_VISCOSITY | P.F_ARTI_VISC
    c2.params.pa_sph = pa_sph
    return c2


@pytest.mark.parametrize("pa_sph", [1, 3])
def test_scheme_momentum_conservation(pa_sph):
    """Both forms are antisymmetric in the pair at equal h: p* of the PVRS
    solver is the same seen from either particle."""
    c = _closed_box(pa_sph)
    o = O.Oracle(c)
    o.rates()
    a = o.field("DVDT")[: c.n_real]
    mom = (c.mass[:, None] * a).sum(0)
    scale = (c.mass[:, None] * np.abs(a)).sum(0)
    assert np.all(np.abs(mom) < 1e-11 * scale)


@pytest.mark.parametrize("pa_sph", [1, 2, 3])
def test_scheme_galilean_invariance(pa_sph):
    """A uniform velocity added to every particle changes no rate: the
    Riemann velocity v* moves with it, so v_i - v* does not."""
    c = _closed_box(pa_sph)
    o = O.Oracle(c)
    o.rates()
    ref = {k: o.field(k)[: c.n_real].copy() for k in ("DVDT", "DEDT", "DRHODT")}
    c.v = c.v + np.array([0.3, -0.2])
    o2 = O.Oracle(c)
    o2.rates()
    for k, r in ref.items():
        assert rel_l2(o2.field(k)[: c.n_real], r) < 1e-12, k


def test_riemann_at_rest_equals_sph1():
    """At rest with one pressure, p* = P: the PVRS force is the SPH = 1 force,
    and the Riemann density rate and both energy rates vanish."""
    out = {}
    for pa_sph in (1, 3):
        c = _closed_box(pa_sph)
        c.params.flags = P.F_VISCOSITY
        c.v[:] = 0.0
        c.rho[:] = 1010.0                    # one density: one Tait pressure
        c.p[:] = O.eos(c.params.materials[0], False, 1010.0)[0]   # c stays the case's
        o = O.Oracle(c)
        o.rates()
        out[pa_sph] = {k: o.field(k)[: c.n_real].copy() for k in ("DVDT", "DEDT", "DRHODT")}
    assert rel_l2(out[3]["DVDT"], out[1]["DVDT"]) < 1e-13
    assert np.max(np.abs(out[1]["DVDT"])) > 0
    for k in ("DEDT", "DRHODT"):
        assert np.all(np.abs(out[3][k]) < 1e-12)


def test_elastic_gate_grows_without_bound():
    """The elastic gate with the reference's coupling is not a bounded
    physical run: in the oracle itself (dx = 2.5 mm, 12,880 real particles)
    the largest speed grows by orders of magnitude within a few hundred
    steps, while a water column released from rest moves at about g t
    (under 0.04 m/s at t = 3.6 ms).  The 20,000-step run of this geometry is
    therefore no measurement, on the CPU or on the GPU; the GPU tests use the
    gate only over windows where it stays bounded."""
    c = cases.gate_2d(dx=0.0025)
    nr = c.n_real
    o = O.Oracle(c, omp=True)
    o.advance(300)
    early = float(np.linalg.norm(o.field("V")[:nr], axis=1).max())
    o.advance(500)
    late = float(np.linalg.norm(o.field("V")[:nr], axis=1).max())
    t = o.info()[1]
    assert early < 1.0
    assert late > 50.0 * early and late > 100.0 * 9.81 * t, (early, late, t)


def test_artificial_heat_matches_direct_sum():
    """arti_heat (artificialHeat.f90:6-56) on a perturbed fluid with a varied
    internal energy: q = 0.1 h c + h^2 (|div v| - div v) per particle (div v
    of this step; walls 0), de_i = sum_j 2 m_j q_ij (dx . dW_ij) (e_i - e_j)
    / (rho_ij (r^2 + 0.01 h_ij^2)) over the BGGS set with pair averages, and
    the energy rate assembled as in + av + ah (singleStep.f90:141)."""
    c = perturb(cases.dam_break_2d(dx=0.05), seed=12, v_amp=0.5, x_frac=0.2)
    rng = np.random.default_rng(13)
    c.e = c.e.copy()
    c.e[: c.n_real] = rng.uniform(0.0, 50.0, c.n_real)
    c.params = c.params.copy()
    c.params.flags |= P.F_ARTI_HEAT
    o = O.Oracle(c)
    o.bggs()
    off, lst = o.neighbors()
    o.rates()
    cs, rho, divv = o.field("C"), o.field("RHO"), o.field("DIVV")
    q = 0.1 * c.h * cs + c.h ** 2 * (np.abs(divv) - divv)
    want = np.zeros(c.n_real)
    for i in range(c.n_real):
        for j in lst[off[i]:off[i + 1]] - 1:
            dx = c.x[i] - c.x[j]
            dw = O.kernel(1, 2, float(np.sqrt(dx @ dx)), dx, float(c.h[i]))[1]
            qij, hij, rij = 0.5 * (q[i] + q[j]), 0.5 * (c.h[i] + c.h[j]), 0.5 * (rho[i] + rho[j])
            aux = qij * (dx @ dw) / (rij * (dx @ dx + 0.01 * hij ** 2))
            want[i] += 2 * c.mass[j] * aux * (c.e[i] - c.e[j])
    got = o.field("AH_DEDT")
    assert np.abs(want).max() > 0 and np.all(divv[c.n_real:] == 0.0)
    assert rel_l2(got, want) < 1e-12
    dedt = o.field("DEDT")[: c.n_real]
    assert rel_l2(dedt, o.field("IN_DEDT") + o.field("AV_DEDT") + got) < 1e-15
