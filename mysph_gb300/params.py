"""ctypes mirror of ``sph_params`` / ``sph_material`` (include/sph_gpu.h).

The run parameters are the sph.toml keys read by
src/Initialize/getValueFromToml.f90:95-185 plus every constant the reference
hard-codes per case nick (EOS, viscosity table, AV coefficients, wall force,
artificial stress).  ``reference_preset(nick)`` returns the values the
reference itself uses for a nick, with its single-precision literals rounded
exactly as gfortran rounds them (``f32``).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

# status codes
SPH_OK = 0
SPH_E_INVALID = -1
SPH_E_NOMEM = -2
SPH_E_CUDA = -3
SPH_E_STATE = -4
SPH_E_UNSUPPORTED = -5
SPH_E_NONFINITE = -6
SPH_E_OVERFLOW = -7
SPH_E_TIMEOUT = -8
SPH_E_RANGE = -9
SPH_E_TOO_LARGE = -10
NOALLOC_MAX_PAIRS = 1 << 20

# flags (getValueFromToml.f90:135-154)
F_SUM_DENSITY = 1 << 0
F_NORM_DENSITY = 1 << 1
F_VISCOSITY = 1 << 2
F_GRAVITY = 1 << 3
F_EXT_FORCE = 1 << 4
F_ARTI_VISC = 1 << 5
F_ARTI_STRESS = 1 << 6
F_AVER_VELOCITY = 1 << 7
F_DUMMY = 1 << 8
F_GRAVITY_SKIP_SOLIDS = 1 << 9
F_FSI_FLUID_VISCOUS = 1 << 10
F_KERNEL_CORRECTION = 1 << 11
F_ARTI_HEAT = 1 << 12

TOML_FLAG_KEYS = {
    "summationDensity": F_SUM_DENSITY,
    "normalizeDensity": F_NORM_DENSITY,
    "viscosity": F_VISCOSITY,
    "gravity": F_GRAVITY,
    "externalForce": F_EXT_FORCE,
    "artificialViscosity": F_ARTI_VISC,
    "artificialStress": F_ARTI_STRESS,
    "averageVelocity": F_AVER_VELOCITY,
    "artificialHeat": F_ARTI_HEAT,
    "dummyParticle": F_DUMMY,
}

EOS_NONE, EOS_GAS, EOS_TAIT, EOS_MORRIS = 0, 1, 2, 3
EOS_MG_SOLID, EOS_LINEAR = 101, 102
MAX_MATERIALS = 8

PREC_FP64, PREC_MIXED, PREC_DF64 = 0, 1, 2

FIELD = dict(X=1, V=2, MASS=3, RHO=4, P=5, E=6, C=7, H=8, DIVX=9, DIVV=10,
             DISP=11, STRESS=12, SHEAR=13, DSDT=14, DVDT=15, DRHODT=16,
             DEDT=17, NNEIGH=18, TYPE=19, VISC=20, STRAIN=21, AVER=22)
# components per particle: 'v' = dim, 't' = dim*dim, 's' = 1
FIELD_SHAPE = dict(X="v", V="v", MASS="s", RHO="s", P="s", E="s", C="s", H="s",
                   DIVX="s", DIVV="s", DISP="v", STRESS="t", SHEAR="t",
                   DSDT="t", DVDT="v", DRHODT="s", DEDT="s", NNEIGH="s",
                   TYPE="s", VISC="s", STRAIN="t", AVER="v")

TERM_INTERNAL, TERM_ARTI_VISC, TERM_EXTERNAL, TERM_ARTI_STRESS, TERM_ARTI_HEAT = 1, 2, 4, 8, 16

OPT_GRAPHS, OPT_SMEM_CARVEOUT, OPT_BLOCK_SIZE, OPT_LIST_LEN, OPT_PERSISTENT, OPT_LANES = 1, 2, 3, 4, 5, 6

STAGES = ("hash", "permute", "pass_a", "pass_b", "update")


class SphBlock(C.Structure):
    """sph_block of include/sph_gpu.h: a lattice block generated on the device."""
    _fields_ = [
        ("n", C.c_int32 * 3), ("type", C.c_int32), ("state", C.c_int32), ("up_axis", C.c_int32),
        ("clamp_axis", C.c_int32), ("reserved", C.c_int32),
        ("origin", C.c_double * 3), ("spacing", C.c_double * 3),
        ("mass", C.c_double), ("h", C.c_double), ("c", C.c_double), ("rho", C.c_double),
        ("p_rho0_g", C.c_double), ("p_level", C.c_double),
        ("tait_b", C.c_double), ("tait_gamma", C.c_double), ("tait_rho0", C.c_double),
        ("v", C.c_double * 3), ("v_ramp", C.c_double * 3), ("v_ramp_len", C.c_double),
        ("clamp_below", C.c_double), ("clamp_above", C.c_double),
    ]


def block(n, origin, spacing, *, mass, h, c=0.0, rho=0.0, type_id=2, state=0, up_axis=1,
          p_rho0_g=0.0, p_level=0.0, tait=None, v=(0.0, 0.0, 0.0), v_ramp=(0.0, 0.0, 0.0),
          v_ramp_len=0.0, clamp_below=-math.inf, clamp_above=math.inf, clamp_axis=0) -> SphBlock:
    """One block; `tait` = (b, gamma, rho0) derives the density from the
    hydrostatic pressure with the inverse Tait EOS."""
    b = SphBlock()
    for a in range(3):
        b.n[a] = int(n[a]) if a < len(n) else 1
        b.origin[a] = float(origin[a]) if a < len(origin) else 0.0
        b.spacing[a] = float(spacing[a]) if a < len(spacing) else 0.0
        b.v[a] = float(v[a]) if a < len(v) else 0.0
        b.v_ramp[a] = float(v_ramp[a]) if a < len(v_ramp) else 0.0
    b.type, b.state, b.up_axis = int(type_id), int(state), int(up_axis)
    b.mass, b.h, b.c, b.rho = float(mass), float(h), float(c), float(rho)
    b.p_rho0_g, b.p_level = float(p_rho0_g), float(p_level)
    if tait is not None:
        b.tait_b, b.tait_gamma, b.tait_rho0 = (float(t) for t in tait)
    b.v_ramp_len = float(v_ramp_len)
    b.clamp_below = float(clamp_below)
    b.clamp_above = float(clamp_above)
    b.clamp_axis = int(clamp_axis)
    return b


def f32(x: float) -> float:
    """A Fortran default-real literal as the reference's real(8) sees it."""
    return float(np.float32(x))


class SphMaterial(C.Structure):
    _fields_ = [
        ("type", C.c_int32), ("eos", C.c_int32), ("solid", C.c_int32),
        ("yield_", C.c_int32),
        ("rho0", C.c_double), ("c0", C.c_double), ("gamma", C.c_double),
        ("K", C.c_double), ("eta", C.c_double), ("sigma_y", C.c_double),
        ("mg_cs", C.c_double), ("mg_s", C.c_double),
    ]


class SphParams(C.Structure):
    _fields_ = [
        ("dim", C.c_int32), ("skf", C.c_int32), ("pa_sph", C.c_int32),
        ("sle", C.c_int32), ("flags", C.c_uint32), ("precision", C.c_int32),
        ("dt", C.c_double),
        ("gravity", C.c_double),
        ("av_alpha", C.c_double), ("av_beta", C.c_double), ("av_psi", C.c_double),
        ("av_alpha_solid", C.c_double), ("av_beta_solid", C.c_double),
        ("cour_alpha", C.c_double), ("cour_beta", C.c_double),
        ("wall_fs", C.c_double), ("wall_r0", C.c_double),
        ("wall_p1", C.c_double), ("wall_p2", C.c_double),
        ("pen_factor", C.c_double), ("pen_n1", C.c_double), ("pen_n2", C.c_double),
        ("contact_delta", C.c_double),
        ("as_eps", C.c_double), ("as_n", C.c_double), ("as_dp", C.c_double),
        ("xsph_eps", C.c_double),
        ("n_materials", C.c_int32), ("reserved0", C.c_int32),
        ("materials", SphMaterial * MAX_MATERIALS),
        ("cell_size", C.c_double),
        ("domain_lo", C.c_double * 3), ("domain_hi", C.c_double * 3),
        ("grid_margin", C.c_double),
    ]

    def copy(self) -> "SphParams":
        out = SphParams()
        C.memmove(C.byref(out), C.byref(self), C.sizeof(SphParams))
        return out

    def add_material(self, **kw) -> None:
        if self.n_materials >= MAX_MATERIALS:
            raise ValueError("material table full")
        m = self.materials[self.n_materials]
        for k, v in kw.items():
            setattr(m, k, v)
        self.n_materials += 1

    def material(self, type_id: int) -> SphMaterial:
        for k in range(self.n_materials):
            if self.materials[k].type == abs(type_id):
                return self.materials[k]
        raise KeyError(type_id)


def water(c0: float, rho0: float = 1000.0, eta: float = f32(1e-3)) -> dict:
    """Tait water, type 2 (eos.f90:23-53; eta of viscosity.f90:17-18)."""
    return dict(type=2, eos=EOS_TAIT, solid=0, rho0=rho0, c0=c0, gamma=7.0, eta=eta)


def linear_solid(type_id: int, rho0: float, K: float, G: float,
                 sigma_y: float = 0.0) -> dict:
    """Linear-EOS solid (eos.f90:219-248) with shear modulus G."""
    return dict(type=type_id, eos=EOS_LINEAR, solid=1, rho0=rho0, K=K, eta=G,
                sigma_y=sigma_y, yield_=1 if sigma_y > 0 else 0)


def base_params(dim: int, dt: float) -> SphParams:
    """Defaults of getValueFromToml.f90:113-151 and the `case default`
    constants of the physics modules (externalForce.f90:62-72,
    artificialViscosity.f90:75-78, courantNumber.f90:22-24,
    artificialTerm.f90:17, correctVelocity.f90:20)."""
    p = SphParams()
    p.dim = dim
    p.skf = 1
    p.pa_sph = 2
    p.sle = 0
    p.flags = F_SUM_DENSITY  # summationDensity defaults to .true.
    p.precision = PREC_FP64
    p.dt = dt
    p.gravity = -9.81
    p.av_alpha, p.av_beta, p.av_psi = 1.0, 1.0, f32(0.1)
    p.av_alpha_solid, p.av_beta_solid = 1.0, 1.0
    p.cour_alpha, p.cour_beta = 1.0, 1.0
    p.wall_fs, p.wall_r0, p.wall_p1, p.wall_p2 = f32(1e-2), f32(1.25e-5), 12.0, 4.0
    p.pen_factor, p.pen_n1, p.pen_n2 = 1e5, 6.0, 4.0
    p.contact_delta = f32(0.001)
    p.as_eps, p.as_n, p.as_dp = f32(0.2), 4.0, 0.0
    p.xsph_eps = f32(0.3)
    p.n_materials = 0
    p.cell_size = 0.0
    p.grid_margin = 0.0
    return p


def reference_materials(p: SphParams, tait_c0: float) -> None:
    """The reference's material constants (eos.f90, viscosity.f90,
    timeIntegration.f90:147-158) as one table."""
    p.add_material(**water(tait_c0))
    p.add_material(type=101, eos=EOS_MG_SOLID, solid=1, rho0=7850.0,
                   gamma=f32(1.81), mg_cs=3630.0, mg_s=f32(1.8), eta=f32(8e10),
                   sigma_y=f32(6e8), yield_=1)
    p.add_material(**linear_solid(102, 1100.0, f32(2e7), f32(4.27e6)))
    p.add_material(**linear_solid(103, 2500.0, f32(0.33e6), f32(0.5e6)))
    p.add_material(**linear_solid(104, 2700.0, f32(7.235e10), f32(2.77443609023e10),
                                  sigma_y=f32(3e8)))


def reference_preset(nick: str, dim: int, dt: float) -> SphParams:
    """Per-nick constants of the reference, made explicit."""
    p = base_params(dim, dt)
    c_tait = {"dam_break": 50.0, "water_impact": 10.0}.get(nick, 0.0)
    reference_materials(p, c_tait)
    if nick == "dam_break":
        p.wall_fs = 10.0           # externalForce.f90:84-87 (r0 set by the case)
        p.contact_delta = f32(0.2)
    elif nick == "db_gate":
        p.contact_delta = f32(0.001)
        p.flags |= F_GRAVITY_SKIP_SOLIDS
    elif nick == "water_impact":
        p.contact_delta = f32(0.002)
        p.flags |= F_GRAVITY_SKIP_SOLIDS
        p.as_dp = 0.0
    elif nick in ("can_beam", "can_beam_3d", "beam_oil"):
        p.av_alpha = p.av_beta = p.av_alpha_solid = p.av_beta_solid = 0.5
        if nick == "can_beam":
            p.as_dp = f32(1e-3)
    elif nick == "taylor_rod":
        p.av_alpha = p.av_beta = p.av_alpha_solid = p.av_beta_solid = 0.5
        p.av_psi = f32(0.01)
        p.wall_fs = f32(1e-2)
    elif nick in ("tnt_bar", "tnt_cylinder", "undex_cylinder", "undex_chamber"):
        p.av_beta = p.av_beta_solid = 10.0
        p.cour_beta = 10.0
    return p


def params_to_dict(p: SphParams) -> dict:
    out = {}
    for name, _ in SphParams._fields_:
        v = getattr(p, name)
        if name == "materials":
            v = [{n: getattr(p.materials[k], n) for n, _ in SphMaterial._fields_}
                 for k in range(p.n_materials)]
        elif isinstance(v, C.Array):
            v = list(v)
        out[name] = v
    return out
