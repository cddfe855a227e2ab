"""Case generators: initial particle lattices and wall ("dummy") particles.

Two families:

* the workloads the GPU path is measured on — 2-D dam break (water column
  1.0 x 2.0 m in a 4.0 x 3.0 m tank), 3-D dam break (block 0.6 x 0.3 x
  0.6 m, L x W x H, in a 1.6 x 0.6 x 1.0 m box), 2-D elastic-gate
  fluid-structure case, 2-D cantilever beam and a seeded dam-break ensemble;
* reference-native presets that reproduce the reference's own case nicks
  (input.f90:1031-1154, 1336-1405; dummyParticles.f90:544-765) including
  its single-precision literals.

Every generator returns a :class:`Case`: real particles first, then walls,
in the column-major layout of include/sph_gpu.h (``x[n*dim + d]``).  Walls
are generated once and stay static; the reference regenerates identical
walls every step (dummyParticles.f90:9-45).  In 3-D the last axis is
vertical, as the reference's gravity acts on ``dvdt(Field%Dim, i)``
(externalForce.f90:47-56).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import params as P

G = 9.81


@dataclass
class Case:
    name: str
    params: P.SphParams
    n_real: int
    n_wall: int
    x: np.ndarray          # (N, dim)
    v: np.ndarray          # (N, dim)
    mass: np.ndarray
    rho: np.ndarray
    p: np.ndarray
    e: np.ndarray
    c: np.ndarray
    h: np.ndarray
    type: np.ndarray       # int32
    state: np.ndarray      # int32
    boundary: np.ndarray   # int32
    shear: np.ndarray | None = None   # (N, dim*dim) column-major per particle
    meta: dict = field(default_factory=dict)

    @property
    def dim(self) -> int:
        return int(self.params.dim)

    @property
    def n(self) -> int:
        return self.n_real + self.n_wall

    def arrays(self):
        """Contiguous arrays in include/sph_gpu.h order."""
        f = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        i = lambda a: np.ascontiguousarray(a, dtype=np.int32)
        sh = None if self.shear is None else f(self.shear)
        return (f(self.x), f(self.v), f(self.mass), f(self.rho), f(self.p),
                f(self.e), f(self.c), f(self.h), i(self.type), i(self.state),
                i(self.boundary), sh)

    def subset_real(self, keep: np.ndarray) -> "Case":
        """Keep a subset of the real particles (all walls stay)."""
        idx = np.concatenate([np.flatnonzero(keep), np.arange(self.n_real, self.n)])
        sel = lambda a: None if a is None else a[idx]
        return Case(self.name, self.params, int(keep.sum()), self.n_wall,
                    self.x[idx], self.v[idx], self.mass[idx], self.rho[idx],
                    self.p[idx], self.e[idx], self.c[idx], self.h[idx],
                    self.type[idx], self.state[idx], self.boundary[idx],
                    sel(self.shear), dict(self.meta))


def tait_density(p: np.ndarray, c0: float, rho0: float = 1000.0, gamma: float = 7.0) -> np.ndarray:
    """Inverse Tait EOS, arti_water_eos_1(Density=.true.) (eos.f90:43-47)."""
    b = ((c0 * c0) * rho0) / gamma
    return np.power(p / b + 1, 1.0 / gamma) * rho0


def _assemble(name, prm, real: dict, walls: dict, meta=None) -> Case:
    dim = prm.dim
    cat = lambda k, dflt: np.concatenate([real.get(k, dflt(len(real["x"]))),
                                          walls.get(k, dflt(len(walls["x"])))])
    zeros = lambda n: np.zeros(n)
    izeros = lambda n: np.zeros(n, dtype=np.int32)
    nr, nw = len(real["x"]), len(walls["x"])
    x = np.concatenate([real["x"], walls["x"]]).reshape(-1, dim)
    v = np.concatenate([real.get("v", np.zeros((nr, dim))), walls.get("v", np.zeros((nw, dim)))])
    shear = None
    if "shear" in real:
        shear = np.concatenate([real["shear"], np.zeros((nw, dim * dim))])
    return Case(name, prm, nr, nw, x, v, cat("mass", zeros), cat("rho", zeros),
                cat("p", zeros), cat("e", zeros), cat("c", zeros), cat("h", zeros),
                cat("type", izeros).astype(np.int32), cat("state", izeros).astype(np.int32),
                cat("boundary", izeros).astype(np.int32), shear, meta or {})


def _grid2(nx, ny, x0, y0, dx, order="xy"):
    """Lattice points ((i-1/2)dx, (j-1/2)dx) with k = (i-1)*ny + j ordering
    (input.f90:1045-1047)."""
    i = np.arange(1, nx + 1)
    j = np.arange(1, ny + 1)
    I, J = np.meshgrid(i, j, indexing="ij")
    return np.stack([x0 + (I.ravel() - 0.5) * dx, y0 + (J.ravel() - 0.5) * dx], axis=1)


def _grid3(nx, ny, nz, x0, y0, z0, dx):
    i, j, k = np.arange(1, nx + 1), np.arange(1, ny + 1), np.arange(1, nz + 1)
    I, J, K = np.meshgrid(i, j, k, indexing="ij")
    return np.stack([x0 + (I.ravel() - 0.5) * dx, y0 + (J.ravel() - 0.5) * dx,
                     z0 + (K.ravel() - 0.5) * dx], axis=1)


def _water_params(dim, dt, c0, dx, alpha=0.1, beta=0.0) -> P.SphParams:
    prm = P.base_params(dim, dt)
    prm.flags = (P.F_VISCOSITY | P.F_GRAVITY | P.F_ARTI_VISC | P.F_DUMMY | P.F_EXT_FORCE)
    prm.add_material(**P.water(c0))
    prm.av_alpha, prm.av_beta = alpha, beta
    prm.av_alpha_solid, prm.av_beta_solid = alpha, beta
    prm.wall_fs, prm.wall_r0 = 10.0, dx
    prm.contact_delta = P.f32(0.2)
    return prm


# ---------------------------------------------------------------------------
# 2-D dam break: 1.0 x 2.0 m column, 4.0 x 3.0 m tank, 3 wall layers
# ---------------------------------------------------------------------------
def dam_break_2d(dx: float = 0.02, width: float = 1.0, height: float = 2.0,
                 tank_w: float = 4.0, tank_h: float = 3.0, layers: int = 3,
                 h_factor: float = 1.2, cfl: float = 0.2, alpha: float = 0.1,
                 beta: float = 0.0) -> Case:
    h = h_factor * dx
    c0 = 10.0 * math.sqrt(2.0 * G * height)
    dt = cfl * h / c0
    prm = _water_params(2, dt, c0, dx, alpha, beta)
    nx, ny = int(round(width / dx)), int(round(height / dx))
    x = _grid2(nx, ny, 0.0, 0.0, dx)
    n = len(x)
    p_h = 1000.0 * G * (height - x[:, 1])
    real = dict(x=x, mass=np.full(n, 1000.0 * dx * dx), p=p_h,
                rho=tait_density(p_h, c0), c=np.full(n, c0), h=np.full(n, h),
                type=np.full(n, 2, dtype=np.int32))
    walls = _walls_2d(dx, tank_w, tank_h, layers, height, c0, h)
    return _assemble("dam_break_2d", prm, real, walls,
                     dict(dx=dx, c0=c0, h=h, width=width, height=height))


def _walls_2d(dx, tank_w, tank_h, layers, fluid_h, c0, h):
    nxw, nyw = int(round(tank_w / dx)), int(round(tank_h / dx))
    pts = []
    for l in range(1, layers + 1):   # bottom, corners included
        xs = (np.arange(1, nxw + 2 * layers + 1) - 0.5) * dx - layers * dx
        pts.append(np.stack([xs, np.full_like(xs, -(l - 0.5) * dx)], 1))
    ys = (np.arange(1, nyw + 1) - 0.5) * dx
    for l in range(1, layers + 1):   # left and right sides
        pts.append(np.stack([np.full_like(ys, -(l - 0.5) * dx), ys], 1))
        pts.append(np.stack([np.full_like(ys, tank_w + (l - 0.5) * dx), ys], 1))
    x = np.concatenate(pts)
    n = len(x)
    p_w = 1000.0 * G * np.maximum(fluid_h - x[:, 1], 0.0)
    return dict(x=x, mass=np.full(n, 1000.0 * dx * dx), p=p_w, rho=tait_density(p_w, c0),
                c=np.zeros(n), h=np.full(n, h), type=np.full(n, -2, dtype=np.int32))


# ---------------------------------------------------------------------------
# 3-D dam break: block L x W x H = 0.6 x 0.3 x 0.6 m in a 1.6 x 0.6 x 1.0 m box
# (x = length, y = width, z = height)
# ---------------------------------------------------------------------------
def dam_break_3d(dx: float = 0.004, block=(0.6, 0.3, 0.6), box=(1.6, 0.6, 1.0),
                 layers: int = 3, h_factor: float = 1.2, cfl: float = 0.2,
                 alpha: float = 0.1, beta: float = 0.0) -> Case:
    L, W, H = block
    BL, BW, BH = box
    h = h_factor * dx
    c0 = 10.0 * math.sqrt(2.0 * G * H)
    dt = cfl * h / c0
    prm = _water_params(3, dt, c0, dx, alpha, beta)
    nx, ny, nz = (int(round(L / dx)), int(round(W / dx)), int(round(H / dx)))
    x = _grid3(nx, ny, nz, 0.0, 0.0, 0.0, dx)
    n = len(x)
    p_h = 1000.0 * G * (H - x[:, 2])
    real = dict(x=x, mass=np.full(n, 1000.0 * dx ** 3), p=p_h,
                rho=tait_density(p_h, c0), c=np.full(n, c0), h=np.full(n, h),
                type=np.full(n, 2, dtype=np.int32))
    nxw, nyw, nzw = int(round(BL / dx)), int(round(BW / dx)), int(round(BH / dx))
    g = layers
    pts = []
    # bottom (z < 0), corners included
    pts.append(_grid3(nxw + 2 * g, nyw + 2 * g, g, -g * dx, -g * dx, -g * dx, dx))
    # x-walls (x < 0, x > BL), full y incl. corners, z in [0, BH]
    pts.append(_grid3(g, nyw + 2 * g, nzw, -g * dx, -g * dx, 0.0, dx))
    pts.append(_grid3(g, nyw + 2 * g, nzw, BL, -g * dx, 0.0, dx))
    # y-walls (y < 0, y > BW), x in [0, BL]
    pts.append(_grid3(nxw, g, nzw, 0.0, -g * dx, 0.0, dx))
    pts.append(_grid3(nxw, g, nzw, 0.0, BW, 0.0, dx))
    xw = np.concatenate(pts)
    nw = len(xw)
    p_w = 1000.0 * G * np.maximum(H - xw[:, 2], 0.0)
    walls = dict(x=xw, mass=np.full(nw, 1000.0 * dx ** 3), p=p_w,
                 rho=tait_density(p_w, c0), c=np.zeros(nw), h=np.full(nw, h),
                 type=np.full(nw, -2, dtype=np.int32))
    return _assemble("dam_break_3d", prm, real, walls,
                     dict(dx=dx, c0=c0, h=h, block=block, box=box))


def _gate_params(dx, wh, h_factor, cfl, as_eps, E, nu, rho_s):
    """Parameters of gate_2d: water, a linear-elastic solid, AV, artificial
    stress; (params, c0, c_s, h, K, G)."""
    h = h_factor * dx
    c0 = 10.0 * math.sqrt(2.0 * G * wh)
    K = E / (3.0 * (1.0 - 2.0 * nu))
    Gm = E / (2.0 * (1.0 + nu))
    c_s = math.sqrt(K / rho_s)
    dt = cfl * h / max(c0, c_s)
    prm = P.base_params(2, dt)
    # F_FSI_FLUID_VISCOUS: with the reference's viscous coupling (a fluid adds
    # a solid neighbour's shear modulus times its strain rate) this case is
    # unstable at any practical dt; see include/sph_gpu.h
    prm.flags = (P.F_VISCOSITY | P.F_GRAVITY | P.F_ARTI_VISC | P.F_DUMMY |
                 P.F_EXT_FORCE | P.F_ARTI_STRESS | P.F_GRAVITY_SKIP_SOLIDS |
                 P.F_FSI_FLUID_VISCOUS)
    prm.add_material(**P.water(c0))
    prm.add_material(**P.linear_solid(102, rho_s, K, Gm))
    prm.av_alpha, prm.av_beta = 0.1, 0.0
    prm.av_alpha_solid, prm.av_beta_solid = 1.0, 1.0
    prm.wall_fs, prm.wall_r0 = 10.0, dx
    prm.contact_delta = dx
    prm.as_eps, prm.as_n, prm.as_dp = as_eps, 4.0, dx
    return prm, c0, c_s, h, K, Gm


# ---------------------------------------------------------------------------
# 2-D fluid-structure: water 0.2 x 0.4 m held by an elastic gate 0.005 x 0.1 m
# (rubber-like, rho 1100, E 12 MPa, nu 0.4, clamped top edge)
# ---------------------------------------------------------------------------
def gate_2d(dx: float = 5e-4, water=(0.2, 0.4), gate=(0.005, 0.1),
            tank=(0.6, 0.45), layers: int = 3, h_factor: float = 1.2,
            cfl: float = 0.2, as_eps: float = 0.3, E: float = 12e6,
            nu: float = 0.4, rho_s: float = 1100.0) -> Case:
    ww, wh = water
    gw, gh = gate
    tw, th = tank
    prm, c0, c_s, h, K, Gm = _gate_params(dx, wh, h_factor, cfl, as_eps, E, nu, rho_s)
    nx, ny = int(round(ww / dx)), int(round(wh / dx))
    xf = _grid2(nx, ny, 0.0, 0.0, dx)
    nf = len(xf)
    p_h = 1000.0 * G * (wh - xf[:, 1])
    ngx, ngy = int(round(gw / dx)), int(round(gh / dx))
    xs = _grid2(ngx, ngy, ww, 0.0, dx)
    ns = len(xs)
    bnd = np.zeros(nf + ns, dtype=np.int32)
    top = np.isclose(xs[:, 1], (ngy - 0.5) * dx)
    bnd[nf:][top] = 1  # clamped top edge (input.f90:1147-1149)
    real = dict(
        x=np.concatenate([xf, xs]),
        mass=np.concatenate([np.full(nf, 1000.0 * dx * dx), np.full(ns, rho_s * dx * dx)]),
        p=np.concatenate([p_h, np.zeros(ns)]),
        rho=np.concatenate([tait_density(p_h, c0), np.full(ns, rho_s)]),
        c=np.concatenate([np.full(nf, c0), np.full(ns, c_s)]),
        h=np.full(nf + ns, h),
        type=np.concatenate([np.full(nf, 2), np.full(ns, 102)]).astype(np.int32),
        boundary=bnd,
        shear=np.zeros((nf + ns, 4)),
    )
    walls = _walls_2d(dx, tw, th, layers, wh, c0, h)
    # rigid block above the gate up to the tank top ("Middle Wall",
    # dummyParticles.f90:721-741)
    nby = int(round((th - gh) / dx))
    xb = _grid2(ngx, nby, ww, gh, dx)
    nb = len(xb)
    p_b = 1000.0 * G * np.maximum(wh - xb[:, 1], 0.0)
    walls = {k: np.concatenate([walls[k], v]) for k, v in dict(
        x=xb, mass=np.full(nb, 1000.0 * dx * dx), p=p_b, rho=tait_density(p_b, c0),
        c=np.zeros(nb), h=np.full(nb, h), type=np.full(nb, -2, dtype=np.int32)).items()}
    return _assemble("gate_2d", prm, real, walls,
                     dict(dx=dx, c0=c0, c_s=c_s, h=h, K=K, G=Gm, n_fluid=nf, n_solid=ns))


# ---------------------------------------------------------------------------
# 2-D cantilever beam: steel-like, rho 7850, E 200 GPa, nu 0.3, clamped root,
# transverse initial velocity growing linearly to 5 m/s at the tip
# ---------------------------------------------------------------------------
def cantilever_2d(dx: float = 1e-3, length: float = 0.2, thickness: float = 0.02,
                  clamp_cols: int = 3, tip_v: float = 5.0, rho: float = 7850.0,
                  E: float = 200e9, nu: float = 0.3, h_factor: float = 1.2,
                  cfl: float = 0.2) -> Case:
    K = E / (3.0 * (1.0 - 2.0 * nu))
    Gm = E / (2.0 * (1.0 + nu))
    c_s = math.sqrt(K / rho)
    h = h_factor * dx
    dt = cfl * h / c_s
    prm = P.base_params(2, dt)
    prm.flags = P.F_VISCOSITY | P.F_ARTI_VISC | P.F_DUMMY | P.F_EXT_FORCE
    prm.add_material(**P.linear_solid(102, rho, K, Gm))
    prm.av_alpha = prm.av_beta = prm.av_alpha_solid = prm.av_beta_solid = 0.5
    nx, ny = int(round(length / dx)) + clamp_cols, max(int(round(thickness / dx)), 3)
    x = _grid2(nx, ny, -clamp_cols * dx, -0.5 * ny * dx, dx)
    n = len(x)
    v = np.zeros((n, 2))
    v[:, 1] = tip_v * np.clip(x[:, 0], 0.0, None) / length
    bnd = (x[:, 0] < 0).astype(np.int32)
    v[bnd == 1] = 0.0
    real = dict(x=x, v=v, mass=np.full(n, rho * dx * dx), p=np.zeros(n),
                rho=np.full(n, rho), c=np.full(n, c_s), h=np.full(n, h),
                type=np.full(n, 102, dtype=np.int32), boundary=bnd,
                shear=np.zeros((n, 4)))
    walls = dict(x=np.zeros((0, 2)))
    return _assemble("cantilever_2d", prm, real, walls,
                     dict(dx=dx, c_s=c_s, h=h, K=K, G=Gm, length=length))


# ---------------------------------------------------------------------------
# the same cases as lattice blocks generated on the device (sph_block)
# ---------------------------------------------------------------------------
@dataclass
class BlockCase:
    """A case described by lattice blocks (real blocks first); the device
    generates its particles (sph_upload_blocks / sph_batch_add_blocks)."""
    name: str
    params: P.SphParams
    blocks: list
    n_real_blocks: int
    meta: dict = field(default_factory=dict)

    @property
    def dim(self) -> int:
        return int(self.params.dim)

    def counts(self) -> tuple[int, int]:
        nr = nw = 0
        for k, b in enumerate(self.blocks):
            c = 1
            for a in range(self.dim):
                c *= b.n[a]
            if k < self.n_real_blocks:
                nr += c
            else:
                nw += c
        return nr, nw

    @property
    def n_real(self) -> int:
        return self.counts()[0]

    @property
    def n_wall(self) -> int:
        return self.counts()[1]

    @property
    def n(self) -> int:
        return sum(self.counts())

    def array(self):
        arr = (P.SphBlock * len(self.blocks))(*self.blocks)
        return arr


def dam_break_2d_blocks(dx: float = 0.02, width: float = 1.0, height: float = 2.0,
                        tank_w: float = 4.0, tank_h: float = 3.0, layers: int = 3,
                        h_factor: float = 1.2, cfl: float = 0.2, alpha: float = 0.1,
                        beta: float = 0.0) -> BlockCase:
    """dam_break_2d as blocks: the column and the wall layers of _walls_2d,
    in the same particle order, with the same arithmetic."""
    h = h_factor * dx
    c0 = 10.0 * math.sqrt(2.0 * G * height)
    dt = cfl * h / c0
    prm = _water_params(2, dt, c0, dx, alpha, beta)
    nx, ny = int(round(width / dx)), int(round(height / dx))
    tait = (((c0 * c0) * 1000.0) / 7.0, 7.0, 1000.0)
    mass = 1000.0 * dx * dx
    rho_g = 1000.0 * G
    blocks = [P.block((nx, ny), (0.0, 0.0), (dx, dx), mass=mass, h=h, c=c0, type_id=2,
                      p_rho0_g=rho_g, p_level=height, tait=tait)]
    blocks += _walls_2d_blocks(dx, tank_w, tank_h, layers, height, c0, h)
    return BlockCase("dam_break_2d", prm, blocks, 1, dict(dx=dx, c0=c0, h=h, width=width, height=height))


def cantilever_2d_blocks(dx: float = 1e-3, length: float = 0.2, thickness: float = 0.02,
                         clamp_cols: int = 3, tip_v: float = 5.0, rho: float = 7850.0,
                         E: float = 200e9, nu: float = 0.3, h_factor: float = 1.2,
                         cfl: float = 0.2) -> BlockCase:
    """cantilever_2d as one block: clamped columns x < 0, tip velocity ramp."""
    ref = cantilever_2d(dx=dx, length=dx * 4, thickness=dx * 3, clamp_cols=clamp_cols, tip_v=tip_v, rho=rho,
                        E=E, nu=nu, h_factor=h_factor, cfl=cfl)   # parameters only
    prm = ref.params
    c_s, h = ref.meta["c_s"], ref.meta["h"]
    nx, ny = int(round(length / dx)) + clamp_cols, max(int(round(thickness / dx)), 3)
    blocks = [P.block((nx, ny), (-clamp_cols * dx, -0.5 * ny * dx), (dx, dx), mass=rho * dx * dx, h=h, c=c_s,
                      rho=rho, type_id=102, v_ramp=(0.0, tip_v), v_ramp_len=length, clamp_below=0.0)]
    return BlockCase("cantilever_2d", prm, blocks, 1, dict(ref.meta, length=length))


def _walls_2d_blocks(dx, tank_w, tank_h, layers, fluid_h, c0, h) -> list:
    """The wall layers of _walls_2d as blocks, in the same order."""
    nxw, nyw = int(round(tank_w / dx)), int(round(tank_h / dx))
    tait = (((c0 * c0) * 1000.0) / 7.0, 7.0, 1000.0)
    wall = dict(mass=1000.0 * dx * dx, h=h, c=0.0, type_id=-2, p_rho0_g=1000.0 * G, p_level=fluid_h, tait=tait)
    out = []
    for l in range(1, layers + 1):   # bottom, corners included
        out.append(P.block((nxw + 2 * layers, 1), (-(layers * dx), -(l - 0.5) * dx), (dx, 0.0), **wall))
    for l in range(1, layers + 1):   # left and right sides
        out.append(P.block((1, nyw), (-(l - 0.5) * dx, 0.0), (0.0, dx), **wall))
        out.append(P.block((1, nyw), (tank_w + (l - 0.5) * dx, 0.0), (0.0, dx), **wall))
    return out


def dam_break_3d_blocks(dx: float = 0.004, block=(0.6, 0.3, 0.6), box=(1.6, 0.6, 1.0),
                        layers: int = 3, h_factor: float = 1.2, cfl: float = 0.2,
                        alpha: float = 0.1, beta: float = 0.0) -> BlockCase:
    """dam_break_3d as six blocks (the column, the floor and four side walls),
    in the host case's particle order and arithmetic: the bench's 1.69 M
    particle case is a few hundred bytes to upload."""
    L, W, H = block
    BL, BW, BH = box
    h = h_factor * dx
    c0 = 10.0 * math.sqrt(2.0 * G * H)
    dt = cfl * h / c0
    prm = _water_params(3, dt, c0, dx, alpha, beta)
    nx, ny, nz = (int(round(L / dx)), int(round(W / dx)), int(round(H / dx)))
    tait = (((c0 * c0) * 1000.0) / 7.0, 7.0, 1000.0)
    common = dict(mass=1000.0 * dx ** 3, h=h, up_axis=2, p_rho0_g=1000.0 * G, p_level=H, tait=tait)
    sp = (dx, dx, dx)
    blocks = [P.block((nx, ny, nz), (0.0, 0.0, 0.0), sp, c=c0, type_id=2, **common)]
    nxw, nyw, nzw = int(round(BL / dx)), int(round(BW / dx)), int(round(BH / dx))
    g = layers
    wall = dict(common, c=0.0, type_id=-2)
    blocks += [
        P.block((nxw + 2 * g, nyw + 2 * g, g), (-g * dx, -g * dx, -g * dx), sp, **wall),   # floor
        P.block((g, nyw + 2 * g, nzw), (-g * dx, -g * dx, 0.0), sp, **wall),             # x < 0
        P.block((g, nyw + 2 * g, nzw), (BL, -g * dx, 0.0), sp, **wall),                  # x > BL
        P.block((nxw, g, nzw), (0.0, -g * dx, 0.0), sp, **wall),                         # y < 0
        P.block((nxw, g, nzw), (0.0, BW, 0.0), sp, **wall),                              # y > BW
    ]
    return BlockCase("dam_break_3d", prm, blocks, 1, dict(dx=dx, c0=c0, h=h, block=block, box=box))


def gate_2d_blocks(dx: float = 5e-4, water=(0.2, 0.4), gate=(0.005, 0.1),
                   tank=(0.6, 0.45), layers: int = 3, h_factor: float = 1.2,
                   cfl: float = 0.2, as_eps: float = 0.3, E: float = 12e6,
                   nu: float = 0.4, rho_s: float = 1100.0) -> BlockCase:
    """gate_2d as blocks: the water column, the gate with its clamped top row
    (clamp on y), the tank walls and the rigid block above the gate."""
    ww, wh = water
    gw, gh = gate
    tw, th = tank
    prm, c0, c_s, h, K, Gm = _gate_params(dx, wh, h_factor, cfl, as_eps, E, nu, rho_s)
    nx, ny = int(round(ww / dx)), int(round(wh / dx))
    ngx, ngy = int(round(gw / dx)), int(round(gh / dx))
    tait = (((c0 * c0) * 1000.0) / 7.0, 7.0, 1000.0)
    blocks = [
        P.block((nx, ny), (0.0, 0.0), (dx, dx), mass=1000.0 * dx * dx, h=h, c=c0, type_id=2,
                p_rho0_g=1000.0 * G, p_level=wh, tait=tait),
        P.block((ngx, ngy), (ww, 0.0), (dx, dx), mass=rho_s * dx * dx, h=h, c=c_s, rho=rho_s, type_id=102,
                clamp_axis=1, clamp_above=(ngy - 1) * dx),
    ]
    blocks += _walls_2d_blocks(dx, tw, th, layers, wh, c0, h)
    nby = int(round((th - gh) / dx))
    blocks.append(P.block((ngx, nby), (ww, gh), (dx, dx), mass=1000.0 * dx * dx, h=h, c=0.0, type_id=-2,
                          p_rho0_g=1000.0 * G, p_level=wh, tait=tait))
    return BlockCase("gate_2d", prm, blocks, 2,
                     dict(dx=dx, c0=c0, c_s=c_s, h=h, K=K, G=Gm, n_fluid=nx * ny, n_solid=ngx * ngy))


def ensemble_member_blocks(spec: dict, h_factor: float = 1.2, cfl: float = 0.2) -> BlockCase:
    w, hgt, dx = spec["width"], spec["height"], spec["dx"]
    return dam_break_2d_blocks(dx=dx, width=w, height=hgt, tank_w=max(4.0 * w, w + 8 * dx),
                               tank_h=1.5 * hgt, h_factor=h_factor, cfl=cfl)


# ---------------------------------------------------------------------------
# seeded ensemble of 2-D dam breaks (aspect in [0.25, 2], dx in [0.005, 0.02])
# ---------------------------------------------------------------------------
def ensemble_specs(count: int = 256, seed: int = 20261203, n_lo: int = 2000,
                   n_hi: int = 60000) -> list[dict]:
    """Column sizes for a dam-break ensemble.  Draws aspect a ~ U[0.25, 2]
    and a particle count log-uniform in [n_lo, n_hi]; dx follows from the
    count and is clipped to [0.005, 0.02] m (the count is re-derived)."""
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < count:
        a = rng.uniform(0.25, 2.0)
        n_target = math.exp(rng.uniform(math.log(n_lo), math.log(n_hi)))
        dx = rng.uniform(0.005, 0.02)
        # column area fixed by dx and count: n = (w/dx) * (a w/dx)
        w = dx * math.sqrt(n_target / a)
        nx, ny = max(int(round(w / dx)), 4), max(int(round(a * w / dx)), 4)
        if not (n_lo <= nx * ny <= n_hi):
            continue
        out.append(dict(dx=dx, width=nx * dx, height=ny * dx, aspect=a, n=nx * ny))
    return out


def ensemble_member(spec: dict, h_factor: float = 1.2, cfl: float = 0.2) -> Case:
    w, hgt, dx = spec["width"], spec["height"], spec["dx"]
    return dam_break_2d(dx=dx, width=w, height=hgt, tank_w=max(4.0 * w, w + 8 * dx),
                        tank_h=1.5 * hgt, h_factor=h_factor, cfl=cfl)


# ---------------------------------------------------------------------------
# reference-native presets
# ---------------------------------------------------------------------------
def reference_dam_break(dt: float = 1e-3) -> Case:
    """nick 'dam_break': input.f90:1031-1088 and dummyParticles.f90:544-659
    (125 x 125 column of dx = 0.2 (single-precision literal), c = 50, h = dx,
    4 wall layers, baffle and lid)."""
    dx = P.f32(0.2)
    nx = ny = int(25.0 / dx)
    x = _grid2(nx, ny, 0.0, 0.0, dx)
    n = len(x)
    prm = P.reference_preset("dam_break", 2, dt)
    prm.flags = P.F_VISCOSITY | P.F_GRAVITY | P.F_ARTI_VISC | P.F_DUMMY | P.F_EXT_FORCE
    p_h = 1000.0 * P.f32(9.81) * (25.0 - x[:, 1])
    real = dict(x=x, mass=np.full(n, 1000.0 * dx * dx), p=p_h, rho=tait_density(p_h, 50.0),
                c=np.full(n, 50.0), h=np.full(n, dx), type=np.full(n, 2, dtype=np.int32))
    # r0 = |P(2)%x(1) - P(2)%x(2)| (externalForce.f90:86)
    prm.wall_r0 = abs(x[1, 0] - x[1, 1])
    wdx = abs(x[1, 0] - x[1, 1])  # dummyParticles.f90:562
    wd = [0.0, 100.0, 0.0, 40.0]
    layer = 4
    pts, rho_w, p_w, m_w = [], [], [], []

    def add(px, py, dens, pres, mass, inverse):
        px = np.atleast_1d(px).astype(float)
        py = np.atleast_1d(py).astype(float) * np.ones_like(px)
        pts.append(np.stack([px, py], 1))
        pres = np.broadcast_to(pres, px.shape).astype(float)
        rho_w.append(tait_density(pres, 50.0) if inverse else np.full(px.shape, dens))
        p_w.append(pres if inverse else np.zeros(px.shape))
        m_w.append(np.full(px.shape, mass))

    for l in range(1, layer + 1):
        Nyw = int(math.floor((wd[3] - wd[2]) / wdx)) + layer
        i = np.arange(1, Nyw + 1)
        yy = wd[2] + (i - layer - 0.5) * wdx
        pr = 1000.0 * P.f32(9.81) * np.maximum(25.0 - yy, 0.0)
        add(np.full(Nyw, wd[0] - (l - 0.5) * wdx), yy, 1000.0, pr, 1000.0 * wdx * wdx, True)
        add(np.full(Nyw, wd[1] + (l - 0.5) * wdx), yy, 1000.0, pr, 1000.0 * wdx * wdx, True)
        Nxw = int(math.floor((wd[1] - wd[0]) / wdx)) + 1
        i = np.arange(1, Nxw + 1)
        add(wd[0] + (i - 0.5) * wdx, wd[2] - (l - 0.5) * wdx, 1000.0, 0.0, 1000.0 * wdx * wdx, False)
    Nb = int(math.floor(3 / (wdx / 2)))
    for l in range(1, layer + 1):
        i = np.arange(1, Nb - l + 2)
        xx = (wd[0] + wd[1]) / 2 + (i + l - 1.5) * wdx / 2
        yy = wd[2] + (i - 0.5) * wdx / 2
        pr = 1000.0 * P.f32(9.81) * np.maximum(25.0 - yy, 0.0)
        add(xx, yy, 1000.0, pr, 1000.0 * wdx * wdx / 4, True)
    Nl = int(math.floor((wd[1] - wd[0]) / wdx)) + 1
    for l in range(1, layer + 1):
        i = np.arange(1, Nl + 1)
        add(wd[0] + (i - 0.5) * wdx, wd[3] - (l + 0.5) * wdx, 1000.0, 0.0, 1000.0 * wdx * wdx, False)
    xw = np.concatenate(pts)
    nw = len(xw)
    walls = dict(x=xw, mass=np.concatenate(m_w), p=np.concatenate(p_w),
                 rho=np.concatenate(rho_w), c=np.zeros(nw), h=np.full(nw, wdx),
                 type=np.full(nw, -2, dtype=np.int32))
    return _assemble("reference_dam_break", prm, real, walls, dict(dx=dx, c0=50.0, h=dx))


def reference_can_beam(dt: float = 2e-6) -> Case:
    """nick 'can_beam' (input.f90:1336-1366): 101 x 5 particles of type 102,
    dx = 1e-3, h = 2 dx, clamped first column; gravity-loaded as
    data/cantileverBeam/sph.toml (without kernelCorrection)."""
    dx = P.f32(1e-3)
    nx, ny = 101, 5
    I, J = np.meshgrid(np.arange(1, nx + 1), np.arange(1, ny + 1), indexing="ij")
    x = np.stack([(I.ravel() - 1) * dx, (J.ravel() - 1 - ny // 2) * dx], 1)
    n = len(x)
    c = math.sqrt(P.f32(2e7) / 1100.0)
    prm = P.reference_preset("can_beam", 2, dt)
    prm.flags = P.F_VISCOSITY | P.F_GRAVITY | P.F_ARTI_VISC | P.F_DUMMY | P.F_EXT_FORCE
    bnd = (I.ravel() == 1).astype(np.int32)
    real = dict(x=x, mass=np.full(n, 1100.0 * dx ** 2), p=np.zeros(n), rho=np.full(n, 1100.0),
                c=np.full(n, c), h=np.full(n, dx * 2), type=np.full(n, 102, dtype=np.int32),
                boundary=bnd, shear=np.zeros((n, 4)))
    return _assemble("reference_can_beam", prm, real, dict(x=np.zeros((0, 2))),
                     dict(dx=dx, c_s=c, h=2 * dx))


def reference_can_beam_3d(dt: float = 2e-6) -> Case:
    """nick 'can_beam_3d' (input.f90:1368-1405): 201 x 5 x 9 particles of type
    102, dx = 5e-4 (single-precision literal), h = 2 dx, clamped first layer
    (i = 1), c = sqrt(K / rho0); no dummy particles for this nick
    (dummyParticles.f90:9-45)."""
    dx = P.f32(5e-4)
    nx, ny, nz = 201, 5, 9
    I, J, K = np.meshgrid(np.arange(1, nx + 1), np.arange(1, ny + 1), np.arange(1, nz + 1), indexing="ij")
    x = np.stack([(I.ravel() - 1) * dx, (J.ravel() - 1 - ny // 2) * dx, (K.ravel() - 1 - nz // 2) * dx], 1)
    n = len(x)
    rho0 = 1100.0
    c = math.sqrt(P.f32(2e7) / rho0)
    prm = P.reference_preset("can_beam_3d", 3, dt)
    prm.flags = P.F_VISCOSITY | P.F_GRAVITY | P.F_ARTI_VISC | P.F_DUMMY | P.F_EXT_FORCE
    bnd = (I.ravel() == 1).astype(np.int32)
    mass = rho0 * ((dx * dx) * dx)   # Density * dx**3, expanded as gfortran does
    real = dict(x=x, mass=np.full(n, mass), p=np.zeros(n), rho=np.full(n, rho0),
                c=np.full(n, c), h=np.full(n, dx * 2), type=np.full(n, 102, dtype=np.int32),
                boundary=bnd, shear=np.zeros((n, 9)))
    return _assemble("reference_can_beam_3d", prm, real, dict(x=np.zeros((0, 3))),
                     dict(dx=dx, c_s=c, h=2 * dx))


def _rect(center, length, dx, ex=(1, 1), off=(0.5, 0.5)):
    """A rectangle_t lattice of the reference's generators: nx = int(l_x / dx)
    + ex_x (likewise y), x = (center - length / 2) + (i - off_x, j - off_y) dx
    for i = 1..nx (outer), j = 1..ny, with the single-precision literals of
    the Fortran source (input.f90, dummyParticles.f90)."""
    c = [P.f32(v) for v in center]
    l = [P.f32(v) for v in length]
    nx, ny = int(l[0] / dx) + ex[0], int(l[1] / dx) + ex[1]
    I, J = np.meshgrid(np.arange(1, nx + 1), np.arange(1, ny + 1), indexing="ij")
    x0, y0 = c[0] - l[0] / 2, c[1] - l[1] / 2
    return np.stack([x0 + (I.ravel() - off[0]) * dx, y0 + (J.ravel() - off[1]) * dx], 1), J.ravel(), ny


def reference_water_impact(dt: float = 5e-6) -> Case:
    """nick 'water_impact': a water column (input.f90:1156-1191, c = 10,
    hydrostatic pressure with the inverse Tait EOS) released onto an elastic
    plate of type 103 (:1193-1217, h = 1.2 dx, bottom row clamped), in a
    closed box of six wall blocks (dummyParticles.f90:767-913)."""
    dx = P.f32(0.002)
    h = P.f32(0.292)
    g = 1000.0 * P.f32(9.81)
    xf, _, _ = _rect((0.073, 0.146), (0.146, 0.292), dx)
    nf = len(xf)
    p_f = g * np.maximum(h - xf[:, 1], 0.0)
    xs, js, _ = _rect((0.292, 0.04), (0.012, 0.08), dx)
    ns = len(xs)
    real = dict(
        x=np.concatenate([xf, xs]),
        mass=np.concatenate([np.full(nf, 1000.0 * dx * dx), np.full(ns, 2500.0 * dx * dx)]),
        p=np.concatenate([p_f, np.zeros(ns)]),
        rho=np.concatenate([tait_density(p_f, 10.0), np.full(ns, 2500.0)]),
        c=np.concatenate([np.full(nf, 10.0), np.full(ns, P.f32(11.489))]),
        h=np.concatenate([np.full(nf, dx), np.full(ns, dx * P.f32(1.2))]),
        type=np.concatenate([np.full(nf, 2), np.full(ns, 103)]).astype(np.int32),
        boundary=np.concatenate([np.zeros(nf), (js == 1).astype(float)]).astype(np.int32),
        shear=np.zeros((nf + ns, 4)),
    )
    blocks = [((-0.006, 0.183), (0.012, 0.366)), ((0.292, -0.006), (0.630, 0.012)),
              ((0.59, 0.183), (0.012, 0.366)), ((0.292, 0.600), (0.630, 0.012)),
              ((-0.029, 0.297), (0.012, 0.618)), ((0.613, 0.297), (0.012, 0.618))]
    xw = np.concatenate([_rect(cc, ll, dx)[0] for cc, ll in blocks])
    nw = len(xw)
    walls = dict(x=xw, mass=np.full(nw, 1000.0 * dx * dx), p=np.zeros(nw), rho=np.full(nw, 1000.0),
                 c=np.zeros(nw), h=np.full(nw, dx), type=np.full(nw, -2, dtype=np.int32))
    prm = P.reference_preset("water_impact", 2, dt)
    prm.flags |= P.F_VISCOSITY | P.F_GRAVITY | P.F_ARTI_VISC | P.F_DUMMY | P.F_EXT_FORCE
    return _assemble("reference_water_impact", prm, real, walls, dict(dx=dx, c0=10.0, h=dx))


CONFIGS = {
    "dam_break_2d": dam_break_2d,
    "dam_break_3d": dam_break_3d,
    "gate_2d": gate_2d,
    "cantilever_2d": cantilever_2d,
    "reference_dam_break": reference_dam_break,
    "reference_can_beam": reference_can_beam,
    "reference_can_beam_3d": reference_can_beam_3d,
    "reference_water_impact": reference_water_impact,
}
