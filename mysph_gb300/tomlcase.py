"""Case input from the reference's `sph.toml` (getValueFromToml.f90:80-185).

A mySPH project directory holds one `sph.toml`: the project `name` and
`nick`, a `[Parameter]` table of switches and sizes, `[Parallel]` and
`[postProcess]`.  This module reads the same keys with the same defaults,
maps the switches onto `sph_params` flags, builds the nick's particle set
(the reference-native generators in `cases.py`) and runs it on the GPU with
the reference's print cadence:

    python -m mysph_gb300.tomlcase path/to/sph.toml [--steps N] [--precision mixed|df64]

Options the GPU path does not implement (openBoundary, shifting,
readInitialFile, dpInput, SLE > 2, SPH = 4, DIM = 1) raise
UnsupportedOption unless `allow_unsupported` drops them with a warning.
kernelCorrection maps to SPH_F_KERNEL_CORRECTION (FP64, solid cases) and
artificialHeat to SPH_F_ARTI_HEAT (FP64).
"""
from __future__ import annotations

import argparse
import sys
import time
import tomllib
import warnings
from dataclasses import dataclass, field
from pathlib import Path

from . import cases
from . import params as P


class UnsupportedOption(ValueError):
    """An sph.toml switch the GPU path does not implement."""


@dataclass
class TomlConfig:
    """The values get_details_from_sph_toml reads, with its defaults
    (getValueFromToml.f90:108-163, 181-183)."""
    name: str = "untitled"
    nick: str = "unknown"
    dim: int = 0
    maxn: int = 5000
    ntotal: int | None = None
    kpair: int = 20
    pa_sph: int = 2
    nnps: int = 1
    skf: int = 1
    sle: int = 0
    monitor_particle: int = 1
    print_interval: int = 100
    save_interval: int = 500
    delta_t: float = P.f32(5e-4)   # dble(5e-4): a single-precision literal
    max_time_step: int = 1000
    print_statistics: bool = True
    sum_density: bool = True
    aver_velocity: bool = False
    read_ini_file: bool = False
    dummy_particle: bool = False
    dp_input: bool = False
    viscosity: bool = False
    ex_force: bool = False
    gravity: bool = False
    arti_visc: bool = False
    arti_heat: bool = False
    norm_density: bool = False
    open_boundary: bool = False
    kernel_correction: bool = False
    shifting: bool = False
    arti_stress: bool = False
    nthreads: int = 0
    write_dp: bool = True
    write_vtk: bool = True
    write_dp_vtk: bool = True
    source: str = ""
    extra: dict = field(default_factory=dict)


# [Parameter] key -> (attribute, type)
_PARAMETER_KEYS = {
    "DIM": ("dim", int), "maxN": ("maxn", int), "ntotal": ("ntotal", int), "kPair": ("kpair", int),
    "SPH": ("pa_sph", int), "NNPS": ("nnps", int), "SKF": ("skf", int), "SLE": ("sle", int),
    "monitorParticle": ("monitor_particle", int), "printInterval": ("print_interval", int),
    "saveInterval": ("save_interval", int), "deltaT": ("delta_t", float),
    "maxTimeStep": ("max_time_step", int), "printStatistics": ("print_statistics", bool),
    "summationDensity": ("sum_density", bool), "averageVelocity": ("aver_velocity", bool),
    "readInitialFile": ("read_ini_file", bool), "dummyParticle": ("dummy_particle", bool),
    "dpInput": ("dp_input", bool), "viscosity": ("viscosity", bool),
    "externalForce": ("ex_force", bool), "gravity": ("gravity", bool),
    "artificialViscosity": ("arti_visc", bool), "artificialHeat": ("arti_heat", bool),
    "normalizeDensity": ("norm_density", bool), "openBoundary": ("open_boundary", bool),
    "kernelCorrection": ("kernel_correction", bool), "shifting": ("shifting", bool),
    "artificialStress": ("arti_stress", bool),
}
_POST_KEYS = {"writeDummyParticle": "write_dp", "writeVTKfile": "write_vtk",
              "writeDummyParticle2VTK": "write_dp_vtk"}


def parse(src: str | Path) -> TomlConfig:
    """Read an sph.toml file (or its text)."""
    p = Path(src) if not isinstance(src, str) or "\n" not in src else None
    text = p.read_text(encoding="utf-8") if p is not None else src
    doc = tomllib.loads(text)
    cfg = TomlConfig(source=str(p) if p is not None else "<string>")
    cfg.name = str(doc.get("name", cfg.name))
    cfg.nick = str(doc.get("nick", cfg.nick))
    par = doc.get("Parameter", {})
    for key, val in par.items():
        if key in _PARAMETER_KEYS:
            attr, typ = _PARAMETER_KEYS[key]
            if typ is bool and not isinstance(val, bool):
                raise ValueError(f"{key} must be true or false")
            setattr(cfg, attr, typ(val))
        else:
            cfg.extra[key] = val
    if "DIM" not in par:
        raise ValueError("[Parameter] DIM is required")
    # dummy particles or gravity switch the external force on (:152-154)
    if cfg.dummy_particle or cfg.gravity:
        cfg.ex_force = True
    cfg.nthreads = int(doc.get("Parallel", {}).get("OMP_NUM_THREADS", 0))
    for key, attr in _POST_KEYS.items():
        if key in doc.get("postProcess", {}):
            setattr(cfg, attr, bool(doc["postProcess"][key]))
    return cfg


def unsupported(cfg: TomlConfig) -> list[str]:
    """Switches of this configuration that the GPU path does not implement."""
    out = []
    for attr, key in (("open_boundary", "openBoundary"),
                      ("shifting", "shifting"),
                      ("read_ini_file", "readInitialFile"), ("dp_input", "dpInput")):
        if getattr(cfg, attr):
            out.append(key)
    if cfg.sle not in (0, 1, 2):
        out.append(f"SLE = {cfg.sle}")
    if cfg.pa_sph not in (1, 2, 3):
        # SPH = 4 (sum_density_dsph) has no internal-force form in the
        # reference: internal_force stops on it (internalForce.f90:326-328)
        out.append(f"SPH = {cfg.pa_sph}")
    if cfg.dim not in (2, 3):
        out.append(f"DIM = {cfg.dim}")
    return out


def flags(cfg: TomlConfig) -> int:
    f = 0
    for attr, bit in (("sum_density", P.F_SUM_DENSITY), ("norm_density", P.F_NORM_DENSITY),
                      ("viscosity", P.F_VISCOSITY), ("gravity", P.F_GRAVITY),
                      ("ex_force", P.F_EXT_FORCE), ("arti_visc", P.F_ARTI_VISC),
                      ("arti_stress", P.F_ARTI_STRESS), ("aver_velocity", P.F_AVER_VELOCITY),
                      ("dummy_particle", P.F_DUMMY), ("kernel_correction", P.F_KERNEL_CORRECTION),
                      ("arti_heat", P.F_ARTI_HEAT)):
        if getattr(cfg, attr):
            f |= bit
    return f


# nick -> generator of the reference-native particle set
_GENERATORS = {
    "dam_break": lambda cfg: cases.reference_dam_break(dt=cfg.delta_t),
    "can_beam": lambda cfg: cases.reference_can_beam(dt=cfg.delta_t),
    "can_beam_3d": lambda cfg: cases.reference_can_beam_3d(dt=cfg.delta_t),
    "water_impact": lambda cfg: cases.reference_water_impact(dt=cfg.delta_t),
}


def build_case(cfg: TomlConfig, allow_unsupported: bool = False, precision: int = P.PREC_FP64):
    """The nick's particles with the parameters of this sph.toml."""
    bad = unsupported(cfg)
    if bad:
        if not allow_unsupported:
            raise UnsupportedOption(f"{cfg.source}: not implemented on the GPU path: {', '.join(bad)}")
        warnings.warn(f"ignoring options the GPU path does not implement: {', '.join(bad)}")
    if cfg.nick not in _GENERATORS:
        raise ValueError(f"no particle generator for nick {cfg.nick!r} (have: {', '.join(sorted(_GENERATORS))})")
    case = _GENERATORS[cfg.nick](cfg)
    if case.dim != cfg.dim:
        raise ValueError(f"nick {cfg.nick!r} is a {case.dim}-D case, sph.toml says DIM = {cfg.dim}")
    prm = case.params.copy()
    keep = prm.flags & (P.F_GRAVITY_SKIP_SOLIDS | P.F_FSI_FLUID_VISCOUS)   # nick-level flags
    prm.flags = flags(cfg) | keep
    prm.dt = cfg.delta_t
    prm.skf = cfg.skf
    prm.pa_sph = cfg.pa_sph
    prm.sle = cfg.sle
    prm.precision = precision
    case.params = prm
    if cfg.maxn < case.n:
        warnings.warn(f"maxN = {cfg.maxn} is below the {case.n} particles of nick {cfg.nick!r}; "
                      "the device context is sized to the particles")
    return case


def run(src, steps: int | None = None, precision: int = P.PREC_FP64, allow_unsupported: bool = False,
        out=print, out_dir=None, dat_dir=None, binary: bool = False) -> dict:
    """Advance the case of an sph.toml for maxTimeStep steps (or `steps`),
    printing the step, time, Courant numbers and neighbour statistics every
    printInterval steps as the reference's time_integration does.  With
    `out_dir`, VTK snapshots are written at step 0 and every saveInterval
    steps (walls included when writeDummyParticle2VTK is set; BINARY with
    `binary`), and with `dat_dir` the `.dat` files beside them."""
    from .output import SnapshotWriter
    from .solver import GpuSolver
    cfg = parse(src)
    case = build_case(cfg, allow_unsupported, precision)
    total = int(steps if steps is not None else cfg.max_time_step)
    pi, si = max(cfg.print_interval, 1), max(cfg.save_interval, 1)
    t0 = time.perf_counter()
    writer = None
    with GpuSolver(case) as s:
        if out_dir is not None:
            writer = SnapshotWriter(out_dir, case.dim, case.state, case.boundary, with_walls=cfg.write_dp_vtk,
                                    dat_dir=dat_dir, binary=binary)
            writer.snapshot(s, 0, case.n_real)
        done = 0
        mx = mean = 0.0
        while done < total:
            nxt = min((done // pi + 1) * pi, (done // si + 1) * si if writer else total, total)
            mx, mean = s.advance(nxt - done)
            done = nxt
            if out and cfg.print_statistics and done % pi == 0:
                st = s.statistics()
                out(f"step {done:>8d}  t = {s.info()['time']:.6e}  courant max {mx:.4f} mean {mean:.4f}  "
                    f"neighbours max {st['max']} min {st['min']} mean {st['mean']:.2f}")
            if writer and done % si == 0:
                writer.snapshot(s, done, case.n_real)
        info = s.info()
        fields = {k: s.field(k)[: case.n_real] for k in ("X", "V", "RHO", "P")}
    files = writer.close() if writer else []
    wall = time.perf_counter() - t0
    return {"name": cfg.name, "nick": cfg.nick, "steps": total, "time": info["time"],
            "n_real": case.n_real, "n_wall": case.n_wall, "max_courant": mx, "mean_courant": mean,
            "wall_s": wall, "fields": fields, "files": files}


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("toml")
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--precision", choices=["fp64", "mixed", "df64"], default="fp64")
    ap.add_argument("--allow-unsupported", action="store_true")
    ap.add_argument("--out", default=None, help="directory for VTK snapshots every saveInterval steps")
    ap.add_argument("--dat", default=None, help="directory for the .dat files of the same snapshots")
    ap.add_argument("--binary", action="store_true", help="legacy VTK in BINARY form")
    a = ap.parse_args(argv)
    if (a.dat or a.binary) and not a.out:
        ap.error("--dat and --binary write beside the VTK snapshots: give --out as well")
    prec = {"fp64": P.PREC_FP64, "mixed": P.PREC_MIXED, "df64": P.PREC_DF64}[a.precision]
    try:
        r = run(a.toml, a.steps, prec, a.allow_unsupported, out_dir=a.out, dat_dir=a.dat, binary=a.binary)
    except (UnsupportedOption, ValueError) as ex:
        print(f"error: {ex}", file=sys.stderr)
        return 2
    print(f"{r['name']}: {r['steps']} steps, t = {r['time']:.6e} s, {r['n_real']} real + {r['n_wall']} wall "
          f"particles, {r['wall_s']:.2f} s")
    return 0


if __name__ == "__main__":
    sys.exit(main())
