"""Host-side mirror of the reference's module interface over libsphgpu.

The Fortran reference exposes module procedures that take `type(Particle)`
arrays and mutate them in place; this class keeps their names and argument
meaning on top of the C ABI:

  BGGS(Targets, Sources, skipItsSelf)   -> nnps()/neighbor_lists()
                                           (src/NNPS/asymmetricSearch.f90:160)
  con_density(ntotal, P, drhodt)        -> con_density()   (density.f90:83)
  divergence(ntotal, P)                 -> divergence()    (divergence.f90:6)
  internal_force(ntotal, P, dvdt, ...)  -> internal_force() (internalForce.f90:10)
  external_force(ntotal, P, dvdt)       -> external_force() (externalForce.f90:7)
  arti_visc(ntotal, P, dvdt, dedt)      -> arti_visc()     (artificialViscosity.f90:7)
  artificialStress(ntotal, P, dvdt)     -> artificial_stress() (artificialTerm.f90:7)
  single_step(...)                      -> rates()         (singleStep.f90:1)
  leap_frog(ntotal, P) one iteration    -> single_step()   (timeIntegration.f90:85)
  time_integration(ntotal, P)           -> advance(nsteps)
  print_statistics(Particles)           -> statistics()    (nnps.f90:377)

Errors raise SphError instead of the reference's `error stop`.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import params as P
from ._lib import SphError, dp, i64p, ip, load


def _dp(a):
    return None if a is None else a.ctypes.data_as(dp)


class GpuSolver:
    """One particle system resident on the current CUDA device."""

    def __init__(self, case, params: P.SphParams | None = None, capacity: int | None = None):
        self.lib = load()
        self.prm = (params or case.params).copy()
        self.dim = int(self.prm.dim)
        self.ctx = C.c_void_p()
        cap = int(capacity or case.n)
        self._call("sph_create", C.byref(self.prm), cap, C.byref(self.ctx), ctx=False)
        self.case = case
        self.upload(case)

    # -- plumbing ----------------------------------------------------------
    def _call(self, name: str, *args, ctx: bool = True):
        f = getattr(self.lib, name)
        st = f(self.ctx, *args) if ctx else f(*args)
        if st != 0:
            msg = ""
            if ctx and self.ctx:
                buf = C.create_string_buffer(512)
                self.lib.sph_status(self.ctx, buf, 512)
                msg = buf.value.decode(errors="replace")
            raise SphError(st, name, msg)
        return st

    def close(self) -> None:
        if getattr(self, "ctx", None) and self.ctx:
            self.lib.sph_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- data in / out -------------------------------------------------------
    def upload(self, case) -> None:
        x, v, m, rho, p, e, c, h, t, s, b, sh = case.arrays()
        self._keep = (x, v, m, rho, p, e, c, h, t, s, b, sh)
        self._call("sph_upload", case.n_real, case.n_wall, _dp(x), _dp(v), _dp(m), _dp(rho),
                   _dp(p), _dp(e), _dp(c), _dp(h), t.ctypes.data_as(ip), s.ctypes.data_as(ip),
                   b.ctypes.data_as(ip), _dp(sh))
        self.n_real, self.n_wall, self.n = case.n_real, case.n_wall, case.n

    def field(self, name: str) -> np.ndarray:
        comp = {"v": self.dim, "t": self.dim * self.dim, "s": 1}[P.FIELD_SHAPE[name]]
        out = np.empty(self.n * comp)
        self._call("sph_get_field", P.FIELD[name], _dp(out))
        return out.reshape(self.n, comp) if comp > 1 else out

    def set_field(self, name: str, values: np.ndarray) -> None:
        a = np.ascontiguousarray(values, dtype=np.float64)
        self._call("sph_set_field", P.FIELD[name], _dp(a))

    def info(self):
        nr, nw, st = C.c_int64(), C.c_int64(), C.c_int64()
        t = C.c_double()
        self._call("sph_info", C.byref(nr), C.byref(nw), C.byref(st), C.byref(t))
        return dict(n_real=nr.value, n_wall=nw.value, step=st.value, time=t.value)

    # -- NNPS ---------------------------------------------------------------
    def nnps(self) -> None:
        self._call("sph_nnps")

    def neighbor_counts(self) -> np.ndarray:
        cnt = np.zeros(self.n_real, dtype=np.int32)
        tot = C.c_int64()
        self._call("sph_neighbor_counts", cnt.ctypes.data_as(ip), C.byref(tot))
        return cnt

    def neighbor_lists(self):
        """CSR (offsets, 1-based neighbour indices) of the last nnps()."""
        tot = C.c_int64()
        self._call("sph_neighbor_counts", None, C.byref(tot))
        off = np.zeros(self.n_real + 1, dtype=np.int64)
        lst = np.zeros(max(tot.value, 1), dtype=np.int32)
        self._call("sph_export_neighbors", off.ctypes.data_as(i64p), lst.ctypes.data_as(ip), tot.value)
        return off, lst[:tot.value]

    def statistics(self) -> dict:
        out = np.zeros(6)
        self._call("sph_statistics", _dp(out))
        return dict(max=int(out[0]), min=int(out[1]), mean=float(out[2]), no_neighbors=int(out[3]),
                    argmax=int(out[4]), argmin=int(out[5]))

    def boundary(self, dvdt: np.ndarray | None = None) -> np.ndarray | None:
        """fixedBoundary (boundaryCondition.f90:32-45): zero the velocity rate
        where Boundary == 1, in `dvdt` (n_real x dim, upload order; a copy is
        returned) and in the context's assembled rates."""
        if dvdt is None:
            self._call("sph_boundary", None)
            return None
        out = np.ascontiguousarray(dvdt, dtype=np.float64).copy()
        self._call("sph_boundary", _dp(out))
        return out

    def courant_num(self, hsml, div_v, c) -> np.ndarray:
        """courant_num (courantNumber.f90:7-31) elementwise, with this
        context's deltaT and Courant alpha / beta."""
        h = np.ascontiguousarray(hsml, dtype=np.float64)
        dv = np.ascontiguousarray(div_v, dtype=np.float64)
        cc = np.ascontiguousarray(c, dtype=np.float64)
        if not (h.shape == dv.shape == cc.shape):
            raise ValueError("hsml, div_v and c must have one shape")
        xi = np.empty_like(h)
        self._call("sph_courant_num", h.size, _dp(h), _dp(dv), _dp(cc), _dp(xi))
        return xi

    # -- modules (rates on the current state) ---------------------------------
    def con_density(self) -> np.ndarray:
        out = np.zeros(self.n_real)
        self._call("sph_density", _dp(out))
        return out

    def divergence(self):
        dx, dv = np.zeros(self.n_real), np.zeros(self.n_real)
        self._call("sph_divergence", _dp(dx), _dp(dv))
        return dx, dv

    def internal_force(self):
        a = np.zeros((self.n_real, self.dim))
        e = np.zeros(self.n_real)
        s = np.zeros((self.n_real, self.dim * self.dim))
        self._call("sph_internal_force", _dp(a), _dp(e), _dp(s))
        return a, e, s

    def external_force(self) -> np.ndarray:
        a = np.zeros((self.n_real, self.dim))
        self._call("sph_external_force", _dp(a))
        return a

    def arti_visc(self):
        a = np.zeros((self.n_real, self.dim))
        e = np.zeros(self.n_real)
        self._call("sph_arti_visc", _dp(a), _dp(e))
        return a, e

    def artificial_stress(self) -> np.ndarray:
        a = np.zeros((self.n_real, self.dim))
        self._call("sph_arti_stress", _dp(a))
        return a

    def energy(self, inst: int = -1) -> dict:
        """FP64 energy sums of the real particles (sph_energy)."""
        out = np.zeros(4)
        self._call("sph_energy", int(inst), _dp(out))
        return dict(kinetic=out[0], internal=out[1], gravitational=out[2], total=out[3])

    def arti_heat(self) -> np.ndarray:
        """arti_heat (artificialHeat.f90:6-56): the artificial-heat energy rate."""
        e = np.zeros(self.n_real)
        self._call("sph_arti_heat", _dp(e))
        return e

    def rates(self):
        a = np.zeros((self.n_real, self.dim))
        r = np.zeros(self.n_real)
        e = np.zeros(self.n_real)
        self._call("sph_rates", _dp(a), _dp(r), _dp(e))
        return a, r, e

    # -- time integration -----------------------------------------------------
    def single_step(self) -> None:
        self._call("sph_single_step")

    def advance(self, nsteps: int):
        mx, mean = C.c_double(), C.c_double()
        self._call("sph_advance", int(nsteps), C.byref(mx), C.byref(mean))
        return mx.value, mean.value

    def advance_async(self, nsteps: int) -> None:
        """Queue nsteps steps on the context's stream (sph_advance_async)."""
        self._call("sph_advance_async", int(nsteps))

    def sync(self):
        """Wait for the queued steps; their status and last Courant numbers."""
        mx, mean = C.c_double(), C.c_double()
        self._call("sph_sync", C.byref(mx), C.byref(mean))
        return mx.value, mean.value

    # -- measurement ----------------------------------------------------------
    def stream(self) -> int:
        s = C.c_void_p()
        self._call("sph_get_stream", C.byref(s))
        return s.value or 0

    def enable_stage_timing(self, on: bool = True) -> None:
        self._call("sph_enable_stage_timing", int(on))

    def stage_times(self):
        ms = np.zeros(len(P.STAGES))
        n = C.c_int64()
        self._call("sph_stage_times", _dp(ms), C.byref(n))
        return dict(zip(P.STAGES, ms.tolist())), n.value

    def set_option(self, option: int, value: float) -> None:
        self._call("sph_set_option", int(option), float(value))

    def tune_lanes(self, steps: int = 30, choices=(1, 2, 4, 8, 16)) -> int:
        """Time `steps` steps at each lanes-per-target setting (SPH_OPT_LANES)
        on a copy of the current state, set the fastest on this context and
        return it.  The context's own state does not move.  Worth it for small
        systems (a few thousand particles); large ones keep 1."""
        import torch
        blob = self.save_state()
        best, best_ms = 1, None
        for lanes in choices:
            probe = type(self).from_state(blob)
            try:
                probe.set_option(P.OPT_LANES, lanes)
                probe.advance(3)   # first launches and the graph capture
                stream = torch.cuda.ExternalStream(probe.stream())
                torch.cuda.synchronize()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                probe.advance(steps)
                e1.record(stream)
                torch.cuda.synchronize()
                ms = e0.elapsed_time(e1)
            finally:
                probe.close()
            if best_ms is None or ms < best_ms:
                best, best_ms = lanes, ms
        self.set_option(P.OPT_LANES, best)
        return best

    def launch_count(self) -> int:
        n = C.c_int64()
        self._call("sph_launch_count", C.byref(n))
        return n.value

    def device_bytes(self) -> int:
        n = C.c_int64()
        self._call("sph_device_bytes", C.byref(n))
        return n.value

    # -- device-generated cases ----------------------------------------------------
    @classmethod
    def from_blocks(cls, bc, params: P.SphParams | None = None, capacity: int | None = None):
        """A context whose particles the device generates (sph_upload_blocks)."""
        self = cls.__new__(cls)
        self.lib = load()
        self.prm = (params or bc.params).copy()
        self.dim = int(self.prm.dim)
        self.ctx = C.c_void_p()
        self._call("sph_create", C.byref(self.prm), int(capacity or bc.n), C.byref(self.ctx), ctx=False)
        self.case = None
        arr = bc.array()
        self._call("sph_upload_blocks", len(bc.blocks), arr, bc.n_real_blocks)
        self.n_real, self.n_wall = bc.counts()
        self.n = self.n_real + self.n_wall
        return self

    # -- state snapshots ---------------------------------------------------------
    def save_state(self) -> bytes:
        """The full state of the context between steps (sph_state_save)."""
        n = C.c_int64()
        self._call("sph_state_bytes", C.byref(n))
        buf = C.create_string_buffer(n.value)
        self._call("sph_state_save", C.cast(buf, C.c_void_p), n.value)
        return buf.raw

    @classmethod
    def from_state(cls, blob: bytes):
        """A new context resumed from save_state() (sph_state_load)."""
        self = cls.__new__(cls)
        self.lib = load()
        self.ctx = C.c_void_p()
        buf = C.create_string_buffer(blob, len(blob))
        st = self.lib.sph_state_load(C.cast(buf, C.c_void_p), len(blob), C.byref(self.ctx))
        if st != 0:
            raise SphError(st, "sph_state_load")
        self.prm = P.SphParams()
        self._call("sph_get_params", C.byref(self.prm))
        self.dim = int(self.prm.dim)
        self.case = None
        self._restored()
        return self

    def _restored(self) -> None:
        inf = self.info()
        self.n_real, self.n_wall = inf["n_real"], inf["n_wall"]
        self.n = self.n_real + self.n_wall


def probe_fp64_gflops() -> float:
    lib = load()
    g = C.c_double()
    st = lib.sph_probe_fp64_gflops(C.byref(g))
    if st != 0:
        raise SphError(st, "sph_probe_fp64_gflops")
    return g.value


class GpuBatch:
    """Many independent systems advanced together (sph_batch_* of the C ABI).

    One launch per stage covers every live system; each keeps its own hash
    grid, material table and time step.  Systems can be added and removed
    between steps (continuous batching)."""

    def __init__(self, params: P.SphParams, max_instances: int, real_capacity: int,
                 wall_capacity: int):
        self.lib = load()
        self.prm = params.copy()
        self.dim = int(self.prm.dim)
        self.ctx = C.c_void_p()
        st = self.lib.sph_batch_create(C.byref(self.prm), int(max_instances), int(real_capacity),
                                       int(wall_capacity), C.byref(self.ctx))
        if st != 0:
            raise SphError(st, "sph_batch_create")
        self.sizes: dict[int, tuple[int, int]] = {}
        self._keep = {}

    _call = GpuSolver._call
    close = GpuSolver.close
    __del__ = GpuSolver.__del__
    __enter__ = GpuSolver.__enter__
    __exit__ = GpuSolver.__exit__
    stream = GpuSolver.stream
    advance_async = GpuSolver.advance_async
    sync = GpuSolver.sync
    energy = GpuSolver.energy
    enable_stage_timing = GpuSolver.enable_stage_timing
    stage_times = GpuSolver.stage_times
    launch_count = GpuSolver.launch_count
    set_option = GpuSolver.set_option
    device_bytes = GpuSolver.device_bytes

    def add(self, case, params: P.SphParams | None = None) -> int:
        prm = (params or case.params).copy()
        x, v, m, rho, p, e, c, h, t, s, b, sh = case.arrays()
        inst = C.c_int32()
        self._call("sph_batch_add", C.byref(prm), case.n_real, case.n_wall, _dp(x), _dp(v), _dp(m),
                   _dp(rho), _dp(p), _dp(e), _dp(c), _dp(h), t.ctypes.data_as(ip), s.ctypes.data_as(ip),
                   b.ctypes.data_as(ip), _dp(sh), C.byref(inst))
        self.sizes[inst.value] = (case.n_real, case.n_wall)
        return inst.value

    def add_blocks(self, bc, params: P.SphParams | None = None) -> int:
        """Add a system generated on the device from lattice blocks."""
        prm = (params or bc.params).copy()
        inst = C.c_int32()
        self._call("sph_batch_add_blocks", C.byref(prm), len(bc.blocks), bc.array(), bc.n_real_blocks,
                   C.byref(inst))
        self.sizes[inst.value] = bc.counts()
        return inst.value

    def remove(self, inst: int) -> None:
        self._call("sph_batch_remove", int(inst))
        self.sizes.pop(inst, None)

    def field(self, inst: int, name: str) -> np.ndarray:
        nr, nw = self.sizes[inst]
        comp = {"v": self.dim, "t": self.dim * self.dim, "s": 1}[P.FIELD_SHAPE[name]]
        out = np.empty((nr + nw) * comp)
        self._call("sph_batch_get_field", int(inst), P.FIELD[name], _dp(out))
        return out.reshape(nr + nw, comp) if comp > 1 else out

    def info(self, inst: int) -> dict:
        nr, nw, st = C.c_int64(), C.c_int64(), C.c_int64()
        t, mx, mean = C.c_double(), C.c_double(), C.c_double()
        self._call("sph_batch_info", int(inst), C.byref(nr), C.byref(nw), C.byref(st), C.byref(t),
                   C.byref(mx), C.byref(mean))
        return dict(n_real=nr.value, n_wall=nw.value, step=st.value, time=t.value,
                    max_courant=mx.value, mean_courant=mean.value)

    def capacity(self) -> dict:
        fr, fw = C.c_int64(), C.c_int64()
        fs = C.c_int32()
        self._call("sph_batch_capacity", C.byref(fr), C.byref(fw), C.byref(fs))
        return dict(free_real=fr.value, free_wall=fw.value, free_slots=fs.value)

    def advance(self, nsteps: int) -> None:
        mx, mean = C.c_double(), C.c_double()
        self._call("sph_advance", int(nsteps), C.byref(mx), C.byref(mean))

    save_state = GpuSolver.save_state
    from_state = classmethod(GpuSolver.from_state.__func__)

    def slots(self) -> list[int]:
        """Instance ids of the live systems (sph_batch_slots)."""
        m = C.c_int32()
        self._call("sph_batch_slots", C.byref(m), None)
        live = (C.c_uint8 * max(m.value, 1))()
        self._call("sph_batch_slots", C.byref(m), live)
        return [k for k in range(m.value) if live[k]]

    def _restored(self) -> None:
        self.sizes, self._keep = {}, {}
        for k in self.slots():
            inf = self.info(k)
            self.sizes[k] = (inf["n_real"], inf["n_wall"])
