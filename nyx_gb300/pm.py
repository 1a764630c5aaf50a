"""Host-side mirror of Nyx's PM call surface over libnyxpm.

Names and argument meanings follow the reference classes so a caller of Nyx's
particle-mesh path finds the same operations:

* ``DarkMatterParticleContainer`` -- moveKickDrift / moveKick
  (Source/Particle/DarkMatterParticleContainer.cpp:76-247), AssignDensitySingleLevel /
  AssignDensity (Source/Particle/NyxParticleContainer.H:90-97), RedistributeLocal
  (:123-136), sumParticleMass (:70-79);
* ``Gravity`` -- solve_for_phi / solve_for_old_phi / solve_for_new_phi
  (Source/Gravity/Gravity.cpp:202-315), get_old_grav_vector / get_new_grav_vector
  (:781-850), set_mass_offset (:975-1030);
* ``Nyx`` -- advance_particles_only (Source/TimeStep/Nyx_advance_particles.cpp:9-272),
  post_init solve, integrate_comoving_a / integrate_comoving_a_to_a
  (Source/Driver/comoving.cpp).

Where Nyx aborts (amrex::Abort / amrex::Error), these raise ``NyxPMError``.
All state lives on the GPU inside the box; numpy arrays cross only on upload,
download and the optional field read-backs.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib as _L
from .ics import GCONST


class NyxPMError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{_L.STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None and a.shape != shape:
        a = a.reshape(shape)
    return a


def _ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


class Context:
    """A CUDA device + stream + solver parameters (nyxpm_ctx)."""

    def __init__(self, device: int = 0, stream: int | None = None, OmM: float = 1.0,
                 OmR: float = 0.0, h: float = 0.675, rel_tol: float = 1e-10,
                 max_vcycles: int = 100, nu1: int = 2, nu2: int = 2, gconst: float | None = None,
                 mg_fused_edge: int | None = None):
        self.lib = _L.load()
        p = _L.Params()
        self.lib.nyxpm_default_params(C.byref(p))
        p.device = device
        p.stream = stream
        p.comoving_OmM, p.comoving_OmR, p.comoving_h = OmM, OmR, h
        if gconst is not None:
            p.gconst = gconst
        p.rel_tol, p.max_vcycles, p.nu1, p.nu2 = rel_tol, max_vcycles, nu1, nu2
        if mg_fused_edge is not None:
            p.mg_fused_edge = mg_fused_edge
        self.params = p
        h_ = C.c_void_p()
        st = self.lib.nyxpm_create(C.byref(p), C.byref(h_))
        if st != _L.NYXPM_OK:
            raise NyxPMError(st, "nyxpm_create failed")
        self.handle = h_

    def check(self, st: int, what: str = ""):
        if st != _L.NYXPM_OK:
            msg = self.lib.nyxpm_last_error(self.handle)
            raise NyxPMError(st, f"{what}: {msg.decode() if msg else ''}")

    @property
    def stream(self) -> int:
        return self.lib.nyxpm_stream(self.handle) or 0

    def synchronize(self):
        self.check(self.lib.nyxpm_synchronize(self.handle), "synchronize")

    def launch_count(self) -> int:
        return int(self.lib.nyxpm_launch_count(self.handle))

    def measure_fp64_peak(self) -> tuple[float, float]:
        """(FP64 TFLOP/s on FMA chains, T FP64 additions/s) this GPU sustains
        (nyxpm_measure_fp64_peak)."""
        v, a = C.c_double(0), C.c_double(0)
        self.check(self.lib.nyxpm_measure_fp64_peak(self.handle, C.byref(v), C.byref(a)),
                   "measure_fp64_peak")
        return v.value, a.value

    def set_profiling(self, on: bool):
        self.check(self.lib.nyxpm_set_profiling(self.handle, 1 if on else 0), "set_profiling")

    def profile(self, reset: bool = False) -> dict:
        pr = _L.Profile()
        self.check(self.lib.nyxpm_get_profile(self.handle, C.byref(pr), 1 if reset else 0), "profile")
        stages = {name: {"launches": int(pr.launches[i]), "ms": float(pr.ms[i]),
                         "bytes": float(pr.bytes[i])} for i, name in enumerate(_L.STAGE_NAMES)}
        return {"stages": stages, "fine_smooth": {"launches": int(pr.fine_smooth_launches),
                                                  "ms": float(pr.fine_smooth_ms),
                                                  "bytes": float(pr.fine_smooth_bytes)}}

    # a(t), FP64 on the host (comoving.cpp)
    def integrate_comoving_a(self, a_old: float, dt: float) -> float:
        return self.lib.nyxpm_integrate_a(C.byref(self.params), a_old, dt)

    def integrate_comoving_a_to_a(self, a_old: float, a_value: float, dt_window: float) -> float:
        return self.lib.nyxpm_dt_for_da(C.byref(self.params), a_old, a_value, dt_window)

    def dt_params(self, **overrides) -> "_L.DtParams":
        """nyxpm_dt_params with the reference defaults, then the given fields."""
        dp = _L.DtParams()
        self.lib.nyxpm_default_dt_params(C.byref(dp))
        for k, v in overrides.items():
            setattr(dp, k, float(v))
        return dp

    def comoving_est_dt(self, a: float, estdt: float, **dt_params) -> float:
        """Nyx::comoving_est_time_step (comoving.cpp:353-483): estdt limited by how fast a
        may change."""
        out = C.c_double(0)
        st = self.lib.nyxpm_comoving_est_dt(C.byref(self.params), float(a), float(estdt),
                                            C.byref(self.dt_params(**dt_params)), C.byref(out))
        if st != _L.NYXPM_OK:
            raise NyxPMError(st, "comoving_est_dt: a past final_a or no convergence")
        return out.value

    def cosmo_ic_factors(self, source: str, n: int, L: float, redshift: float = -1.0):
        """Nyx::initcosmo's (disp_fac, vel_fac, particle_mass) for ic-source "MUSIC" or "nyx"."""
        df, vf, m = (C.c_double * 3)(), (C.c_double * 3)(), C.c_double(0)
        src = {"MUSIC": 0, "nyx": 1}[source]
        st = self.lib.nyxpm_cosmo_ic_factors(C.byref(self.params), src, int(n), float(L),
                                             float(redshift), df, vf, C.byref(m))
        if st != _L.NYXPM_OK:
            raise NyxPMError(st, "cosmo_ic_factors: bad arguments")
        return list(df), list(vf), m.value

    def hubble(self, a: float) -> float:
        p = self.params
        OmL = 1.0 - p.comoving_OmM - p.comoving_OmR
        return p.comoving_h * 100.0 * math.sqrt(p.comoving_OmM / a ** 3 + p.comoving_OmR / a ** 4 + OmL)

    def step_schedule(self, a_start: float, a_end: float, nsteps: int):
        """Equal-delta-a steps: [(a_old, a_new, dt)], dt from integrate_comoving_a_to_a and
        a_new re-integrated from dt as Nyx::integrate_comoving_a does."""
        out = []
        a = a_start
        da = (a_end - a_start) / nsteps
        for _ in range(nsteps):
            target = a + da
            adot_min = min(a * self.hubble(a), target * self.hubble(target))
            window = 1.01 * da / adot_min
            dt = self.integrate_comoving_a_to_a(a, target, window)
            a_new = self.integrate_comoving_a(a, dt)
            out.append((a, a_new, dt))
            a = a_new
        return out

    def close(self):
        if getattr(self, "handle", None):
            self.lib.nyxpm_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def box_bytes(n: int, np_: int, precision: str = "fp64") -> int:
    lib = _L.load()
    return int(lib.nyxpm_box_bytes(n, np_, _L.NYXPM_MIXED if precision == "mixed" else _L.NYXPM_FP64))


class Box:
    """One periodic n^3 grid with its particles, resident on the GPU (nyxpm_box)."""

    def __init__(self, ctx: Context, n: int, L: float, np_: int, precision: str = "fp64"):
        self.ctx, self.n, self.L, self.np = ctx, n, L, int(np_)
        self.precision = precision
        prec = _L.NYXPM_MIXED if precision == "mixed" else _L.NYXPM_FP64
        h = C.c_void_p()
        ctx.check(ctx.lib.nyxpm_box_create(ctx.handle, n, float(L), self.np, prec, C.byref(h)),
                  "box_create")
        self.handle = h

    def _c(self, fn, *args, what=""):
        self.ctx.check(fn(self.ctx.handle, self.handle, *args), what)

    def upload(self, pos, vel, mass):
        pos = _f64(pos, (self.np, 3))
        vel = _f64(vel, (self.np, 3))
        if np.ndim(mass) == 0:
            self._c(self.ctx.lib.nyxpm_box_upload, _ptr(pos), _ptr(vel), None, float(mass), what="upload")
            self.mass = float(mass)
        else:
            m = _f64(mass, (self.np,))
            self._c(self.ctx.lib.nyxpm_box_upload, _ptr(pos), _ptr(vel), _ptr(m), 0.0, what="upload")
            self.mass = m.copy()

    def init_cosmo_1ppc(self, disp, vel, disp_fac, vel_fac, particle_mass: float):
        """InitCosmo1ppcMultiLevel on this level: one particle per cell from the IC fields."""
        disp = _f64(np.asarray(disp).reshape(3, -1))
        vel = _f64(np.asarray(vel).reshape(3, -1))
        df = _f64(np.asarray(disp_fac, dtype=np.float64))
        vf = _f64(np.asarray(vel_fac, dtype=np.float64))
        self._c(self.ctx.lib.nyxpm_box_init_cosmo_1ppc, _ptr(disp), _ptr(vel), _ptr(df), _ptr(vf),
                float(particle_mass), what="init_cosmo_1ppc")
        self.mass = float(particle_mass)

    def upload_ptr(self, pos_ptr: int, vel_ptr: int, mass: float):
        """Upload from raw host pointers (pinned buffers), uniform mass."""
        self._c(self.ctx.lib.nyxpm_box_upload, C.c_void_p(pos_ptr), C.c_void_p(vel_ptr), None,
                float(mass), what="upload")

    def download(self):
        pos = np.empty((self.np, 3))
        vel = np.empty((self.np, 3))
        self._c(self.ctx.lib.nyxpm_box_download, _ptr(pos), _ptr(vel), what="download")
        return pos, vel

    def download_ptr(self, pos_ptr: int, vel_ptr: int):
        self._c(self.ctx.lib.nyxpm_box_download, C.c_void_p(pos_ptr), C.c_void_p(vel_ptr),
                what="download")

    def mass_offset(self) -> float:
        v = C.c_double()
        self._c(self.ctx.lib.nyxpm_set_mass_offset, C.byref(v), what="set_mass_offset")
        return v.value

    def redistribute(self):
        self._c(self.ctx.lib.nyxpm_redistribute, what="redistribute")

    def deposit(self, read_back: bool = True):
        rho = np.empty(self.n ** 3) if read_back else None
        self._c(self.ctx.lib.nyxpm_deposit, _ptr(rho), what="deposit")
        return rho

    def solve_phi(self, a: float, zero_guess: bool = False) -> dict:
        info = _L.SolveInfo()
        self._c(self.ctx.lib.nyxpm_solve_phi, float(a), 1 if zero_guess else 0, C.byref(info),
                what="solve_phi")
        return info.as_dict()

    def get_phi(self):
        phi = np.empty(self.n ** 3)
        self._c(self.ctx.lib.nyxpm_get_phi, _ptr(phi), what="get_phi")
        return phi

    def set_phi(self, phi):
        phi = _f64(phi, (self.n ** 3,))
        self._c(self.ctx.lib.nyxpm_set_phi, _ptr(phi), what="set_phi")

    def grav_vector(self, read_back: bool = True):
        g = np.empty(3 * self.n ** 3) if read_back else None
        self._c(self.ctx.lib.nyxpm_grav_vector, _ptr(g), what="grav_vector")
        return g

    def set_grav_vector(self, g):
        """The caller's acceleration for the next kicks (nyxpm_set_grav_vector): 3 n^3
        values, component-major, x fastest -- a numpy array (host memory) or any object
        with ``data_ptr()`` and ``is_cuda`` true (device memory on the context's device,
        e.g. a torch tensor), float64 and contiguous."""
        count = 3 * self.n ** 3
        if getattr(g, "is_cuda", False) and hasattr(g, "data_ptr"):
            if g.numel() != count or str(g.dtype) != "torch.float64" or not g.is_contiguous():
                raise ValueError(f"device g must be {count} contiguous float64 values")
            self._c(self.ctx.lib.nyxpm_set_grav_vector, C.c_void_p(g.data_ptr()), 1,
                    what="set_grav_vector")
            return
        garr = _f64(np.asarray(g).reshape(-1))
        if garr.size != count:
            raise ValueError(f"g must hold {count} values (3 n^3)")
        self._c(self.ctx.lib.nyxpm_set_grav_vector, _ptr(garr), 0, what="set_grav_vector")

    def kick_drift(self, dt, a_old, a_half):
        self._c(self.ctx.lib.nyxpm_kick_drift, float(dt), float(a_old), float(a_half), what="kick_drift")

    def kick(self, dt, a_new, a_half):
        self._c(self.ctx.lib.nyxpm_kick, float(dt), float(a_new), float(a_half), what="kick")

    def init_field(self, a: float) -> dict:
        info = _L.SolveInfo()
        self._c(self.ctx.lib.nyxpm_init_field, float(a), C.byref(info), what="init_field")
        return info.as_dict()

    def est_time_step(self, cfl: float, a: float) -> float:
        """Particle time-step limit (NyxParticleContainer::estTimestep) with the box's field."""
        out = C.c_double(0)
        self._c(self.ctx.lib.nyxpm_est_time_step, float(cfl), float(a), C.byref(out),
                what="est_time_step")
        return out.value

    def compute_new_dt(self, time: float, a: float, dt_old: float, **dt_params):
        """Nyx::computeNewDt at level 0 (particles, a-change limit, change_max, stop_time);
        returns (dt, a_new)."""
        dt, a_new = C.c_double(0), C.c_double(0)
        self._c(self.ctx.lib.nyxpm_compute_new_dt, C.byref(self.ctx.dt_params(**dt_params)),
                float(time), float(a), float(dt_old), C.byref(dt), C.byref(a_new),
                what="compute_new_dt")
        return dt.value, a_new.value

    def step(self, a_old, a_new, dt, reuse_field: bool = False) -> dict:
        info = _L.StepInfo()
        flags = _L.NYXPM_STEP_REUSE_FIELD if reuse_field else 0
        self._c(self.ctx.lib.nyxpm_step, float(a_old), float(a_new), float(dt), flags,
                C.byref(info), what="step")
        return {"old_solve": info.old_solve.as_dict(), "new_solve": info.new_solve.as_dict()}

    def step_host(self, pos, vel, mass, a_old, a_new, dt, reuse_field: bool = False) -> dict:
        """upload + step + download in one call (nyxpm_step_host): pos and vel
        (np x 3 float64, C order) are overwritten in place with the stepped state."""
        for arr in (pos, vel):
            if not (isinstance(arr, np.ndarray) and arr.dtype == np.float64 and arr.shape == (self.np, 3)
                    and arr.flags.c_contiguous and arr.flags.writeable):
                raise ValueError("pos and vel must be writeable C-contiguous float64 arrays of shape (np, 3)")
        return self.step_host_ptr(pos.ctypes.data, vel.ctypes.data, mass, a_old, a_new, dt, reuse_field)

    def step_host_ptr(self, pos_ptr: int, vel_ptr: int, mass, a_old, a_new, dt,
                      reuse_field: bool = False) -> dict:
        """step_host on raw host pointers (pinned buffers let the copies overlap the step)."""
        info = _L.StepInfo()
        flags = _L.NYXPM_STEP_REUSE_FIELD if reuse_field else 0
        if np.ndim(mass) == 0:
            mptr, ms = None, float(mass)
        else:
            m = _f64(mass, (self.np,))
            mptr, ms = _ptr(m), 0.0
        self._c(self.ctx.lib.nyxpm_step_host, C.c_void_p(pos_ptr), C.c_void_p(vel_ptr), mptr, ms,
                float(a_old), float(a_new), float(dt), flags, C.byref(info), what="step_host")
        self.mass = float(mass) if np.ndim(mass) == 0 else np.asarray(mass, dtype=np.float64).copy()
        return {"old_solve": info.old_solve.as_dict(), "new_solve": info.new_solve.as_dict()}

    def close(self):
        if getattr(self, "handle", None) and self.ctx.handle:
            self.ctx.lib.nyxpm_box_destroy(self.ctx.handle, self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# particle files and the comoving_a file (host I/O in the library)
# ---------------------------------------------------------------------------
FILE_FORMATS = {"ascii": _L.NYXPM_FILE_ASCII, "binary": _L.NYXPM_FILE_BINARY,
                "binary_meta": _L.NYXPM_FILE_BINARY_META, "binary64": _L.NYXPM_FILE_BINARY_F64}


def _io_call(fn, *args):
    err = C.create_string_buffer(512)
    st = fn(*args, err, len(err))
    if st != _L.NYXPM_OK:
        raise NyxPMError(st, err.value.decode(errors="replace"))


def read_particle_file(path: str, fmt: str = "ascii"):
    """Nyx's AsciiFile / BinaryFile / BinaryMetaFile particle ICs -> (pos, vel, mass),
    pos and vel (np, 3) float64, mass (np,) float64."""
    lib = _L.load()
    f = FILE_FORMATS[fmt]
    np_ = C.c_int64(0)
    _io_call(lib.nyxpm_particle_file_count, str(path).encode(), f, C.byref(np_))
    n = np_.value
    pos, vel, mass = np.empty((n, 3)), np.empty((n, 3)), np.empty(n)
    got = C.c_int64(0)
    _io_call(lib.nyxpm_particle_file_read, str(path).encode(), f, n, _ptr(pos), _ptr(vel),
             _ptr(mass), C.byref(got))
    return pos[:got.value], vel[:got.value], mass[:got.value]


def write_particle_file(path: str, pos, vel, mass, fmt: str = "ascii"):
    """Write particles as an AsciiFile or BinaryFile; mass is an array or a scalar."""
    lib = _L.load()
    pos = _f64(pos)
    vel = _f64(vel)
    marr = None if np.ndim(mass) == 0 else _f64(mass)
    _io_call(lib.nyxpm_particle_file_write, str(path).encode(), FILE_FORMATS[fmt], len(pos),
             _ptr(pos), _ptr(vel), _ptr(marr), float(mass) if marr is None else 0.0)


def uniform_mass(mass):
    """The scalar mass if every particle has the same one, else the array."""
    mass = np.asarray(mass, dtype=np.float64)
    return float(mass[0]) if mass.size and np.all(mass == mass[0]) else mass


def cosmo_1ppc_particles(n: int, L: float, disp, vel, disp_fac, vel_fac):
    """One particle per cell from displacement and velocity fields (3, n^3) or
    (3, n, n, n) in Nyx's component order (InitCosmo1ppcMultiLevel) -> (pos, vel)."""
    lib = _L.load()
    disp = _f64(np.asarray(disp).reshape(3, -1))
    vel = _f64(np.asarray(vel).reshape(3, -1))
    df, vf = _f64(np.asarray(disp_fac, dtype=np.float64)), _f64(np.asarray(vel_fac, dtype=np.float64))
    pos, v = np.empty((n ** 3, 3)), np.empty((n ** 3, 3))
    st = lib.nyxpm_cosmo_1ppc_particles(n, float(L), _ptr(disp), _ptr(vel), _ptr(df), _ptr(vf),
                                        _ptr(pos), _ptr(v))
    if st != _L.NYXPM_OK:
        raise NyxPMError(st, "cosmo_1ppc_particles: bad arguments")
    return pos, v


def particles_info(directory: str) -> dict:
    """Header of an AMReX particle directory (a checkpoint's or plotfile's "DM")."""
    lib = _L.load()
    h = _L.ParticleHeader()
    _io_call(lib.nyxpm_particles_info, str(directory).encode(), C.byref(h))
    return h.as_dict()


def read_particles_dir(directory: str, with_ids: bool = False):
    """The particles of an AMReX particle directory -> (pos, vel, mass[, ids])."""
    lib = _L.load()
    n = particles_info(directory)["num_particles"]
    pos, vel, mass = np.empty((n, 3)), np.empty((n, 3)), np.empty(n)
    ids = np.empty(n, dtype=np.int64) if with_ids else None
    got = C.c_int64(0)
    _io_call(lib.nyxpm_particles_read, str(directory).encode(), n, _ptr(pos), _ptr(vel), _ptr(mass),
             _ptr(ids), C.byref(got))
    out = (pos[:got.value], vel[:got.value], mass[:got.value])
    return out + (ids[:got.value],) if with_ids else out


def write_particles_dir(directory: str, n: int, pos, vel, mass, checkpoint: bool = True,
                        single_precision: bool = False):
    """Write particles as an AMReX particle directory (Version_Two_Dot_Zero), one grid
    over the n^3 domain; mass is an array or a scalar."""
    lib = _L.load()
    pos, vel = _f64(pos), _f64(vel)
    marr = None if np.ndim(mass) == 0 else _f64(mass)
    _io_call(lib.nyxpm_particles_write, str(directory).encode(), int(n), len(pos), _ptr(pos), _ptr(vel),
             _ptr(marr), float(mass) if marr is None else 0.0, 1 if checkpoint else 0,
             1 if single_precision else 0)


def write_comoving_a(directory: str, a: float):
    _io_call(_L.load().nyxpm_write_comoving_a, str(directory).encode(), float(a))


def read_comoving_a(directory: str) -> float:
    a = C.c_double(0)
    _io_call(_L.load().nyxpm_read_comoving_a, str(directory).encode(), C.byref(a))
    return a.value


# ---------------------------------------------------------------------------
# the reference-named facade
# ---------------------------------------------------------------------------
class DarkMatterParticleContainer:
    """Nyx's DM particle container on one periodic level, resident on the GPU."""

    def __init__(self, box: Box):
        self.box = box

    def InitFromArrays(self, pos, vel, mass):
        """Particle fill (init_particles AsciiFile/BinaryFile/Cosmological, NyxParticles.cpp:378-591)."""
        self.box.upload(pos, vel, mass)

    def _init_from_file(self, path, fmt):
        pos, vel, mass = read_particle_file(path, fmt)
        if len(pos) != self.box.np:
            raise NyxPMError(1, f"{path} holds {len(pos)} particles, the box {self.box.np}")
        self.box.upload(pos, vel, uniform_mass(mass))

    def InitFromAsciiFile(self, path, nextra: int = 4):
        """nyx.particle_init_type = AsciiFile (NyxParticles.cpp:506-523)."""
        self._init_from_file(path, "ascii")

    def InitFromBinaryFile(self, path, nextra: int = 4):
        """nyx.particle_init_type = BinaryFile (NyxParticles.cpp:525-543)."""
        self._init_from_file(path, "binary")

    def InitFromBinaryMetaFile(self, path, nextra: int = 4):
        """nyx.particle_init_type = BinaryMetaFile (NyxParticles.cpp:545-560)."""
        self._init_from_file(path, "binary_meta")

    def WriteAsciiFile(self, path):
        """The particles in AsciiFile layout (count line, then x y z mass vx vy vz)."""
        pos, vel = self.box.download()
        write_particle_file(path, pos, vel, self.box.mass)

    def moveKickDrift(self, acceleration=None, lev: int = 0, dt: float = 0.0, a_old: float = 1.0,
                      a_half: float = 1.0, where_width: int = 0):
        """Kick by dt/2 with the CIC-interpolated acceleration, then drift by dt.
        ``acceleration`` is the caller's cell-centred field (3 n^3 values, component-major,
        x fastest; host array or device tensor), as the reference's ``acc`` MultiFab; None
        kicks with the box's own gravity vector, kept in step with phi on the device."""
        if lev != 0:
            raise NyxPMError(1, "single level only")
        if acceleration is not None:
            self.box.set_grav_vector(acceleration)
        self.box.kick_drift(dt, a_old, a_half)

    def moveKick(self, acceleration=None, lev: int = 0, dt: float = 0.0, a_new: float = 1.0,
                 a_half: float = 1.0):
        """Kick by dt/2 with the CIC-interpolated acceleration (see moveKickDrift)."""
        if lev != 0:
            raise NyxPMError(1, "single level only")
        if acceleration is not None:
            self.box.set_grav_vector(acceleration)
        self.box.kick(dt, a_new, a_half)

    def AssignDensitySingleLevel(self, mf=None, lev: int = 0, ncomp: int = 1,
                                 particle_lvl_offset: int = 0):
        """CIC mass density; fills ``mf`` (n^3 array) when given and returns it."""
        if lev != 0 or ncomp != 1 or particle_lvl_offset != 0:
            raise NyxPMError(1, "single level, one component, no level offset")
        rho = self.box.deposit(read_back=True)
        if mf is not None:
            mf[...] = rho.reshape(mf.shape)
            return mf
        return rho

    def AssignDensity(self, mf: list, lev_min: int = 0, ncomp: int = 1, finest_level: int = -1,
                      ngrow: int = 1):
        """Callee-allocating form: appends the level-0 density to ``mf``."""
        if lev_min != 0 or finest_level not in (-1, 0):
            raise NyxPMError(1, "single level only")
        mf.clear()
        mf.append(self.box.deposit(read_back=True).reshape(self.box.n, self.box.n, self.box.n))
        return mf

    def RedistributeLocal(self, lev_min: int = 0, lev_max: int = -1, nGrow: int = 0):
        self.box.redistribute()

    def estTimestep(self, acceleration=None, a: float = 1.0, lev: int = 0, cfl: float = 0.5) -> float:
        """NyxParticleContainer::estTimestep (NyxParticleContainer.H:329-465) with the
        caller's acceleration (as in moveKickDrift) or, for None, the box's own gravity vector."""
        if lev != 0:
            raise NyxPMError(1, "single level only")
        if acceleration is not None:
            self.box.set_grav_vector(acceleration)
        return self.box.est_time_step(cfl, a)

    def sumParticleMass(self, lev: int = 0) -> float:
        return self.box.mass_offset() * self.box.L ** 3

    def GetParticles(self):
        return self.box.download()


class Gravity:
    """The comoving Poisson solve of one periodic level."""

    def __init__(self, box: Box):
        self.box = box
        self.mass_offset = 0.0
        self.level_solver_resnorm = [0.0]
        self.last_info: dict = {}

    def set_mass_offset(self, time: float = 0.0) -> float:
        self.mass_offset = self.box.mass_offset()
        return self.mass_offset

    def solve_for_phi(self, level: int, a: float, zero_guess: bool = False):
        """Deposit already done; RHS from it, V-cycles (Gravity.cpp:267-315)."""
        info = self.box.solve_phi(a, zero_guess)
        self.level_solver_resnorm[0] = info["resnorm"]
        self.last_info = info
        return info

    def solve_for_old_phi(self, level: int, a_old: float):
        self.box.deposit(read_back=False)
        return self.solve_for_phi(level, a_old, zero_guess=True)

    def solve_for_new_phi(self, level: int, a_new: float):
        self.box.deposit(read_back=False)
        return self.solve_for_phi(level, a_new, zero_guess=False)

    def get_phi(self):
        return self.box.get_phi()

    def get_new_grav_vector(self, level: int = 0):
        return self.box.grav_vector(read_back=True).reshape(3, self.box.n, self.box.n, self.box.n)

    get_old_grav_vector = get_new_grav_vector


class Nyx:
    """Level-0 driver of the particle-only PM step."""

    def __init__(self, ctx: Context, n: int, L: float, pos, vel, mass):
        self.ctx = ctx
        self.box = Box(ctx, n, L, len(pos))
        self.particles = DarkMatterParticleContainer(self.box)
        self.particles.InitFromArrays(pos, vel, mass)
        self.gravity = Gravity(self.box)
        self.gravity.set_mass_offset()

    def comoving_a_post_restart(self, restart_dir: str) -> float:
        """Nyx::comoving_a_post_restart (comoving.cpp:690-705): a from <dir>/comoving_a."""
        return read_comoving_a(restart_dir)

    def write_comoving_a(self, directory: str, a: float):
        """The comoving_a file of Nyx::checkPointPost (Nyx_output.cpp:994-1010)."""
        write_comoving_a(directory, a)

    def post_init(self, a: float):
        """Nyx::post_init (Nyx.cpp:1957-2005): solve for phi at the initial a."""
        return self.box.init_field(a)

    def advance_particles_only(self, a_old: float, a_new: float, dt: float,
                               reuse_field: bool = False) -> dict:
        return self.box.step(a_old, a_new, dt, reuse_field=reuse_field)

    def computeNewDt(self, time: float, a: float, dt_old: float, **dt_params):
        """Nyx::computeNewDt at level 0 without subcycling (Nyx.cpp:1023-1208);
        returns (dt, a_new)."""
        return self.box.compute_new_dt(time, a, dt_old, **dt_params)
