"""ctypes front end of the CPU FP64 oracle (oracle/pm_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU-baseline leg of bench.py, as the checker.  The product library
(nyx_gb300) never imports this module.

Each function names the reference code it restates (paths inside the Nyx tree).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle_pm.so")
_lib = None

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def build(force: bool = False) -> str:
    """Compile the oracle shared library with its Makefile (g++ + OpenMP)."""
    srcs = [os.path.join(_HERE, f) for f in ("pm_oracle.cpp", "pm_amr_oracle.cpp")]
    if force or not os.path.exists(_LIB_PATH) or (
        os.path.getmtime(_LIB_PATH) < max(os.path.getmtime(f) for f in srcs)
    ):
        subprocess.run(["make", "-s", "-C", _HERE, "liboracle_pm.so"], check=True)
    return _LIB_PATH


class _Cfg(C.Structure):
    _fields_ = [
        ("n", C.c_int),
        ("L", C.c_double),
        ("mass_offset", C.c_double),
        ("ggrav", C.c_double),
        ("rel_tol", C.c_double),
        ("max_cycles", C.c_int),
        ("nu1", C.c_int),
        ("nu2", C.c_int),
        ("reuse_field", C.c_int),
    ]


class _AmrCfg(C.Structure):
    _fields_ = [
        ("mass_offset", C.c_double),
        ("ggrav", C.c_double),
        ("rel_tol", C.c_double),
        ("max_cycles", C.c_int),
        ("nu1", C.c_int),
        ("nu2", C.c_int),
    ]


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        L.orc_gconst.restype = C.c_double
        L.orc_num_threads.restype = C.c_int
        L.orc_set_num_threads.argtypes = [C.c_int]
        L.orc_wrap.argtypes = [C.c_double, C.c_long, _dp, _dp, _dp]
        L.orc_sort.restype = C.c_int
        L.orc_sort.argtypes = [C.c_int, C.c_double, C.c_long] + [C.c_void_p] * 7 + [C.c_void_p, _ip]
        L.orc_deposit.argtypes = [C.c_int, C.c_double, C.c_long, _dp, _dp, _dp, C.c_void_p,
                                  C.c_double, _ip, _dp]
        L.orc_canonical_sum.restype = C.c_double
        L.orc_canonical_sum.argtypes = [C.c_int, _dp]
        L.orc_make_rhs.restype = C.c_double
        L.orc_make_rhs.argtypes = [C.c_int, C.c_double, _dp, C.c_double, C.c_double, C.c_double, _dp]
        L.orc_mg_levels.restype = C.c_int
        L.orc_mg_levels.argtypes = [C.c_int]
        L.orc_mg_solve.restype = C.c_int
        L.orc_mg_solve.argtypes = [C.c_int, C.c_double, _dp, _dp, C.c_double, C.c_int, C.c_int,
                                   C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                   C.POINTER(C.c_double)]
        L.orc_bottom_green.argtypes = [C.c_int, C.c_double, _dp]
        L.orc_grav_vector.argtypes = [C.c_int, C.c_double, _dp, _dp]
        L.orc_move.argtypes = [C.c_int, C.c_double, C.c_long, _dp, _dp, _dp, _dp, _dp, _dp, _dp,
                               C.c_double, C.c_double, C.c_double, C.c_int]
        L.orc_integrate_a.restype = C.c_double
        L.orc_integrate_a.argtypes = [C.c_double] * 5
        L.orc_dt_for_da.restype = C.c_double
        L.orc_dt_for_da.argtypes = [C.c_double] * 6
        L.orc_est_time_step.restype = C.c_double
        L.orc_est_time_step.argtypes = [C.c_int, C.c_double, C.c_long, _dp, _dp, _dp, _dp, _dp, _dp,
                                        _dp, C.c_double, C.c_double]
        L.orc_cosmo_1ppc.argtypes = [C.c_int, C.c_double, _dp, _dp, _dp, _dp, _dp, _dp]
        L.orc_comoving_est_dt.restype = C.c_double
        L.orc_comoving_est_dt.argtypes = [C.c_double] * 9 + [C.POINTER(C.c_int)]
        L.orc_step.restype = C.c_int
        L.orc_step.argtypes = [C.POINTER(_Cfg), C.c_long, _dp, _dp, _dp, _dp, _dp, _dp, C.c_void_p,
                               C.c_double, C.c_void_p, C.c_double, C.c_double, C.c_double, _dp, _dp,
                               C.c_void_p, _ip]
        L.orc_amr_create.restype = C.c_void_p
        L.orc_amr_create.argtypes = [C.c_int, C.c_double, C.c_int, _ip, _ip, C.c_char_p, C.c_int]
        L.orc_amr_destroy.argtypes = [C.c_void_p]
        L.orc_amr_assign.argtypes = [C.c_void_p, C.c_long, _dp, _dp, _dp, _ip, _ip]
        L.orc_amr_deposit.argtypes = [C.c_void_p, C.c_long, _dp, _dp, _dp, C.c_void_p, C.c_double,
                                      _ip]
        L.orc_amr_solve.restype = C.c_int
        L.orc_amr_solve.argtypes = [C.c_void_p, C.POINTER(_AmrCfg), C.c_double,
                                    C.POINTER(C.c_int), C.POINTER(C.c_double),
                                    C.POINTER(C.c_double)]
        L.orc_amr_grav.argtypes = [C.c_void_p]
        L.orc_amr_move.restype = C.c_int
        L.orc_amr_move.argtypes = [C.c_void_p, C.c_long, _dp, _dp, _dp, _dp, _dp, _dp, _ip, _ip,
                                   C.c_double, C.c_double, C.c_double, C.c_int]
        L.orc_amr_step.restype = C.c_int
        L.orc_amr_step.argtypes = [C.c_void_p, C.POINTER(_AmrCfg), C.c_long, _dp, _dp, _dp, _dp,
                                   _dp, _dp, C.c_void_p, C.c_double, C.c_double, C.c_double,
                                   C.c_double, _ip, _ip, _ip]
        L.orc_amr_field.restype = C.c_int
        L.orc_amr_field.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp]
        L.orc_amr_total_mass.restype = C.c_double
        L.orc_amr_total_mass.argtypes = [C.c_void_p]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def gconst() -> float:
    """Gconst of Source/Driver/constants_cosmo.H:15-16 (Mpc, M_sun, km/s)."""
    return lib().orc_gconst()


def set_num_threads(t: int) -> None:
    lib().orc_set_num_threads(int(t))


def num_threads() -> int:
    return lib().orc_num_threads()


class Particles:
    """FP64 SoA particle state (AMReX Particle<4,0>: pos + mass, vx, vy, vz)."""

    def __init__(self, pos, vel, mass, ids=None):
        # always copies: the oracle steps its arrays in place, and a column of a
        # column-major (np, 3) array would otherwise be the caller's own memory
        pos = np.asarray(pos, dtype=np.float64)
        vel = np.asarray(vel, dtype=np.float64)
        self.x = np.array(pos[:, 0], dtype=np.float64, order="C", copy=True)
        self.y = np.array(pos[:, 1], dtype=np.float64, order="C", copy=True)
        self.z = np.array(pos[:, 2], dtype=np.float64, order="C", copy=True)
        self.vx = np.array(vel[:, 0], dtype=np.float64, order="C", copy=True)
        self.vy = np.array(vel[:, 1], dtype=np.float64, order="C", copy=True)
        self.vz = np.array(vel[:, 2], dtype=np.float64, order="C", copy=True)
        if np.ndim(mass) == 0:
            self.m = None
            self.mscalar = float(mass)
        else:
            self.m = np.array(mass, dtype=np.float64, order="C", copy=True)
            self.mscalar = 0.0
        self.id = (np.arange(len(self.x), dtype=np.int32) if ids is None
                   else np.array(ids, dtype=np.int32, order="C", copy=True))

    @property
    def np(self) -> int:
        return len(self.x)

    def pos(self):
        return np.stack([self.x, self.y, self.z], axis=1)

    def vel(self):
        return np.stack([self.vx, self.vy, self.vz], axis=1)

    def by_id(self):
        """(pos, vel) ordered by particle id."""
        o = np.argsort(self.id, kind="stable")
        return self.pos()[o], self.vel()[o]

    def total_mass(self) -> float:
        """Sequential sum in id order (the order libnyxpm's upload sums in)."""
        if self.m is None:
            return self.mscalar * float(self.np)
        o = np.argsort(self.id, kind="stable")
        return float(np.cumsum(self.m[o])[-1])


def wrap(L, p: Particles):
    """Periodic shift into [0, L) (RedistributeLocal, Nyx.cpp:1421-1437)."""
    lib().orc_wrap(L, p.np, p.x, p.y, p.z)


def sort(n, L, p: Particles):
    """Stable counting sort by deposit key; returns cell_start (n^3 + 1)."""
    cs = np.zeros(n ** 3 + 1, dtype=np.int32)
    lib().orc_sort(n, L, p.np, _ptr(p.x), _ptr(p.y), _ptr(p.z), _ptr(p.vx), _ptr(p.vy),
                   _ptr(p.vz), _ptr(p.m), _ptr(p.id), cs)
    return cs


def deposit(n, L, p: Particles, cell_start):
    """CIC mass density (AssignDensitySingleLevel; NeutrinoParticleContainer.cpp:209-302)."""
    rho = np.zeros(n ** 3, dtype=np.float64)
    lib().orc_deposit(n, L, p.np, p.x, p.y, p.z, _ptr(p.m), p.mscalar, cell_start, rho)
    return rho


def canonical_sum(n, f) -> float:
    return lib().orc_canonical_sum(n, np.ascontiguousarray(f, dtype=np.float64))


def make_rhs(n, L, rho, mass_offset, ggrav, a):
    """RHS of solve_for_phi (Gravity.cpp:267-290, 1207-1244); returns (rhs, mean)."""
    rhs = np.zeros(n ** 3, dtype=np.float64)
    mean = lib().orc_make_rhs(n, L, np.ascontiguousarray(rho), mass_offset, ggrav, a, rhs)
    return rhs, mean


def mg_levels(n) -> int:
    return lib().orc_mg_levels(n)


def mg_solve(n, L, rhs, phi0=None, rel_tol=1e-10, max_cycles=100, nu1=2, nu2=2):
    """Periodic 7-point Poisson solve by V-cycles; returns (phi, status, cycles, r0, r)."""
    phi = (np.zeros(n ** 3) if phi0 is None else np.array(phi0, dtype=np.float64, copy=True))
    nc, r0, r = C.c_int(0), C.c_double(0), C.c_double(0)
    st = lib().orc_mg_solve(n, L, np.ascontiguousarray(rhs), phi, rel_tol, max_cycles, nu1, nu2,
                            C.byref(nc), C.byref(r0), C.byref(r))
    return phi, st, nc.value, r0.value, r.value


def bottom_green(nb, h):
    G = np.zeros(nb ** 3)
    lib().orc_bottom_green(nb, h, G)
    return G


def grav_vector(n, L, phi):
    """Cell-centred gravity vector, component-major (3, n^3) (Gravity.cpp:817-850)."""
    g = np.zeros(3 * n ** 3)
    lib().orc_grav_vector(n, L, np.ascontiguousarray(phi), g)
    return g


def move(n, L, p: Particles, g, dt, a_prev, a_cur, do_move):
    """update_dm_particle_single over all particles (DarkMatterParticleContainer.cpp:250-306)."""
    lib().orc_move(n, L, p.np, p.x, p.y, p.z, p.vx, p.vy, p.vz, np.ascontiguousarray(g), dt,
                   a_prev, a_cur, int(do_move))


def integrate_a(OmM, OmR, h, a_old, dt) -> float:
    """integrate_comoving_a (comoving.cpp:629-688)."""
    return lib().orc_integrate_a(OmM, OmR, h, a_old, dt)


def dt_for_da(OmM, OmR, h, a_old, a_value, dt_window) -> float:
    """integrate_comoving_a_to_a (comoving.cpp:74-130)."""
    return lib().orc_dt_for_da(OmM, OmR, h, a_old, a_value, dt_window)


def est_time_step(n, L, p: Particles, g, cfl, a) -> float:
    """Particle time-step limit (NyxParticleContainer::estTimestep,
    NyxParticleContainer.H:329-465) with the cell-centred gravity g."""
    return lib().orc_est_time_step(n, L, p.np, p.x, p.y, p.z, p.vx, p.vy, p.vz,
                                   np.ascontiguousarray(g, dtype=np.float64), cfl, a)


def cosmo_1ppc(n, L, disp, vel, disp_fac, vel_fac):
    """InitCosmo1ppcMultiLevel on one level (DarkMatterParticleContainer.cpp:309-450);
    disp, vel (3, n^3) component-major -> (pos, vel) (n^3, 3)."""
    pos = np.zeros((n ** 3, 3))
    velo = np.zeros((n ** 3, 3))
    lib().orc_cosmo_1ppc(n, L, np.ascontiguousarray(disp, dtype=np.float64).ravel(),
                         np.ascontiguousarray(vel, dtype=np.float64).ravel(),
                         np.ascontiguousarray(disp_fac, dtype=np.float64),
                         np.ascontiguousarray(vel_fac, dtype=np.float64), pos, velo)
    return pos, velo


def comoving_est_dt(OmM, OmR, h, a, estdt, relative_max_change_a=0.01,
                    absolute_max_change_a=-1.0, final_a=-1.0, dt_binpow=-1.0):
    """Nyx::comoving_est_time_step (comoving.cpp:353-483); returns (dt, status)."""
    st = C.c_int(0)
    dt = lib().orc_comoving_est_dt(OmM, OmR, h, a, estdt, relative_max_change_a,
                                   absolute_max_change_a, final_a, dt_binpow, C.byref(st))
    return dt, st.value


class PMOracle:
    """The FP64 PM step of Nyx::advance_particles_only on one periodic level."""

    def __init__(self, n, L, particles: Particles, OmM=1.0, OmR=0.0, h=0.675, rel_tol=1e-10,
                 max_cycles=100, nu1=2, nu2=2, reuse_field=False):
        self.n, self.L, self.p = n, L, particles
        self.OmM, self.OmR, self.h = OmM, OmR, h
        self.cfg = _Cfg(n=n, L=L, mass_offset=particles.total_mass() / (L * L * L),
                        ggrav=-4.0 * np.pi * gconst(), rel_tol=rel_tol, max_cycles=max_cycles,
                        nu1=nu1, nu2=nu2, reuse_field=1 if reuse_field else 0)
        self.phi = np.zeros(n ** 3)
        self.g = np.zeros(3 * n ** 3)
        self.rho = np.zeros(n ** 3)
        self.cycles = np.zeros(2, dtype=np.int32)

    def init_field(self, a):
        """post_init solve (Nyx.cpp:1957-2005): deposit, solve from zero, gravity vector."""
        wrap(self.L, self.p)
        cs = sort(self.n, self.L, self.p)
        self.rho = deposit(self.n, self.L, self.p, cs)
        rhs, _ = make_rhs(self.n, self.L, self.rho, self.cfg.mass_offset, self.cfg.ggrav, a)
        self.phi, st, nc, _, _ = mg_solve(self.n, self.L, rhs, None, self.cfg.rel_tol,
                                          self.cfg.max_cycles, self.cfg.nu1, self.cfg.nu2)
        self.g = grav_vector(self.n, self.L, self.phi)
        return st, nc

    def step(self, a_old, a_new, dt):
        p = self.p
        st = lib().orc_step(C.byref(self.cfg), p.np, p.x, p.y, p.z, p.vx, p.vy, p.vz, _ptr(p.m),
                            p.mscalar, _ptr(p.id), a_old, a_new, dt, self.phi, self.g,
                            _ptr(self.rho), self.cycles)
        if st == 1:
            raise ValueError("grid size not supported by the multigrid hierarchy")
        return st


class AmrOracle:
    """The multilevel (AMR) FP64 PM step without subcycling
    (Nyx_advance_particles.cpp:9-272 with finest_level > 0 and
    amr.subcycling_mode = None; Gravity::actual_multilevel_solve,
    Gravity.cpp:602-779).  ``boxes`` lists, for each level above 0, its boxes as
    ((lo_x, lo_y, lo_z), (hi_x, hi_y, hi_z)) in that level's index space."""

    FIELDS = {"rho": 0, "phi": 1, "gx": 2, "gy": 3, "gz": 4, "mass": 5}

    def __init__(self, n0, L, boxes, particles: Particles, rel_tol=1e-10, max_cycles=100, nu1=2,
                 nu2=2):
        self.n0, self.L, self.p = n0, L, particles
        self.nlev = len(boxes) + 1
        self.boxes = [[(tuple(lo), tuple(hi)) for lo, hi in lv] for lv in boxes]
        nbox = np.array([len(lv) for lv in boxes] or [0], dtype=np.int32)
        flat = np.array([c for lv in boxes for lo, hi in lv for c in (*lo, *hi)] or [0],
                        dtype=np.int32)
        err = C.create_string_buffer(256)
        self.h = lib().orc_amr_create(n0, L, self.nlev, nbox, flat, err, 256)
        if not self.h:
            raise ValueError(err.value.decode())
        self.cfg = _AmrCfg(mass_offset=particles.total_mass() / (L * L * L),
                           ggrav=-4.0 * np.pi * gconst(), rel_tol=rel_tol, max_cycles=max_cycles,
                           nu1=nu1, nu2=nu2)
        self.cycles = np.zeros(2, dtype=np.int32)
        self.lev = np.zeros(particles.np, dtype=np.int32)
        self.box = np.zeros(particles.np, dtype=np.int32)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_amr_destroy(self.h)
            self.h = None

    def box_shape(self, b):
        flat = [bx for lv in self.boxes for bx in lv]
        lo, hi = flat[b]
        return tuple(hi[d] - lo[d] + 1 for d in (2, 1, 0))

    def assign(self):
        p = self.p
        lib().orc_amr_assign(self.h, p.np, p.x, p.y, p.z, self.lev, self.box)
        return self.lev.copy(), self.box.copy()

    def deposit(self):
        p = self.p
        lib().orc_amr_deposit(self.h, p.np, p.x, p.y, p.z, _ptr(p.m), p.mscalar, self.lev)

    def solve(self, a):
        nc, r0, r = C.c_int(0), C.c_double(0), C.c_double(0)
        st = lib().orc_amr_solve(self.h, C.byref(self.cfg), a, C.byref(nc), C.byref(r0),
                                 C.byref(r))
        return st, nc.value, r0.value, r.value

    def grav(self):
        lib().orc_amr_grav(self.h)

    def move(self, dt, a_prev, a_cur, do_move):
        p = self.p
        return lib().orc_amr_move(self.h, p.np, p.x, p.y, p.z, p.vx, p.vy, p.vz, self.lev,
                                  self.box, dt, a_prev, a_cur, do_move)

    def step(self, a_old, a_new, dt):
        p = self.p
        st = lib().orc_amr_step(self.h, C.byref(self.cfg), p.np, p.x, p.y, p.z, p.vx, p.vy, p.vz,
                                _ptr(p.m), p.mscalar, a_old, a_new, dt, self.cycles, self.lev,
                                self.box)
        if st == 1:
            raise ValueError("grid size not supported by the multigrid hierarchy")
        return st

    def field(self, name, box=-1):
        """A field on level 0 (box -1, (n0, n0, n0) z-major) or on one box."""
        shape = (self.n0,) * 3 if box < 0 else self.box_shape(box)
        out = np.zeros(int(np.prod(shape)))
        if lib().orc_amr_field(self.h, self.FIELDS[name], box, out):
            raise ValueError("bad field or box")
        return out.reshape(shape)

    def total_mass(self):
        return lib().orc_amr_total_mass(self.h)
