"""Multilevel (AMR) PM step without subcycling on fixed grids (nyxpm_amr_*).

The GPU form of Nyx::advance_particles_only with finest_level > 0 and
amr.subcycling_mode = None (Source/TimeStep/Nyx_advance_particles.cpp:9-272)
and of Gravity::actual_multilevel_solve (Source/Gravity/Gravity.cpp:602-779),
on grids fixed as an amr.regrid_file fixes them (the reference's
Exec/ParticleOnlyTest/inputs.mass.nosub).  ``boxes`` lists, for each level above
0, its boxes as ((lo_x, lo_y, lo_z), (hi_x, hi_y, hi_z)) in that level's own
index space (level l has n0 * 2^l cells per side).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as _L
from .pm import Context, _ptr

FIELDS = {"rho": 0, "phi": 1, "gx": 2, "gy": 3, "gz": 4, "mass": 5}


def regrid_file_boxes(lines, ref_ratio=2):
    """Boxes of an AMReX regrid file (amr.regrid_file): the number of refined
    levels, then per level the number of boxes and the boxes
    ((lo_x,lo_y,lo_z) (hi_x,hi_y,hi_z) (0,0,0)), each given in the index space of
    the level below and refined by the ratio on reading (Amr::regrid's file
    path, AMReX).  Returns the per-level box lists in each level's own index
    space."""
    import re
    toks = []
    for line in lines:
        toks.extend(re.findall(r"\(\s*\(\s*([-\d]+)\s*,\s*([-\d]+)\s*,\s*([-\d]+)\s*\)\s*"
                               r"\(\s*([-\d]+)\s*,\s*([-\d]+)\s*,\s*([-\d]+)\s*\)", line) or
                    [(v,) for v in line.split()])
    it = iter(toks)
    nlev = int(next(it)[0])
    out = []
    for _ in range(nlev):
        nb = int(next(it)[0])
        lv = []
        for _ in range(nb):
            t = [int(v) for v in next(it)]
            lo = tuple(ref_ratio * v for v in t[:3])
            hi = tuple(ref_ratio * (v + 1) - 1 for v in t[3:6])
            lv.append((lo, hi))
        out.append(lv)
    return out


class AmrHierarchy:
    """Levels 0 .. len(boxes), particles and composite fields on the GPU."""

    def __init__(self, ctx: Context, n0: int, L: float, boxes, np_: int):
        self.ctx, self.n0, self.L, self.np = ctx, n0, L, int(np_)
        self.lib = ctx.lib
        self.nlev = len(boxes) + 1
        self.boxes = [[(tuple(lo), tuple(hi)) for lo, hi in lv] for lv in boxes]
        nbox = (C.c_int * max(1, len(boxes)))(*[len(lv) for lv in boxes])
        flat = [c for lv in boxes for lo, hi in lv for c in (*lo, *hi)]
        fb = (C.c_int * max(1, len(flat)))(*flat)
        h = C.c_void_p()
        ctx.check(self.lib.nyxpm_amr_create(ctx.handle, n0, L, self.nlev, nbox, fb, self.np, C.byref(h)),
                  "nyxpm_amr_create")
        self.handle = h

    def close(self):
        if getattr(self, "handle", None):
            self.lib.nyxpm_amr_destroy(self.ctx.handle, self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, pos, vel, mass):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        vel = np.ascontiguousarray(vel, dtype=np.float64)
        if np.ndim(mass) == 0:
            m, ms = None, float(mass)
        else:
            m, ms = np.ascontiguousarray(mass, dtype=np.float64), 0.0
        self.ctx.check(self.lib.nyxpm_amr_upload(self.ctx.handle, self.handle, _ptr(pos), _ptr(vel), _ptr(m),
                                                 ms), "nyxpm_amr_upload")

    def download(self):
        pos = np.zeros((self.np, 3))
        vel = np.zeros((self.np, 3))
        self.ctx.check(self.lib.nyxpm_amr_download(self.ctx.handle, self.handle, _ptr(pos), _ptr(vel)),
                       "nyxpm_amr_download")
        return pos, vel

    def step(self, a_old: float, a_new: float, dt: float) -> dict:
        info = _L.StepInfo()
        self.ctx.check(self.lib.nyxpm_amr_step(self.ctx.handle, self.handle, a_old, a_new, dt, C.byref(info)),
                       "nyxpm_amr_step")
        return {"old_solve": info.old_solve.as_dict(), "new_solve": info.new_solve.as_dict()}

    def assign(self):
        lev = np.zeros(self.np, dtype=np.int32)
        box = np.zeros(self.np, dtype=np.int32)
        self.ctx.check(self.lib.nyxpm_amr_assign(self.ctx.handle, self.handle, _ptr(lev), _ptr(box)),
                       "nyxpm_amr_assign")
        return lev, box

    def deposit(self):
        self.ctx.check(self.lib.nyxpm_amr_deposit(self.ctx.handle, self.handle), "nyxpm_amr_deposit")

    def solve(self, a: float) -> dict:
        info = _L.SolveInfo()
        self.ctx.check(self.lib.nyxpm_amr_solve(self.ctx.handle, self.handle, a, C.byref(info)),
                       "nyxpm_amr_solve")
        return info.as_dict()

    def grav_vector(self):
        self.ctx.check(self.lib.nyxpm_amr_grav_vector(self.ctx.handle, self.handle), "nyxpm_amr_grav_vector")

    def kick(self, dt: float, a_prev: float, a_cur: float, do_move: bool):
        self.ctx.check(self.lib.nyxpm_amr_kick(self.ctx.handle, self.handle, dt, a_prev, a_cur,
                                               1 if do_move else 0), "nyxpm_amr_kick")

    def box_shape(self, b: int):
        lo, hi = [bx for lv in self.boxes for bx in lv][b]
        return tuple(hi[d] - lo[d] + 1 for d in (2, 1, 0))

    def field(self, name: str, box: int = -1) -> np.ndarray:
        """A field on level 0 (box -1, shape (n0, n0, n0), z-major) or on one box."""
        shape = (self.n0,) * 3 if box < 0 else self.box_shape(box)
        out = np.zeros(int(np.prod(shape)))
        self.ctx.check(self.lib.nyxpm_amr_field(self.ctx.handle, self.handle, FIELDS[name], box, _ptr(out)),
                       "nyxpm_amr_field")
        return out.reshape(shape)
