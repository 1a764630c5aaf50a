"""Batched ensembles of independent PM boxes (mixed precision) over libnyxpm.

``Ensemble`` wraps nyxpm_ensemble: boxes of uneven sizes share one device arena
of a fixed byte budget and advance together, one persistent launch per stage
and one graph replay per step.  ``ensemble_workload`` draws the seeded
ensemble configuration (grid sizes log-uniform over {32, 48, 64, 96, 128},
particle count = cells x {0.5 or 1}, power-law slope uniform in [-2.5, -1.5]).
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import _lib as _L
from .ics import zeldovich_ics
from .pm import Context, NyxPMError


def _ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


class Ensemble:
    """A set of periodic boxes advanced together (nyxpm_ensemble)."""

    def __init__(self, ctx: Context, arena_bytes: int):
        self.ctx = ctx
        self.lib = ctx.lib
        h = C.c_void_p()
        ctx.check(self.lib.nyxpm_ensemble_create(ctx.handle, int(arena_bytes), C.byref(h)),
                  "ensemble_create")
        self.handle = h
        self.boxes: dict[int, dict] = {}

    @staticmethod
    def box_bytes(n: int, np_: int) -> int:
        return int(_L.load().nyxpm_ensemble_box_bytes(n, np_))

    def arena_used(self) -> int:
        return int(self.lib.nyxpm_ensemble_arena_used(self.handle))

    def add(self, n: int, L: float, np_: int) -> int:
        slot = C.c_int()
        st = self.lib.nyxpm_ensemble_add(self.ctx.handle, self.handle, n, float(L), int(np_),
                                         C.byref(slot))
        self.ctx.check(st, "ensemble_add")
        self.boxes[slot.value] = {"n": n, "L": L, "np": int(np_)}
        return slot.value

    def try_add(self, n: int, L: float, np_: int):
        """Like add, but returns None when the memory budget is exhausted."""
        slot = C.c_int()
        st = self.lib.nyxpm_ensemble_add(self.ctx.handle, self.handle, n, float(L), int(np_),
                                         C.byref(slot))
        if st == 2:
            return None
        self.ctx.check(st, "ensemble_add")
        self.boxes[slot.value] = {"n": n, "L": L, "np": int(np_)}
        return slot.value

    def remove(self, slot: int):
        self.ctx.check(self.lib.nyxpm_ensemble_remove(self.ctx.handle, self.handle, slot),
                       "ensemble_remove")
        self.boxes.pop(slot, None)

    def upload(self, slot: int, pos, vel, mass: float):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        vel = np.ascontiguousarray(vel, dtype=np.float64)
        self.ctx.check(self.lib.nyxpm_ensemble_upload(self.ctx.handle, self.handle, slot, _ptr(pos),
                                                      _ptr(vel), float(mass)), "ensemble_upload")

    def download(self, slot: int):
        np_ = self.boxes[slot]["np"]
        pos = np.empty((np_, 3))
        vel = np.empty((np_, 3))
        self.ctx.check(self.lib.nyxpm_ensemble_download(self.ctx.handle, self.handle, slot,
                                                        _ptr(pos), _ptr(vel)), "ensemble_download")
        return pos, vel

    def get_phi(self, slot: int):
        n = self.boxes[slot]["n"]
        phi = np.empty(n ** 3)
        self.ctx.check(self.lib.nyxpm_ensemble_get_phi(self.ctx.handle, self.handle, slot, _ptr(phi)),
                       "ensemble_get_phi")
        return phi

    def grav_vector(self, slot: int):
        n = self.boxes[slot]["n"]
        g = np.empty(3 * n ** 3)
        self.ctx.check(self.lib.nyxpm_ensemble_grav_vector(self.ctx.handle, self.handle, slot, _ptr(g)),
                       "ensemble_grav_vector")
        return g

    def tuning(self) -> dict:
        t = _L.Tuning()
        self.ctx.check(self.lib.nyxpm_ensemble_get_tuning(self.ctx.handle, self.handle, C.byref(t)),
                       "ensemble_get_tuning")
        return t.as_dict()

    def set_tuning(self, **kw):
        t = _L.Tuning()
        self.ctx.check(self.lib.nyxpm_ensemble_get_tuning(self.ctx.handle, self.handle, C.byref(t)),
                       "ensemble_get_tuning")
        for k, v in kw.items():
            setattr(t, k, int(v))
        self.ctx.check(self.lib.nyxpm_ensemble_set_tuning(self.ctx.handle, self.handle, C.byref(t)),
                       "ensemble_set_tuning")

    def step(self, a_old: dict, a_new: dict, dt: dict) -> dict:
        """One step of the slots in a_old (slot -> a); other slots idle."""
        nslot = max(self.boxes) + 1 if self.boxes else 0
        ao = np.zeros(nslot)
        an = np.zeros(nslot)
        d = np.zeros(nslot)
        for s, v in a_old.items():
            ao[s] = v
            an[s] = a_new[s]
            d[s] = dt[s]
        info = _L.EnsembleInfo()
        dp = C.POINTER(C.c_double)
        st = self.lib.nyxpm_ensemble_step(self.ctx.handle, self.handle, ao.ctypes.data_as(dp),
                                          an.ctypes.data_as(dp), d.ctypes.data_as(dp), C.byref(info))
        self.ctx.check(st, "ensemble_step")
        return info.as_dict()

    def close(self):
        if getattr(self, "handle", None) and self.ctx.handle:
            self.lib.nyxpm_ensemble_destroy(self.ctx.handle, self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class BoxSpec:
    n: int
    fraction: float
    seed: int
    slope: float
    L: float = 1.0

    @property
    def np(self) -> int:
        return int(math.ceil(self.fraction * self.n ** 3))


SIZES = (32, 48, 64, 96, 128)


def ensemble_workload(nboxes: int = 256, seed: int = 4, sizes=SIZES) -> list[BoxSpec]:
    """Seeded ensemble: n drawn log-uniformly over [min, max] and snapped to the
    nearest allowed size in log space; particles = n^3 x {0.5 or 1} (coin flip);
    per-box IC seed; slope uniform in [-2.5, -1.5]."""
    rng = np.random.default_rng(seed)
    logs = np.log(np.asarray(sizes, dtype=np.float64))
    out = []
    for b in range(nboxes):
        u = rng.uniform(logs[0], logs[-1])
        n = int(sizes[int(np.argmin(np.abs(logs - u)))])
        frac = 0.5 if rng.random() < 0.5 else 1.0
        out.append(BoxSpec(n=n, fraction=frac, seed=int(rng.integers(1, 2 ** 31 - 1)),
                           slope=float(rng.uniform(-2.5, -1.5))))
    return out


def box_ics(spec: BoxSpec, a_init: float = 0.02):
    return zeldovich_ics(spec.n, spec.L, spec.slope, spec.seed, a_init, rms_disp_cells=0.2,
                         fraction=spec.fraction)
