"""AMReX MultiFab files (VisMF, header version 1) through the C ABI.

``read_ic_fields`` reads a cosmological IC MultiFab as Nyx::icReadAndPrepareFab
does (Source/Initialization/Nyx_initcosmo.cpp:15-96): ``<init_dir>/Level_0/Cell``
as a whole, refused when it holds a NaN or when its boxes do not cover exactly
the domain.  It then picks the particle displacement and velocity components for
the IC source as Nyx::initcosmo does for a dark-matter-only run (do_hydro = 0,
:229-294): MUSIC displacement 0..2 and velocity 3..5; nyx displacement 0..2,
which also serve as the velocity (the factors differ).

Arrays are (ncomp, nz, ny, nx): x fastest, one component after another, the
layout ``Box.init_cosmo_1ppc`` takes.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib as _L
from .pm import NyxPMError, _f64, _ptr


def _call(fn, *args):
    err = C.create_string_buffer(512)
    st = fn(*args, err, len(err))
    if st != _L.NYXPM_OK:
        raise NyxPMError(st, err.value.decode(errors="replace"))


def _ivec(v):
    return (C.c_int * 3)(*[int(x) for x in v])


def info(name: str) -> dict:
    """ncomp, ngrow, nboxes and the bounding box (lo, hi) of a MultiFab."""
    out = _L.MultiFabInfo()
    _call(_L.load().nyxpm_multifab_info_read, str(name).encode(), C.byref(out))
    return {"ncomp": out.ncomp, "ngrow": out.ngrow, "nboxes": out.nboxes,
            "lo": tuple(out.lo), "hi": tuple(out.hi), "has_minmax": bool(out.has_minmax)}


def boxes(name: str):
    """(boxes (nboxes, 6) int32 as lo x y z, hi x y z; minmax (nboxes, ncomp, 2) or None)."""
    inf = info(name)
    b = np.zeros((inf["nboxes"], 6), dtype=np.int32)
    mm = np.zeros((inf["nboxes"], inf["ncomp"], 2)) if inf["has_minmax"] else None
    _call(_L.load().nyxpm_multifab_boxes, str(name).encode(), _ptr(b),
          _ptr(mm) if mm is not None else None)
    return b, mm


def read(name: str, comps=None, lo=None, hi=None, reject_nan: bool = False) -> np.ndarray:
    """Components ``comps`` (a range or (first, count); all by default) over
    [lo, hi] (the bounding box by default) -> (ncomp, nz, ny, nx) float64."""
    inf = info(name)
    lo = tuple(inf["lo"] if lo is None else lo)
    hi = tuple(inf["hi"] if hi is None else hi)
    if comps is None:
        c0, nc = 0, inf["ncomp"]
    elif isinstance(comps, range):
        if comps.step != 1 or len(comps) == 0:
            raise ValueError("comps must be a contiguous range")
        c0, nc = comps.start, len(comps)
    else:
        c0, nc = int(comps[0]), int(comps[1])
    shape = (nc, hi[2] - lo[2] + 1, hi[1] - lo[1] + 1, hi[0] - lo[0] + 1)
    out = np.empty(shape, dtype=np.float64)
    flags = _L.NYXPM_MF_REJECT_NAN if reject_nan else 0
    _call(_L.load().nyxpm_multifab_read, str(name).encode(), c0, nc, _ivec(lo), _ivec(hi), flags,
          _ptr(out))
    return out


def write(name: str, data, lo=(0, 0, 0), max_grid_size: int = 32, box_list=None):
    """Writes data (ncomp, nz, ny, nx) -- or (nz, ny, nx), one component -- over
    the region starting at lo, cut into boxes of at most max_grid_size cells per
    edge or into ``box_list`` ((nboxes, 6): lo x y z, hi x y z).  The directory of
    ``name`` is created."""
    d = np.asarray(data, dtype=np.float64)
    if d.ndim == 3:
        d = d[None]
    if d.ndim != 4:
        raise ValueError("data must be (ncomp, nz, ny, nx) or (nz, ny, nx)")
    d = _f64(d)
    nc, nz, ny, nx = d.shape
    lo = tuple(int(v) for v in lo)
    hi = (lo[0] + nx - 1, lo[1] + ny - 1, lo[2] + nz - 1)
    parent = os.path.dirname(str(name))
    if parent:
        os.makedirs(parent, exist_ok=True)
    if box_list is not None:
        bl = np.ascontiguousarray(np.asarray(box_list, dtype=np.int32).reshape(-1, 6))
        nb, bp = len(bl), _ptr(bl)
    else:
        nb, bp = 0, None
    _call(_L.load().nyxpm_multifab_write, str(name).encode(), nc, _ivec(lo), _ivec(hi),
          int(max_grid_size), nb, bp, _ptr(d))


IC_COMPONENTS = {"MUSIC": (0, 3), "nyx": (0, 0)}   # (displacement, velocity) first components


def ic_multifab_name(init_dir: str) -> str:
    return os.path.join(str(init_dir), "Level_0", "Cell")


def read_ic_fields(init_dir: str, source: str, n: int):
    """(disp, vel), each (3, n, n, n), from the IC MultiFab of a periodic n^3
    domain for ic-source "MUSIC" or "nyx"."""
    if source not in IC_COMPONENTS:
        raise ValueError(f"cosmo.ic-source {source!r}: MUSIC or nyx")
    name = ic_multifab_name(init_dir)
    inf = info(name)
    if inf["lo"] != (0, 0, 0) or inf["hi"] != (n - 1,) * 3:
        raise ValueError(f"{name}: the MultiFab covers {inf['lo']}..{inf['hi']}, "
                         f"not the domain (0,0,0)..({n - 1},{n - 1},{n - 1})")
    pd, pv = IC_COMPONENTS[source]
    need = max(pd, pv) + 3
    if inf["ncomp"] < need:
        raise ValueError(f"{name}: {inf['ncomp']} components, ic-source {source} needs {need}")
    f = read(name, reject_nan=True)
    return np.ascontiguousarray(f[pd:pd + 3]), np.ascontiguousarray(f[pv:pv + 3])
