"""AMReX MultiFab files (VisMF, header version 1): the reader and writer against
MultiFabs AMReX itself wrote (tests/golden/vismf_slice_00340, copied from the
reference's Util/SliceUtils/slice_00340 by tests/golden/make_vismf_fixture.py),
round trips, the float32 / big-endian FAB path, the errors, and the IC-field
selection of Nyx::icReadAndPrepareFab + Nyx::initcosmo.  Host code only.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from nyx_gb300 import multifab as M
from nyx_gb300.pm import NyxPMError

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "vismf_slice_00340")


def _box_slices(b, lo):
    lo = np.asarray(lo)
    a, z = b[:3] - lo, b[3:] - lo
    return (slice(None), slice(a[2], z[2] + 1), slice(a[1], z[1] + 1), slice(a[0], z[0] + 1))


@pytest.mark.parametrize("name,ncomp,lo,hi", [
    ("State_z", 6, (0, 0, 16), (31, 31, 16)),
    ("Diag_x", 2, (16, 0, 0), (16, 31, 31)),
])
def test_reader_matches_the_min_max_amrex_wrote(name, ncomp, lo, hi):
    """Every per-box, per-component min and max of the AMReX-written header equals
    the one of the values read (17 significant digits: exact)."""
    path = os.path.join(GOLD, name)
    inf = M.info(path)
    assert (inf["ncomp"], inf["ngrow"], inf["nboxes"]) == (ncomp, 0, 16)
    assert inf["lo"] == lo and inf["hi"] == hi and inf["has_minmax"]
    boxes, mm = M.boxes(path)
    f = M.read(path)
    assert f.shape == (ncomp, hi[2] - lo[2] + 1, hi[1] - lo[1] + 1, hi[0] - lo[0] + 1)
    for i, b in enumerate(boxes):
        sub = f[_box_slices(b, lo)].reshape(ncomp, -1)
        assert np.array_equal(sub.min(axis=1), mm[i, :, 0])
        assert np.array_equal(sub.max(axis=1), mm[i, :, 1])


@pytest.mark.parametrize("name", ["State_z", "Diag_x"])
def test_writer_reproduces_the_amrex_files(name, tmp_path):
    """Written with the fixture's boxes, every FAB (text header + float64 values)
    is byte for byte the one AMReX wrote, and the header is the same text apart
    from the FabOnDisk lines (AMReX spread the FABs over 4 files, we use one)."""
    path = os.path.join(GOLD, name)
    inf = M.info(path)
    boxes, _ = M.boxes(path)
    f = M.read(path)
    out = str(tmp_path / name)
    M.write(out, f, lo=inf["lo"], box_list=boxes)

    def fab_list(hdr, d):
        return [(os.path.join(d, ln.split()[1]), int(ln.split()[2]))
                for ln in hdr.splitlines() if ln.startswith("FabOnDisk:")]

    ref_h, my_h = open(path + "_H").read(), open(out + "_H").read()
    for i, ((rf, ro), (mf, mo)) in enumerate(zip(fab_list(ref_h, GOLD), fab_list(my_h, str(tmp_path)))):
        rb = open(rf, "rb").read()[ro:]
        size = rb.index(b"\n") + 1 + 8 * inf["ncomp"] * int(np.prod(boxes[i, 3:] - boxes[i, :3] + 1))
        assert open(mf, "rb").read()[mo:mo + size] == rb[:size]

    def strip(h):
        return [ln for ln in h.splitlines() if not ln.startswith("FabOnDisk:")]
    assert strip(my_h) == strip(ref_h)
    assert my_h.endswith(",\n\n") and ref_h.endswith(",\n\n")


def test_round_trip_chopped_subregion_and_components(tmp_path):
    rng = np.random.default_rng(7)
    data = rng.standard_normal((3, 9, 12, 20))
    name = str(tmp_path / "sub" / "Cell")
    M.write(name, data, lo=(4, -2, 1), max_grid_size=8)
    inf = M.info(name)
    assert inf["lo"] == (4, -2, 1) and inf["hi"] == (23, 9, 9)
    boxes, mm = M.boxes(name)
    assert len(boxes) == 3 * 2 * 2 and np.all(boxes[:, 3:] - boxes[:, :3] + 1 <= 8)
    assert np.array_equal(M.read(name), data)
    part = M.read(name, comps=(1, 2), lo=(6, 0, 3), hi=(17, 5, 8))
    assert np.array_equal(part, data[1:3, 2:8, 2:8, 2:14])
    assert np.array_equal(M.read(name, comps=range(2, 3)), data[2:3])
    for i, b in enumerate(boxes):
        sub = data[_box_slices(b, (4, -2, 1))].reshape(3, -1)
        assert np.array_equal(sub.min(axis=1), mm[i, :, 0]) and np.array_equal(sub.max(axis=1), mm[i, :, 1])


def _write_handmade(tmp_path, name, fabs, ncomp, ngrow_text="0"):
    """A version-1 MultiFab written by hand: fabs = [(valid lo, hi, fab lo, hi,
    nbytes, big_endian, values (ncomp, fab cells))]."""
    data = b""
    lines = []
    offs = []
    for vlo, vhi, flo, fhi, nb, big, vals in fabs:
        fmt = "(64 11 52 0 1 12 0 1023)" if nb == 8 else "(32 8 23 0 1 9 0 127)"
        order = " ".join(str(i + 1) for i in range(nb))
        if not big:
            order = " ".join(str(nb - i) for i in range(nb))
        head = (f"FAB (({nb}, {fmt}),({nb}, ({order})))(({flo[0]},{flo[1]},{flo[2]}) "
                f"({fhi[0]},{fhi[1]},{fhi[2]}) (0,0,0)) {ncomp}\n").encode()
        dt = (">" if big else "<") + ("f8" if nb == 8 else "f4")
        offs.append(len(data))
        data += head + np.asarray(vals, dtype=dt).tobytes()
        lines.append(f"(({vlo[0]},{vlo[1]},{vlo[2]}) ({vhi[0]},{vhi[1]},{vhi[2]}) (0,0,0))")
    with open(tmp_path / (name + "_D_00000"), "wb") as f:
        f.write(data)
    hdr = f"1\n1\n{ncomp}\n{ngrow_text}\n({len(fabs)} 0\n" + "\n".join(lines) + "\n)\n"
    hdr += f"{len(fabs)}\n" + "".join(f"FabOnDisk: {name}_D_00000 {o}\n" for o in offs)
    with open(tmp_path / (name + "_H"), "w") as f:
        f.write(hdr)
    return str(tmp_path / name)


def test_float32_big_endian_fabs_with_ghost_cells(tmp_path):
    """FABs of big-endian float32 whose boxes carry one ghost cell (ngrow 1,
    written as an IntVect): the valid cells are read, the ghosts skipped."""
    rng = np.random.default_rng(3)
    full = rng.standard_normal((2, 4, 4, 8)).astype(np.float32)     # valid region 8 x 4 x 4
    fabs = []
    for x0 in (0, 4):
        g = np.pad(full[:, :, :, x0:x0 + 4], ((0, 0), (1, 1), (1, 1), (1, 1)), constant_values=np.nan)
        fabs.append(((x0, 0, 0), (x0 + 3, 3, 3), (x0 - 1, -1, -1), (x0 + 4, 4, 4), 4, True,
                     g.reshape(2, -1)))
    name = _write_handmade(tmp_path, "F32", fabs, 2, ngrow_text="(1,1,1)")
    inf = M.info(name)
    assert inf["ngrow"] == 1 and not inf["has_minmax"]
    got = M.read(name, reject_nan=True)
    assert np.array_equal(got, full.astype(np.float64))


def test_errors(tmp_path):
    data = np.zeros((1, 4, 4, 4))
    data[0, 1, 2, 3] = np.nan
    name = str(tmp_path / "Nan")
    M.write(name, data, max_grid_size=2)
    assert np.isnan(M.read(name)).sum() == 1
    with pytest.raises(NyxPMError, match="NaN in component 0"):
        M.read(name, reject_nan=True)
    with pytest.raises(NyxPMError, match="do not cover"):
        M.read(name, lo=(0, 0, 0), hi=(4, 3, 3))
    with pytest.raises(NyxPMError, match="components"):
        M.read(name, comps=(0, 2))
    with pytest.raises(NyxPMError, match="cannot read"):
        M.info(str(tmp_path / "Missing"))
    with open(str(tmp_path / "V2") + "_H", "w") as f:
        f.write("2\n1\n1\n0\n(0 0\n)\n0\n")
    with pytest.raises(NyxPMError, match="version 2"):
        M.info(str(tmp_path / "V2"))
    with pytest.raises(NyxPMError, match="tile"):
        M.write(str(tmp_path / "Bad"), np.zeros((1, 2, 2, 2)), box_list=[[0, 0, 0, 1, 1, 0]])
    # a data file cut short
    name2 = str(tmp_path / "Short")
    M.write(name2, np.ones((1, 4, 4, 4)), max_grid_size=4)
    with open(name2 + "_D_00000", "r+b") as f:
        f.truncate(100)
    with pytest.raises(NyxPMError, match="short FAB data"):
        M.read(name2)


def test_ic_fields_follow_initcosmo_component_choice(tmp_path):
    """MUSIC (dark matter only): displacement = components 0..2, velocity 3..5;
    nyx: both from 0..2.  The MultiFab must cover exactly the domain."""
    n = 6
    f = np.random.default_rng(11).standard_normal((6, n, n, n))
    init = tmp_path / "ics"
    M.write(M.ic_multifab_name(str(init)), f, max_grid_size=4)
    d, v = M.read_ic_fields(str(init), "MUSIC", n)
    assert np.array_equal(d, f[0:3]) and np.array_equal(v, f[3:6])
    d, v = M.read_ic_fields(str(init), "nyx", n)
    assert np.array_equal(d, f[0:3]) and np.array_equal(v, f[0:3])
    with pytest.raises(ValueError, match="not the domain"):
        M.read_ic_fields(str(init), "MUSIC", n + 2)
    with pytest.raises(ValueError, match="MUSIC or nyx"):
        M.read_ic_fields(str(init), "grafic", n)
    M.write(M.ic_multifab_name(str(tmp_path / "small")), f[:3], max_grid_size=4)
    with pytest.raises(ValueError, match="needs 6"):
        M.read_ic_fields(str(tmp_path / "small"), "MUSIC", n)
