"""The particle directories of Nyx checkpoints and plotfiles ("DM"): the AMReX
particle container layout Version_Two_Dot_Zero, written by NyxCheckpoint /
WriteNyxPlotFile and read back by Restart.  No GPU.

* round trip through the library's writer and reader, float64 exactly and
  float32 as rounded, per-particle and uniform masses;
* the written directory, parsed independently here the way the reference's
  reader Util/Converters/plotfile2HDF5_particles_amr.py:24-111 parses one
  (Header lines, then per grid at its offset the int32 block of a checkpoint
  and the real block, particle by particle), and its Header and Particle_H text
  line by line;
* a directory laid out by hand with that layout: two levels, three grids in two
  DATA files at non-zero offsets, an empty grid, float32 reals, an extra int
  component, the real components in another order with an extra one, and the
  plotfile form without ids;
* malformed headers are refused with a message.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from nyx_gb300.pm import NyxPMError, particles_info, read_particles_dir, write_particles_dir


def parse_like_the_reference_reader(d):
    """Header and data of an AMReX particle directory, parsed independently."""
    with open(os.path.join(d, "Header")) as f:
        lines = [ln.strip() for ln in f]
    it = iter(lines)
    version = next(it)
    real_t = {"double": np.float64, "single": np.float32}[version.split("_")[-1]]
    dim = int(next(it))
    nr = int(next(it))
    rnames = [next(it) for _ in range(nr)]
    ni = int(next(it))
    inames = [next(it) for _ in range(ni)]
    ckpt = bool(int(next(it)))
    npart = int(next(it))
    next_id = int(next(it))
    finest = int(next(it))
    ngrids = [int(next(it)) for _ in range(finest + 1)]
    grids = [[tuple(int(v) for v in next(it).split()) for _ in range(ng)] for ng in ngrids]
    ints, reals = [], []
    for lvl, lg in enumerate(grids):
        for which, count, where in lg:
            if count == 0:
                continue
            with open(os.path.join(d, f"Level_{lvl}", f"DATA_{which:05d}"), "rb") as f:
                f.seek(where)
                if ckpt:
                    ints.append(np.fromfile(f, dtype=np.int32, count=count * (2 + ni)).reshape(count, 2 + ni))
                reals.append(np.fromfile(f, dtype=real_t, count=count * (dim + nr)).reshape(count, dim + nr))
    return {"version": version, "dim": dim, "real_names": rnames, "int_names": inames,
            "checkpoint": ckpt, "np": npart, "next_id": next_id, "finest": finest, "grids": grids,
            "ints": np.concatenate(ints) if ints else None,
            "reals": np.concatenate(reals) if reals else np.zeros((0, dim + nr))}


def particles(npart, seed=3):
    rng = np.random.default_rng(seed)
    return (rng.random((npart, 3)) * 7.5, rng.standard_normal((npart, 3)) * 300.0,
            1e9 * (1 + rng.random(npart)))


@pytest.mark.parametrize("mass_kind", ["array", "scalar"])
def test_checkpoint_round_trip_float64_exact(tmp_path, mass_kind):
    pos, vel, mass = particles(5000)
    m = mass if mass_kind == "array" else 2.5e9
    d = str(tmp_path / "chk00010" / "DM")
    os.makedirs(os.path.dirname(d))
    write_particles_dir(d, 32, pos, vel, m, checkpoint=True)
    h = particles_info(d)
    assert (h["num_particles"], h["n_real_extra"], h["n_int_extra"], h["is_checkpoint"],
            h["single_precision"], h["finest_level"], h["ngrids"], h["max_next_id"]) == \
        (5000, 4, 0, 1, 0, 0, 1, 5001)
    rp, rv, rm, ids = read_particles_dir(d, with_ids=True)
    assert np.array_equal(rp, pos) and np.array_equal(rv, vel)
    assert np.array_equal(rm, mass if mass_kind == "array" else np.full(5000, 2.5e9))
    assert np.array_equal(ids, np.arange(1, 5001))


def test_plotfile_round_trip_float32_rounded(tmp_path):
    pos, vel, mass = particles(777, seed=4)
    d = str(tmp_path / "DM")
    write_particles_dir(d, 16, pos, vel, mass, checkpoint=False, single_precision=True)
    assert particles_info(d)["single_precision"] == 1 and particles_info(d)["is_checkpoint"] == 0
    rp, rv, rm = read_particles_dir(d)
    assert np.array_equal(rp, pos.astype(np.float32).astype(np.float64))
    assert np.array_equal(rv, vel.astype(np.float32).astype(np.float64))
    assert np.array_equal(rm, mass.astype(np.float32).astype(np.float64))
    with pytest.raises(NyxPMError, match="no particle ids"):
        read_particles_dir(d, with_ids=True)


def test_written_layout_parsed_independently(tmp_path):
    pos, vel, mass = particles(1234, seed=5)
    d = str(tmp_path / "DM")
    write_particles_dir(d, 64, pos, vel, mass, checkpoint=True)
    with open(os.path.join(d, "Header")) as f:
        assert f.read() == ("Version_Two_Dot_Zero_double\n3\n4\nmass\nxvel\nyvel\nzvel\n0\n1\n1234\n"
                            "1235\n0\n1\n0 1234 0\n")
    with open(os.path.join(d, "Level_0", "Particle_H")) as f:
        assert f.read() == "(1 0\n((0,0,0) (63,63,63) (0,0,0))\n)\n"
    r = parse_like_the_reference_reader(d)
    assert r["checkpoint"] and r["np"] == 1234 and r["grids"] == [[(0, 1234, 0)]]
    assert np.array_equal(r["ints"], np.stack([np.arange(1, 1235), np.zeros(1234)], 1))
    assert np.array_equal(r["reals"], np.column_stack([pos, mass, vel]))
    assert os.path.getsize(os.path.join(d, "Level_0", "DATA_00000")) == 1234 * (2 * 4 + 7 * 8)


def write_by_hand(d, checkpoint):
    """Two levels, grids (level, file, count) = (0,0,3) (0,1,0) (0,1,4) (1,0,2) at
    non-zero offsets, float32, real components yvel mass zvel xvel tag, one extra
    int component (plotfile: no ints)."""
    rng = np.random.default_rng(9)
    names = ["yvel", "mass", "zvel", "xvel", "tag"]
    os.makedirs(os.path.join(d, "Level_0"))
    os.makedirs(os.path.join(d, "Level_1"))
    layout = [(0, 0, 3), (0, 1, 0), (0, 1, 4), (1, 0, 2)]
    files, table, expect = {}, [], []
    next_id = 100
    for lvl, which, count in layout:
        key = (lvl, which)
        blob = files.setdefault(key, bytearray(b"\x7f" * (16 + 8 * lvl + 4 * which)))  # leading junk
        where = len(blob)
        rows = rng.random((count, 3 + len(names))).astype(np.float32)
        if checkpoint:
            ints = np.stack([np.arange(next_id, next_id + count), np.full(count, 7),
                             np.full(count, -5)], 1).astype(np.int32)
            blob += ints.tobytes()
        blob += rows.tobytes()
        next_id += count
        table.append((lvl, which, count, where))
        for r in rows.astype(np.float64):
            expect.append((r[0:3], r[3 + 3], r[3 + 0], r[3 + 2], r[3 + 1]))   # pos, vx, vy, vz, m
    for (lvl, which), blob in files.items():
        with open(os.path.join(d, f"Level_{lvl}", f"DATA_{which:05d}"), "wb") as f:
            f.write(bytes(blob))
    hdr = ["Version_Two_Dot_Zero_single", "3", str(len(names)), *names, "1", "flag",
           "1" if checkpoint else "0", str(sum(c for _, _, c in layout)), str(next_id), "1", "3", "1"]
    hdr += [f"{w} {c} {o}" for lvl, w, c, o in table]
    with open(os.path.join(d, "Header"), "w") as f:
        f.write("\n".join(hdr) + "\n")
    pos = np.array([e[0] for e in expect])
    vel = np.array([[e[1], e[2], e[3]] for e in expect])
    mass = np.array([e[4] for e in expect])
    return pos, vel, mass


@pytest.mark.parametrize("checkpoint", [True, False])
def test_reads_a_directory_laid_out_by_hand(tmp_path, checkpoint):
    d = str(tmp_path / "DM")
    pos, vel, mass = write_by_hand(d, checkpoint)
    h = particles_info(d)
    assert (h["num_particles"], h["finest_level"], h["ngrids"], h["n_real_extra"], h["n_int_extra"],
            h["single_precision"], h["is_checkpoint"]) == (9, 1, 4, 5, 1, 1, int(checkpoint))
    out = read_particles_dir(d, with_ids=checkpoint)
    assert np.array_equal(out[0], pos) and np.array_equal(out[1], vel) and np.array_equal(out[2], mass)
    if checkpoint:
        assert np.array_equal(out[3], np.arange(100, 109))
    r = parse_like_the_reference_reader(d)
    assert np.array_equal(r["reals"][:, :3].astype(np.float64), pos)


@pytest.mark.parametrize("edit,msg", [
    (lambda L: ["Version_One_Dot_One"] + L[1:], "version"),
    (lambda L: L[:1] + ["2"] + L[2:], "dimension"),
    (lambda L: L[:-1] + ["0 1233 0"], "grids hold"),
    (lambda L: L[:-1] + ["0 1234"], "grid line"),
])
def test_malformed_headers_are_refused(tmp_path, edit, msg):
    pos, vel, mass = particles(1234, seed=6)
    d = str(tmp_path / "DM")
    write_particles_dir(d, 8, pos, vel, mass)
    with open(os.path.join(d, "Header")) as f:
        lines = f.read().splitlines()
    with open(os.path.join(d, "Header"), "w") as f:
        f.write("\n".join(edit(lines)) + "\n")
    with pytest.raises(NyxPMError, match=msg):
        read_particles_dir(d)
