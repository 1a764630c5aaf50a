"""Generate tests/golden/zeldovich_pancake.json from the reference itself.

Two reference artefacts are used, both from Nyx's Zel'dovich pancake test
(Exec/GravityTests/zeldovich_dm):

1. ``analysis/zeldovich.py`` is imported as is and evaluated for the
   analytic pancake solution x(q, z), v(q, z) on a 32-point lattice at the
   redshifts the tests stop at;
2. ``ics/generate_zeldovich_ics.cpp`` is compiled by ``oracle/Makefile``
   (target ``ref``) into ``oracle/_ref/`` and run in a scratch directory; its
   parameter file and the first particles it writes are stored so that the
   tests can check their own IC construction against the reference generator.

Run with NYX_REFERENCE set to the Nyx source tree:

    make -C oracle ref REF=$NYX_REFERENCE && python tests/golden/make_zeldovich_golden.py
"""
from __future__ import annotations

import csv
import importlib.util
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

REF = os.environ.get("NYX_REFERENCE", "")
if not REF:
    sys.exit("set NYX_REFERENCE to the Nyx source tree")
HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
GEN = os.path.join(REPO, "oracle", "_ref", "generate_zeldovich_ics")

# lattices of the tests: n cells per dimension, one particle per cell centre
# (the 64 lattice is the resolution check's finer grid)
N_LATTICE = 32
N_LATTICE_FINE = 64
Z_STOPS = [100.0, 50.0, 30.0, 20.0]
N_SAMPLE = 256


def load_reference_zeldovich():
    path = os.path.join(REF, "Exec/GravityTests/zeldovich_dm/analysis/zeldovich.py")
    spec = importlib.util.spec_from_file_location("nyx_ref_zeldovich", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def run_generator():
    if not os.path.exists(GEN):
        subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "ref"], check=True)
    with tempfile.TemporaryDirectory() as tmp:
        subprocess.run([GEN], cwd=tmp, check=True, stdout=subprocess.DEVNULL)
        with open(os.path.join(tmp, "zeldovich_params.csv")) as f:
            rows = list(csv.reader(f))
        params = {k: float(v) for k, v in zip(rows[0], rows[1]) if k}
        sample = []
        with open(os.path.join(tmp, "zeldovich_particles.ascii")) as f:
            count = int(f.readline())
            for _ in range(N_SAMPLE):
                sample.append([float(t) for t in f.readline().split()])
    return params, count, sample


def main():
    zel = load_reference_zeldovich()
    params, count, sample = run_generator()
    L = params["box_length"]
    k = params["k"]
    offset = params["offset"]
    H0 = params["H_0"]
    z_c = params["caustic_z"]
    def lattice_stops(nl):
        q = (np.arange(nl) + 0.5) * (L / nl)
        stops = []
        for z in Z_STOPS:
            qq = q + offset
            x = zel.perturbed_x(qq, z, z_c, k) - offset
            v = zel.perturbed_v_x(qq, z, z_c, k, H0)
            stops.append({"z": z, "a": float(zel.get_scale_factor(z)), "x": list(map(float, x)),
                          "xdot": list(map(float, v))})
        return q, stops

    q, stops = lattice_stops(N_LATTICE)
    q_fine, stops_fine = lattice_stops(N_LATTICE_FINE)
    out = {
        "source": "Exec/GravityTests/zeldovich_dm analysis/zeldovich.py + ics/generate_zeldovich_ics.cpp",
        "params": params,
        "generator_particle_count": count,
        "generator_sample": sample,
        "n_lattice": N_LATTICE,
        "q": list(map(float, q)),
        "stops": stops,
        "lattice_fine": {"n_lattice": N_LATTICE_FINE, "q": list(map(float, q_fine)),
                         "stops": stops_fine},
    }
    with open(os.path.join(HERE, "zeldovich_pancake.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", os.path.join(HERE, "zeldovich_pancake.json"), "generator particles:", count)


if __name__ == "__main__":
    sys.exit(main())
