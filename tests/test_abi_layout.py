"""The ctypes mirrors of the public structs (nyx_gb300/_lib.py) against the
C header (include/nyxpm.h): a probe compiled with the host C compiler prints
every struct's size and each mirrored field's offset, which must equal the
ctypes layout.  A field renamed, added or reordered on one side only fails
here (the probe does not compile, or an offset or size differs).  No GPU.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess

import pytest

from nyx_gb300 import _lib as L

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

MIRRORS = {
    "nyxpm_params": L.Params,
    "nyxpm_solve_info": L.SolveInfo,
    "nyxpm_step_info": L.StepInfo,
    "nyxpm_dt_params": L.DtParams,
    "nyxpm_particle_header": L.ParticleHeader,
    "nyxpm_multifab_info": L.MultiFabInfo,
    "nyxpm_tuning": L.Tuning,
    "nyxpm_ensemble_info": L.EnsembleInfo,
    "nyxpm_profile": L.Profile,
}


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no host C compiler")
def test_ctypes_mirrors_match_the_header(tmp_path):
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "nyxpm.h"', "int main(void) {"]
    for cname, st in MIRRORS.items():
        lines.append(f'    printf("{cname} %zu\\n", sizeof({cname}));')
        for field, _ in st._fields_:
            lines.append(f'    printf("{cname}.{field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = dict(line.rsplit(" ", 1) for line in out if line)
    for cname, st in MIRRORS.items():
        assert int(got[cname]) == C.sizeof(st), cname
        for field, _ in st._fields_:
            assert int(got[f"{cname}.{field}"]) == getattr(st, field).offset, (cname, field)


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no host C compiler")
def test_multilevel_field_codes_match_the_header(tmp_path):
    """nyx_gb300.amr.FIELDS (the `which` argument of nyxpm_amr_field) against the
    NYXPM_AMR_* constants of the header, through a probe compiled against it."""
    from nyx_gb300.amr import FIELDS
    names = {"rho": "NYXPM_AMR_RHO", "phi": "NYXPM_AMR_PHI", "gx": "NYXPM_AMR_GX",
             "gy": "NYXPM_AMR_GY", "gz": "NYXPM_AMR_GZ", "mass": "NYXPM_AMR_MASS"}
    assert set(names) == set(FIELDS)
    src = tmp_path / "codes.c"
    src.write_text("#include <stdio.h>\n#include \"nyxpm.h\"\nint main(void) {\n" +
                   "".join(f'    printf("{k} %d\\n", (int){v});\n' for k, v in names.items()) +
                   "    return 0;\n}\n")
    exe = tmp_path / "codes"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    assert {out[i]: int(out[i + 1]) for i in range(0, len(out), 2)} == FIELDS
