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
