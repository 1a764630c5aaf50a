"""Copies two MultiFabs of the reference's slice fixture (Util/SliceUtils/slice_00340:
State_z, 6 components on 16 boxes of a 32 x 32 x 1 slice, and Diag_x, 2 components
on a 1 x 32 x 32 slice) into tests/golden/vismf_slice_00340/.  They are AMReX VisMF
files written by AMReX itself: the golden input of the MultiFab reader and writer
tests.  Run from the repository root:

    python tests/golden/make_vismf_fixture.py <Nyx source tree>
"""
import os
import shutil
import sys

if len(sys.argv) != 2:
    sys.exit("usage: make_vismf_fixture.py <Nyx source tree>")
SRC = os.path.join(sys.argv[1], "Util", "SliceUtils", "slice_00340")
DST = os.path.join(os.path.dirname(os.path.abspath(__file__)), "vismf_slice_00340")

os.makedirs(DST, exist_ok=True)
for name in sorted(os.listdir(SRC)):
    if name.startswith(("State_z", "Diag_x")):
        shutil.copyfile(os.path.join(SRC, name), os.path.join(DST, name))
        print(name)
