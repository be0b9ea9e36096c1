"""Copies the reference's own golden vectors and test inputs into
tests/golden/ref/ so that the test suite does not need the reference tree.

Run from the repository root with the path of a reference checkout:
    python tests/golden/make_golden.py REF

The copied files are data the reference's test suite asserts on
(tests/test_kpar_fast.py:12-31) or feeds to ALPS (tests/*.in,
distribution/*_dist.in) and to its interpolation program
(interpolation/test_interp.in, test_interp_coarse.array); they are copied
byte for byte.
"""
import os
import shutil
import sys

if len(sys.argv) != 2:
    sys.exit("usage: python tests/golden/make_golden.py REF  (REF = a checkout of the reference)")
REF = sys.argv[1]
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref")

FILES = [
    "tests/test_kpar_fast.scan_kpara_1.root_1",
    "tests/test_kpar_fast.eigen_kpara_1.root_1",
    "tests/test_kpar_fast.heat_kpara_1.root_1",
    "tests/test_kpar_fast.heat_mech_kpara_1.root_1",
]
INPUT_DIRS = ["tests", "distribution", "interpolation"]
DATA_FILES = ["interpolation/test_interp_coarse.array"]


def main():
    os.makedirs(OUT, exist_ok=True)
    for f in FILES:
        shutil.copyfile(os.path.join(REF, f), os.path.join(OUT, os.path.basename(f)))
    for d in INPUT_DIRS:
        for name in sorted(os.listdir(os.path.join(REF, d))):
            if name.endswith(".in") and not name.startswith("Makefile"):
                sub = os.path.join(OUT, "inputs", d)
                os.makedirs(sub, exist_ok=True)
                shutil.copyfile(os.path.join(REF, d, name), os.path.join(sub, name))
    for f in DATA_FILES:
        sub = os.path.join(OUT, "inputs", os.path.dirname(f))
        os.makedirs(sub, exist_ok=True)
        shutil.copyfile(os.path.join(REF, f), os.path.join(sub, os.path.basename(f)))
    print("wrote", OUT)


if __name__ == "__main__":
    main()
