"""The photon gather's float-float range decisions against double.

The GPU gather decides "within the radius" and the k-nearest ordering key
without FP64 (sray_gb300/csrc/range_ff.h).  This compiles that same header
for the host (gcc, -ffp-contract=off: the device build has no contraction
either) and checks, on random and adversarial points, that every case it
decides matches the reference's double computation and that it leaves only
a small fraction to the double fallback.
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "sray_gb300", "csrc")


def test_range_ff_matches_double(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = str(tmp_path / "gather_ff_check")
    subprocess.run([cc, "-O2", "-std=c99", "-ffp-contract=off", "-I", CSRC, "-o", exe,
                    os.path.join(HERE, "gather_ff_check.c"), "-lm"], check=True)
    out = subprocess.run([exe, "3000000"], check=True, capture_output=True, text=True)
    n, fall, bad = (int(x) for x in out.stdout.split())
    assert n == 3000000
    assert bad == 0, out.stderr
    # ties and near-boundary sums go to the double path; they must stay rare
    assert fall < 0.05 * n, fall
