"""The integer binary64 multiply and add of quids_gb300/csrc/softfp64.cuh
(the device's complex magnitude products) against the host's IEEE-754
arithmetic, bit for bit: 63 million operations over operand families that
reach exact ties, cancellations, every exponent gap and the edges of the
normal range.  The same source is compiled for the host here."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "softfp", "softfp_check.cpp")


@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
@pytest.mark.parametrize("seed", [1, 2])
def test_soft_fp64_equals_ieee(tmp_path, seed):
    exe = tmp_path / "softfp_check"
    subprocess.run(["g++", "-O2", "-std=c++17", SRC, "-o", str(exe)], check=True)
    r = subprocess.run([str(exe), "1500000", str(seed)], capture_output=True, text=True)
    checked, bad = (int(x) for x in r.stdout.split())
    assert checked == 31_500_000 and bad == 0, r.stderr
