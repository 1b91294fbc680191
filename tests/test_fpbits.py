"""The integer FP64 <-> FP32 conversions and FP64 comparisons of the admission pass and the row
epilogues (csrc/fpbits.h), compiled for the host and checked against the C library (hi/lo split
bit for bit, directed bounds nearest inside the normal range, exact widening of either sign, IEEE
comparisons with NaNs and signed zeros, the check's division filter never skipping a quotient
above the running maximum, and the conversions rounded to nearest, up and down equal to the C
library's under its rounding modes)."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / 'hypergrey-sih-26_gb300' / 'csrc'


@pytest.mark.skipif(shutil.which('g++') is None, reason='needs g++')
def test_fpbits_conversions_match_the_c_library(tmp_path):
    exe = tmp_path / 'fpbits_check'
    subprocess.run(['g++', '-O2', '-std=c++17', '-ffp-contract=off', '-frounding-math', '-I', str(CSRC),
                    str(ROOT / 'tests' / 'fpbits_check.cpp'), '-o', str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert 'failures 0' in out.stdout
    n_split = int(out.stdout.split('split ')[1].split()[0])
    assert n_split > 100000  # the window holds a good share of the random patterns
    skipped = int(out.stdout.split('skipped ')[1].split(')')[0])
    assert int(out.stdout.split('directed ')[1].split()[0]) > 1000000  # three directions per value
    assert skipped > 100000  # the filter's "no" is exercised, near the boundary included
