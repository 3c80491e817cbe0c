"""The solver's shared-reciprocal division (Markstein's method, dvd_r in
smap_solve.cuh) against IEEE division, bit for bit, on 2^32 random operand
pairs per exponent range: narrow, the solver's data, the edge of the fast
path's guard (+-500), and the full range, where the guard falls back."""
import subprocess
from pathlib import Path

import pytest

from fedm_loader import build

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


def test_shared_reciprocal_division_is_ieee_division(tmp_path):
    exe = tmp_path / "division_check"
    subprocess.run([build.NVCC, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                    "-I", str(ROOT / "fastedm-r_gb300" / "csrc"), "-o", str(exe),
                    str(ROOT / "tests" / "division_check.cu")], check=True)
    r = subprocess.run([str(exe), "4", "60", "500", "1022"], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count(" 0 differ") == 4
