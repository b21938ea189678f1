"""CPU check of the strain-relative stable Neo-Hookean forms used by the FP32 element passes (elem_math.cuh:
snh_eval_small in 3D, snh2_eval_small in 2D): tests/host_math_check.cu, built with nvcc as host code,
compares them with the direct formulas (FP64) over random materials and strains from 1e-4 to 3e-1.
FP64: the forms are the same functions (energy to 1e-9 of its magnitude sum, where the direct formula's
own cancellation dominates; stress to 1e-10).  FP32: energy within 1e-6 of the magnitude sum and stress
within 2e-6 relative, the FP32 rounding level that lets the mixed path's early iterations run in FP32.
The 3D increment form (snh_increment, the mixed Newton's last iterations) against the direct formulas'
differences in long double over reference strains 1e-4 .. 3e-1 and increments 1e-7 .. 1e-1 of them: FP32
stress increments within 5e-6 of their own size and energy increments within 1e-6 of the increment's
scale, so the rounding follows the increment, not the stress; FP64 within 1e-7 (the long-double
reference's own limit at the smallest increments)."""
import os
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    return None


def test_strain_relative_forms_match_direct_formulas():
    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("nvcc not available")
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "host_math_check")
        cmd = [nvcc, "-std=c++17", "-O2", "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "ssim_gb300", "csrc"),
               "-x", "cu", os.path.join(HERE, "host_math_check.cu"), "-o", exe]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    rows = {line.split()[0]: [float(v) for v in line.split()[1:]] for line in out if line.strip()}
    for dim in ("3d", "2d"):
        e64, p64, e32, p32 = rows[dim]
        assert e64 <= 1e-9 and p64 <= 1e-10, (dim, rows[dim])
        assert e32 <= 1e-6 and p32 <= 2e-6, (dim, rows[dim])
    e64, p64, e32, p32 = rows["inc"]
    assert e64 <= 1e-7 and p64 <= 1e-7, rows["inc"]
    assert e32 <= 1e-6 and p32 <= 5e-6, rows["inc"]
