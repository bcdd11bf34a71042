"""The integer double -> double-float split of the FP64 tile and phase
kernels (qvm_gb300/csrc/cplx.h: df_split_int) equals the FP64 form it
replaces bit for bit: its host build is run against FP64 arithmetic on 4 M
random and adversarial doubles (no GPU needed)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "qvm_gb300", "csrc")


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else shutil.which("nvcc")


def test_integer_split_matches_fp64(tmp_path):
    nvcc = _nvcc()
    if not nvcc:
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "dfsplit_check")
    subprocess.run([nvcc, "-O2", "-std=c++17", "-I", CSRC, "-o", exe,
                    os.path.join(HERE, "dfsplit_check.cu")], check=True, capture_output=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches 0" in r.stdout
