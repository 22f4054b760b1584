"""The staged binary32 kernels arm each stage's mbarrier with the byte
count of the copies they issue; a mismatch leaves the barrier incomplete
(the kernel then times out and reports an error).  This compiles the
kernels' own copy-list code for the host and checks, over a sweep of
shapes, that expected and copied bytes agree, that every copy lands inside
its stage without overlap, and that all copies are 16-byte aligned."""
import os
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(ROOT, "raytracer_3d_gb300", "csrc")


def _nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        pytest.skip("nvcc not available")
    return exe


def test_stage_copy_lists_match_barrier_bytes():
    with tempfile.TemporaryDirectory() as tmp:
        out = os.path.join(tmp, "stage_layout_check")
        cmd = [_nvcc(), "-std=c++17", "-O1", "-gencode", "arch=compute_103a,code=sm_103a", "-I", CSRC,
               "-I", os.path.join(ROOT, "include"), os.path.join(HERE, "native", "stage_layout_check.cu"), "-o", out]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        r = subprocess.run([out], capture_output=True, text=True, timeout=300)
        print(r.stdout)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "0 failures" in r.stdout


def test_fast_superbee_selection_is_exact():
    """the fast binary64 step's division-free limiter (integer selection of
    Rj, up or twice one of them) equals phi(up/Rj)*Rj exactly and the
    reference's division form to rounding, over special and random cases"""
    with tempfile.TemporaryDirectory() as tmp:
        out = os.path.join(tmp, "superbee_select_check")
        cmd = [_nvcc(), "-std=c++17", "-O1", "-gencode", "arch=compute_103a,code=sm_103a", "-I", CSRC,
               os.path.join(HERE, "native", "superbee_select_check.cu"), "-o", out]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        r = subprocess.run([out], capture_output=True, text=True, timeout=300)
        print(r.stdout)
        assert r.returncode == 0, r.stdout + r.stderr
        assert " 0 failures" in r.stdout


def test_fast_index_division_is_exact():
    """the fast binary64 step's coordinates divide by invariant divisors
    through one wide multiply and a shift; the quotient equals n / d for
    every divisor up to 70000 and sampled larger ones, at the boundary
    numerators and random ones below 2^31"""
    with tempfile.TemporaryDirectory() as tmp:
        out = os.path.join(tmp, "fastdiv_check")
        cmd = [_nvcc(), "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a", "-I", CSRC,
               os.path.join(HERE, "native", "fastdiv_check.cu"), "-o", out]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        r = subprocess.run([out], capture_output=True, text=True, timeout=300)
        print(r.stdout)
        assert r.returncode == 0, r.stdout + r.stderr
        assert " 0 failures" in r.stdout


def test_binary32_update_rounds_without_bias():
    """the binary32 update's stochastic rounding returns a neighbour of the
    exact sum and has zero mean error over the random words, also for
    increments far below half a unit in the last place"""
    with tempfile.TemporaryDirectory() as tmp:
        out = os.path.join(tmp, "sr_round_check")
        cmd = [_nvcc(), "-std=c++17", "-O1", "-gencode", "arch=compute_103a,code=sm_103a", "-I", CSRC,
               os.path.join(HERE, "native", "sr_round_check.cu"), "-o", out]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        r = subprocess.run([out], capture_output=True, text=True, timeout=300)
        print(r.stdout)
        assert r.returncode == 0, r.stdout + r.stderr
        assert " 0 failures" in r.stdout


@pytest.mark.gpu
def test_fast_superbee_selection_device_matches_host():
    """the device form of the limiter (one block of integer PTX) gives the
    host form's bits on every case of the host check"""
    with tempfile.TemporaryDirectory() as tmp:
        out = os.path.join(tmp, "superbee_select_check")
        cmd = [_nvcc(), "-std=c++17", "-O1", "-gencode", "arch=compute_103a,code=sm_103a", "-I", CSRC,
               os.path.join(HERE, "native", "superbee_select_check.cu"), "-o", out]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        r = subprocess.run([out, "--device"], capture_output=True, text=True, timeout=300)
        print(r.stdout)
        assert r.returncode == 0, r.stdout + r.stderr
        assert " 0 mismatches" in r.stdout
