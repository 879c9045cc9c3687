"""Host-side lowering logic of the engine, compiled for the host and checked without a GPU."""

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "chemtensor_gb300", "csrc")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _build_and_run(tmp_path, name, sources, libs):
    exe = tmp_path / name
    cmd = ["g++", "-O2", "-std=c++17", f"-I{CSRC}", f"-I{CUDA}/include", *sources, *libs, "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True)
    env = dict(os.environ, LD_LIBRARY_PATH=f"{CUDA}/lib64:" + os.environ.get("LD_LIBRARY_PATH", ""))
    out = subprocess.run([str(exe)], capture_output=True, text=True, env=env)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "mismatches: 0" in out.stdout


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_block_enumeration_matches_brute_force(tmp_path):
    _build_and_run(tmp_path, "check_meta",
                   [os.path.join(ROOT, "tests", "host", "check_meta.cpp"), os.path.join(CSRC, "ctg_meta.cpp")],
                   [f"-L{CUDA}/lib64", "-lcudart"])


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_cluster_jacobi_schedule_covers_every_pair_once(tmp_path):
    _build_and_run(tmp_path, "check_schedule", [os.path.join(ROOT, "tests", "host", "check_schedule.cpp")], [])
