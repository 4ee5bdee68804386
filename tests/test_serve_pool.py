"""Serving engine slot bookkeeping on the host (no GPU): compiles tests/serve_pool_check.cpp
against torchfsm_gb300/csrc/fsm_serve_pool.h with the host C++ compiler and runs its randomised
admission / tick / leave / cancel / compaction check for several seeds."""

import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "torchfsm_gb300", "csrc")


@pytest.fixture(scope="module")
def pool_check_exe(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path_factory.mktemp("serve_pool") / "serve_pool_check")
    subprocess.run([cxx, "-std=c++17", "-O1", "-Wall", "-Werror", "-I", CSRC,
                    os.path.join(HERE, "serve_pool_check.cpp"), "-o", exe], check=True)
    return exe


@pytest.mark.parametrize("seed", [1, 2, 3, 4])
def test_slot_pool_invariants(pool_check_exe, seed):
    res = subprocess.run([pool_check_exe, str(seed)], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0 and res.stdout.strip() == "ok", res.stdout + res.stderr
