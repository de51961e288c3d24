"""A C++ host program that drives the C ABI in the reference's call order:
tests/abi_replay/he1d_06_replay.cpp replays T_He1d_04 (relaxation, restart
files) and T_He1d_06 (restart load, SIL + RK4 split steps, energy and norm
checks against the golden values).  Built with g++ against
include/cody_gpu.h and libcodygpu.so; run on the GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "abi_replay", "he1d_06_replay.cpp")
OUT = os.path.join(ROOT, "tests", "abi_replay", "_build")


def _build():
    from codyfortran_gb300 import build
    lib = build.build()
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, "he1d_06_replay")
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    cmd = [cxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
           "-L", os.path.dirname(lib), "-lcodygpu", f"-Wl,-rpath,{os.path.dirname(lib)}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_replay_driver_compiles_against_the_header():
    """The driver compiles and links against the C ABI (no GPU needed)."""
    exe = _build()
    assert os.path.exists(exe)


@pytest.mark.gpu
def test_replay_he1d_04_06_call_order(tmp_path, golden):
    exe = _build()
    g04 = golden["he1d_04_mctdhf_imag"]["checks"][0]["golden"]
    g06 = golden["he1d_06_mctdhf_split_sil"]["checks"][1]["golden"]
    r = subprocess.run([exe, str(tmp_path) + "/", repr(g04), repr(g06)], capture_output=True, text=True, timeout=600)
    print(r.stdout, r.stderr)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "OK" in r.stdout
    # the restart files the host program wrote and read, in the reference's names
    names = sorted(os.listdir(tmp_path))
    assert "coeffs.in" in names and "orb01_01.in" in names
