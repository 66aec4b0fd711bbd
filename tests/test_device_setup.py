"""The per-device setup guard of the library (luz_gb300/csrc/device_setup.hpp), built
with the host C++ compiler and run on the CPU: once per level and generation, retried
after a failure, and safe under concurrent host threads."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_device_setup_guard(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "device_setup_check")
    subprocess.run([cxx, "-std=c++17", "-O2", "-pthread", "-Wall", "-Werror", "-o", exe,
                    os.path.join(HERE, "device_setup_check.cpp")], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == "ok"
