"""The C++ host path: include/mcell_gb300_event.hpp (the event class MCell4's World
would create) driven by a scheduler-like loop, compiled with g++ against the
engine library (tests/cpp/event_driver.cpp)."""
import subprocess

import pytest

from tests import harness as H

pytestmark = pytest.mark.gpu


def test_cpp_event_driver(tmp_path):
    exe = tmp_path / "event_driver"
    lib = H.ROOT / "mcell_gb300" / "_lib"
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", str(H.ROOT / "include"), str(H.ROOT / "tests" / "cpp" /
                    "event_driver.cpp"), "-L", str(lib), "-lmcell_gb300", f"-Wl,-rpath,{lib}", "-o", str(exe)],
                   check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
