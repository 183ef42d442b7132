"""The autotuner's persisted cache (pargo_gb300/csrc/tune_cache.h), host
code only: round trips, foreign and malformed files, the path rules and the
write through a temporary file (also from two threads at once), checked by
a C++ driver (tests/cpp/tune_cache_check.cpp) built against the same header
the library compiles."""
import os
import subprocess

from conftest import ROOT


def test_tune_cache_file(tmp_path):
    exe = tmp_path / "tune_cache_check"
    scratch = tmp_path / "scratch"
    scratch.mkdir()
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror",
           "-I" + os.path.join(ROOT, "pargo_gb300", "csrc"),
           os.path.join(ROOT, "tests", "cpp", "tune_cache_check.cpp"), "-o", str(exe), "-pthread"]
    subprocess.run(cmd, check=True)
    r = subprocess.run([str(exe), str(scratch)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
