"""The kernels' 64-row column algebra (csrc/wordslice.cuh: getValue, maxXScore, differenceMasks,
mergeTwoSlices, changedMinScore, getNextSlice, the component queue's heap, IUPAC masks),
compiled for the host and checked on random columns against cell-by-cell restatements and
std::priority_queue (tests/harness/wordslice_props.cpp)."""
import os
import subprocess

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
BUILD = os.path.join(ROOT, "tests", "_build")
SRC = os.path.join(ROOT, "tests", "harness", "wordslice_props.cpp")
HDR = os.path.join(ROOT, "graphaligner_gb300", "csrc", "wordslice.cuh")


def test_column_algebra_matches_cell_by_cell():
    os.makedirs(BUILD, exist_ok=True)
    exe = os.path.join(BUILD, "wordslice_props")
    if not os.path.exists(exe) or os.path.getmtime(exe) < max(os.path.getmtime(SRC), os.path.getmtime(HDR)):
        subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-o", exe, SRC], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0 and out.stdout.startswith("ok"), out.stdout + out.stderr
