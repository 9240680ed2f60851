"""The fixed-point w-screen phase (wsclean_gb300/csrc/screen.cuh) on the CPU.

Column pass B forms the screen of plane q from per-pixel terms computed once
per plan: a + q k in wrapping 32-bit fixed-point turns plus q r in FP32.  The
header is compiled for the host and checked against (w0 + q dw) nu modulo one
turn in extended precision for random plans, pixels and plane indices up to
2^20; the error bound (6e-8 turns) is in the test program.  The GPU side runs
the same header and is checked against the FP64 direct transform by the
parity tests (among them a case with about 650 w planes).
"""
import os
import re
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "screen_phase_test.cpp")


def test_screen_phase_within_two_fp32_roundings(tmp_path):
    exe = str(tmp_path / "screen_phase_test")
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I",
                    os.path.join(ROOT, "wsclean_gb300", "csrc"), SRC, "-o", exe],
                   check=True, capture_output=True)
    r = subprocess.run([exe, "2000000", "7"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    n, err = re.search(r"cases (\d+) max_err_turns (\S+)", r.stdout).groups()
    assert int(n) == 2000000 and float(err) <= 6e-8
