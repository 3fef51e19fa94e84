"""The integer form of the controlled loop's time tests (csrc/va_endtests.h)
against the FP64 expressions of lib/include/detail/runge_kutta.hpp:155-163:
every double within 3000 ulps of both thresholds, for 20,000 end times, must
give the same loop and end-clamp decisions (tests/cpp/endtests_check.cpp,
compiled with g++ without contraction)."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_end_tests_match_fp64(tmp_path):
    exe = str(tmp_path / "endtests_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                    os.path.join(ROOT, "tests", "cpp", "endtests_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert " 0 mismatches" in out.stdout
