"""The neighbour slot code (lattice translation modulo 1024 per axis + minimum-image bit) and the
recovery of the full translation from the two atoms' integer floors (code_t_full), compiled for
the host from the same header the kernels use and checked exhaustively (tests/cpp/code_check.cpp)."""
import os
import subprocess

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA_INC = "/usr/local/cuda/include"


def test_translation_codes_round_trip(tmp_path):
    exe = str(tmp_path / "code_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I" + CUDA_INC, "-I" + os.path.join(REPO, "atomnn_gb300", "csrc"),
                    os.path.join(REPO, "tests", "cpp", "code_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("ok ")
