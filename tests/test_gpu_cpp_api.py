"""The reference's golden test, rewritten against this library's C++ host
API (include/bri17/bri17_gpu.hpp) and run on the GPU: tests/cpp/
test_bri17_gpu.cpp extracts K and B from the operator by unit vectors and
compares them with the assembled Maxima element matrices at the reference's
tolerances (tests/test_bri17.cpp:318-606)."""
import os
import shutil
import subprocess

import pytest

from conftest import REPO

pytestmark = pytest.mark.gpu


def test_cpp_api_golden_sections(golden_elements, tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = tmp_path / "test_bri17_gpu"
    lib_dir = os.path.join(REPO, "bri17_gb300")
    subprocess.run([nvcc, "-std=c++17", "-O2", "-I", os.path.join(REPO, "include"),
                    os.path.join(REPO, "tests", "cpp", "test_bri17_gpu.cpp"), "-o", str(exe),
                    "-L", lib_dir, "-lbri17_gb300", f"-Xlinker=-rpath={lib_dir}"],
                   check=True, capture_output=True)
    g = golden_elements
    lines = []
    for c in g["cases"]:
        vals = " ".join(repr(v) for v in c["values"])
        lines.append(f"{c['kind']} {c['dim']} {' '.join(map(str, c['shape']))} "
                     f"{' '.join(repr(x) for x in c['L'])} {g['mu']!r} {g['nu']!r} "
                     f"{g['rtol']!r} {g['atol']!r} {c['rows']} {c['cols']} {vals}")
    golden = tmp_path / "golden.txt"
    golden.write_text("\n".join(lines) + "\n")
    r = subprocess.run([str(exe), str(golden)], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "6 of 6 sections passed" in r.stdout
