"""The reference-shaped C++ shim (include/ss_gpu_voxel_grid.hpp) drives the
library from a C++ program: integrate, raycast, kokkosICP."""
import subprocess
from pathlib import Path

import pytest

BIN = Path(__file__).resolve().parent.parent / "superscanner_gb300" / "_build" / "shim_roundtrip"


def test_shim_program_builds():
    assert BIN.exists(), "build() compiles tests/cpp/shim_roundtrip.cpp against the shim header"


@pytest.mark.gpu
def test_shim_program_runs():
    out = subprocess.run([str(BIN)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    f = out.stdout.split()
    vals = dict(zip(f[0::2], f[1::2]))
    assert int(vals["blocks"]) > 0
    assert int(vals["hits"]) > 0.9 * 120 * 160
    assert abs(float(vals["mean_z"]) - 1.5) < 0.01
    assert float(vals["icp_offdiag"]) < 1e-5
