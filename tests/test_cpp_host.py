"""The C++ host interface (include/hteno.hpp), shaped like the reference's solver classes: a
program in the style of the reference's main.cpp compiles against it (CPU) and, on the GPU,
reproduces the oracle run of the same case bit for bit."""
from __future__ import annotations

import subprocess
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parent.parent


def build_host(tmp: Path, hteno_lib) -> Path:
    exe = tmp / "host_fv2d"
    lib_dir = REPO / "hermite-teno_gb300" / "lib"
    cmd = ["g++", "-std=c++17", "-O2", "-I", str(REPO / "include"), str(REPO / "tests" / "cpp" / "host_fv2d.cpp"),
           "-L", str(lib_dir), "-lhteno", f"-Wl,-rpath,{lib_dir}", "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_cpp_host_compiles(hteno_lib, tmp_path):
    assert build_host(tmp_path, hteno_lib).exists()


@pytest.mark.gpu
def test_cpp_host_matches_oracle(hteno_lib, cuda, oracle, tmp_path):
    exe = build_host(tmp_path, hteno_lib)
    dat, binf, init = tmp_path / "result.dat", tmp_path / "state.bin", tmp_path / "init.bin"
    out = subprocess.run([str(exe), str(dat), str(binf), str(init)], check=True, capture_output=True, text=True)
    t = float(out.stdout.split("=")[1])
    got = np.fromfile(binf, dtype=np.float64).reshape(4, 48, 64)
    # the same case through the oracle: conservativeOfTaylorIns2D initial data (FV::System2D::
    # Riemann2D), TENO5 + HLLC, to t = 0.05
    g, nx, ny = 1.4, 64, 48
    x = (np.arange(nx) + 0.5) / nx
    y = (np.arange(ny) + 0.5) / ny
    X, Y = np.meshgrid(x, y)
    rho = np.where(Y < 0.5, 2.0, 1.0)
    p = np.where(Y < 0.5, 1.0 + 2.0 * Y, Y + 1.5)
    v = -0.025 * np.sqrt(g * p / rho) * np.cos(8.0 * (4.0 * np.arctan(1.0)) * X)
    q0 = np.ascontiguousarray(np.stack([rho, 0 * rho, rho * v, p / (g - 1) + 0.5 * (rho * v * v)]))
    q_init = np.fromfile(init, dtype=np.float64).reshape(4, 48, 64)
    np.testing.assert_allclose(q_init, q0, rtol=1e-14)  # Riemann2D built the reference's IC
    want, t_o, _ = oracle.fv2d_run(q_init, 100000, t_final=0.05, flux=1)
    assert t == t_o == 0.05
    np.testing.assert_array_equal(got, want)
    lines = dat.read_text().splitlines()
    assert lines[0].startswith("t: ") and lines[1].split() == ["x", "y", "Density", "Ux", "Uy", "Pressure"]
    assert len(lines) == 2 + nx * ny
    first = [float(s) for s in lines[2].split()]
    assert first[0] == pytest.approx(x[0]) and first[2] == pytest.approx(want[0, 0, 0], rel=1e-7)
