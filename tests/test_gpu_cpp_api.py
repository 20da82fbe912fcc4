"""The C++ header mirror (include/pica_gb300.hpp) drives the same device path
as the Python binding: a pica-style host loop compiled with g++ against the
library gives the same particles and fields.  FP64 form: the two runs differ
only by the order of the FP64 atomic current sums (tolerance 1e-13)."""
import os
import subprocess

import numpy as np
import pytest

import pica_gb300 as pg

pytestmark = pytest.mark.gpu

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def python_host_loop(steps):
    n0 = 1e18
    wp = np.sqrt(4 * pg.PI * n0 * pg.ELECTRON_CHARGE ** 2 / pg.ELECTRON_MASS)
    h = 0.05 * pg.LIGHT_VELOCITY / wp
    dt = 0.5 * h / (pg.LIGHT_VELOCITY * np.sqrt(3.0))
    s = pg.Simulation((8, 8, 8), (h, h, h), dt, supercell=(2, 2, 2))
    cols = [[] for _ in range(7)]
    for i in range(8):
        for j in range(8):
            for k in range(8):
                for p in range(2):
                    vals = ((i + 0.25 + 0.5 * p) * h, (j + 0.3) * h, (k + 0.6 - 0.2 * p) * h,
                            0.01 * ((i + p) % 3 - 1), 0.02 * ((j + k) % 2), -0.01, n0 * h * h * h / 2)
                    for c, v in zip(cols, vals):
                        c.append(v)
    s.upload_particles(*[np.array(c) for c in cols])
    f9 = [np.zeros((8, 8, 8)) for _ in range(9)]
    f9[2][3, 4, 5] = 100.0
    f9[4][1, 2, 3] = -50.0
    s.upload_fields(f9)
    for _ in range(steps):
        s.push_deposit()
        s.update_b(0.5 * dt)
        s.update_e(dt)
        s.update_b(0.5 * dt)
        s.migrate()
    return s.particles(), s.fields()


def test_cpp_host_loop_matches_python(tmp_path):
    so = pg._lib.lib_path()
    pg._lib.load()
    exe = str(tmp_path / "host_loop")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "host_loop.cpp"), so, "-o", exe,
                    "-Wl,-rpath," + os.path.dirname(so), "-lpthread"], check=True)
    out = subprocess.run([exe, "3"], capture_output=True, text=True, check=True).stdout.split("\n")
    n = int(out[0])
    rows = np.array([[float(v) for v in line.split()] for line in out[1:1 + n]])
    last = [float(v) for v in out[1 + n].split()]
    p, f = python_host_loop(3)
    for c, k in enumerate(("x", "y", "z", "ux", "uy", "uz")):
        assert np.max(np.abs(rows[:, c] - p[k])) <= 1e-13 * np.max(np.abs(p[k])), k
    np.testing.assert_allclose(last, [f[0][3, 4, 5], f[6][2, 2, 2], f[5][4, 4, 4]], rtol=1e-11, atol=0)


def test_cpp_driver_and_checkpoint(tmp_path):
    so = pg._lib.lib_path()
    pg._lib.load()
    exe = str(tmp_path / "driver_checkpoint")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "driver_checkpoint.cpp"), so, "-o", exe,
                    "-Wl,-rpath," + os.path.dirname(so), "-lpthread"], check=True)
    out = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True, check=True).stdout.split()
    assert out == ["diag", "2", "1", "diag", "4", "1", "diag", "6", "1", "same"]
    assert os.path.exists(tmp_path / "ckpt_3") and os.path.exists(tmp_path / "ckpt_6")


@pytest.mark.parametrize("nranges", [3, 4])
def test_cpp_host_resident_loop_equals_plain_steps(tmp_path, nranges):
    """tests/cpp/host_resident_loop.cpp: the state kept in pinned host memory, moved
    range by range on copy streams every step, equals plain steps bit for bit."""
    from pica_gb300.build import NVCC
    so = pg._lib.lib_path()
    pg._lib.load()
    cuda = os.path.dirname(os.path.dirname(NVCC))
    exe = str(tmp_path / "host_resident_loop")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(cuda, "include"),
                    os.path.join(ROOT, "tests", "cpp", "host_resident_loop.cpp"), so, "-L", os.path.join(cuda, "lib64"),
                    "-lcudart", "-o", exe, "-Wl,-rpath," + os.path.dirname(so), "-lpthread"], check=True)
    r = subprocess.run([exe, "5", str(nranges)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith(f"{nranges} ranges, same"), r.stdout
