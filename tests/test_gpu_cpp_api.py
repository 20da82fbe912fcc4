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


PROTON_MASS = 1.672622964e-24


def python_drop_in(steps, fp32):
    """tests/cpp/pica_drop_in.cpp's loop through the Python binding, call for call:
    the same plasma (positions relative to the ensemble's minimum, as the mirror
    uploads them), the same momentum change after step 2 (then the whole ensemble
    uploaded again, as the mirror sends its host copy), and the same migrations."""
    n0 = 1e18
    wp = np.sqrt(4 * pg.PI * n0 * pg.ELECTRON_CHARGE ** 2 / pg.ELECTRON_MASS)
    h = 0.05 * pg.LIGHT_VELOCITY / wp
    dt = 0.5 * h / (pg.LIGHT_VELOCITY * np.sqrt(3.0))
    real = (lambda v: float(np.float32(v))) if fp32 else float
    mn = (-1.5 * h, 0.25 * h, 0.0)
    kw = dict(form=pg.FORM_FP32_CELL, shape=pg.SHAPE_TSC, deposit=pg.DEPOSIT_ESIRKEPOV, resort_every=2) if fp32 else \
        dict(form=pg.FORM_FP64_PLAIN, shape=pg.SHAPE_CIC, deposit=pg.DEPOSIT_DIRECT, resort_every=0)
    s = pg.Simulation((8, 8, 8), (h, h, h), real(dt), supercell=(2, 2, 2),
                      species=(pg.ELECTRON, (PROTON_MASS, -pg.ELECTRON_CHARGE)), **kw)
    cols = [[] for _ in range(8)]
    for i in range(8):
        for j in range(8):
            for k in range(8):
                for p in range(3):
                    x = mn[0] + ((i + 0.2) + 0.3 * p) * h
                    y = mn[1] + (j + 0.35) * h
                    z = mn[2] + ((k + 0.7) - 0.25 * p) * h
                    vals = (x - mn[0], y - mn[1], z - mn[2], 0.02 * ((i + p) % 3 - 1), 0.03 * ((j + k) % 2) - 0.01,
                            -0.015 + 0.01 * p, n0 * h * h * h / 3, 1 if p == 2 else 0)
                    for c, v in zip(cols, vals):
                        c.append(v)
    s.upload_particles(*[np.array(c) for c in cols[:7]], np.array(cols[7], np.int32))
    f9 = [np.zeros((8, 8, 8)) for _ in range(9)]
    f9[2][3, 4, 5] = 100.0
    f9[4][1, 2, 3] = -50.0
    s.upload_fields(f9)
    for st in range(steps):
        s.push_deposit()
        s.update_b(real(0.5 * dt))
        s.update_e(real(dt))
        s.update_b(real(0.5 * dt))
        s.migrate()
        if st == 1:
            q = s.particles()
            sc27 = np.nonzero(q["supercell"] == 27)[0]
            first = sc27[np.argmin(q["species"][sc27].astype(np.int64) * (1 << 40) + sc27)]   # species 0 first
            q["ux"][first] += 0.05
            q["uy"][first] += 0.0
            q["uz"][first] += -0.02
            s.upload_particles(*[(q[k] + m) - m for k, m in zip("xyz", mn)],
                               *[q[k] for k in ("ux", "uy", "uz", "w")], q["species"])
    q = s.particles()
    order = np.lexsort((np.arange(len(q["x"])), q["species"], q["supercell"]))
    rows = np.stack([q["supercell"][order], q["species"][order]] +
                    [q[k][order] + m for k, m in zip("xyz", mn)] + [q[k][order] for k in ("ux", "uy", "uz")], axis=1)
    f = s.fields()
    return rows, [f[0][3, 4, 5], f[6][2, 2, 2], f[5][4, 4, 4]]


@pytest.mark.parametrize("mode", ["fp64", "fp32"])
def test_pica_drop_in_loop_matches_python(tmp_path, mode):
    """tests/cpp/pica_drop_in.cpp -- a pica host loop whose only changes are the
    include, the namespace and one pushSupercells call -- compiled against the C++
    mirror, gives the particles (supercell by supercell) and fields of the same
    sequence through the Python binding: FP64 CIC/direct within 1e-13 (FP64 atomic
    current sums), FP32 TSC/Esirkepov bit for bit (fixed-point current sums)."""
    so = pg._lib.lib_path()
    pg._lib.load()
    exe = str(tmp_path / "pica_drop_in")
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-Wall", "-Wextra", "-Werror", "-I",
                    os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp", "pica_drop_in.cpp"), so, "-o",
                    exe, "-Wl,-rpath," + os.path.dirname(so), "-lpthread"], check=True)
    steps = 4
    out = subprocess.run([exe, str(steps), mode], capture_output=True, text=True, check=True).stdout.strip().split("\n")
    rows = np.array([[float(v) for v in line.split()] for line in out[:-1]])
    last = [float(v) for v in out[-1].split()[1:]]
    ref, fref = python_drop_in(steps, mode == "fp32")
    assert rows.shape == ref.shape
    assert np.array_equal(rows[:, :2], ref[:, :2])   # supercell and species of every particle, in order
    if mode == "fp32":
        assert np.array_equal(rows[:, 2:], ref[:, 2:])
        assert last == [float(np.float32(v)) for v in fref]
    else:
        for c in range(2, 8):
            assert np.max(np.abs(rows[:, c] - ref[:, c])) <= 1e-13 * np.max(np.abs(ref[:, c])), c
        np.testing.assert_allclose(last, fref, rtol=1e-11, atol=0)


def test_cpp_ensemble_ordered_reorders_on_the_device(tmp_path):
    """pica's EnsembleOrdered host code on the mirror: reorder() through the device
    sort gives the stable lexicographic order of the oracle, ties included."""
    from oracle import pic_oracle as po

    so = pg._lib.lib_path()
    pg._lib.load()
    exe = str(tmp_path / "ordered_ensemble")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "ordered_ensemble.cpp"), so, "-o", exe,
                    "-Wl,-rpath," + os.path.dirname(so), "-lpthread"], check=True)
    for n, seed in ((1, 1), (1000, 2), (9000, 3)):
        out = subprocess.run([exe, str(n), str(seed)], capture_output=True, text=True, check=True).stdout
        rows = np.array([[float(v) for v in line.split()] for line in out.strip().split("\n")])
        perm = rows[:, 0].astype(np.int64)
        xyz = np.empty((n, 3))
        xyz[perm] = rows[:, 1:]                  # positions in input order
        assert np.array_equal(perm, po.order_by_position(xyz[:, 0], xyz[:, 1], xyz[:, 2]))


def python_flat_loop(steps, ordered):
    n0 = 1e18
    wp = np.sqrt(4 * pg.PI * n0 * pg.ELECTRON_CHARGE ** 2 / pg.ELECTRON_MASS)
    h = 0.05 * pg.LIGHT_VELOCITY / wp
    dt = 0.5 * h / (pg.LIGHT_VELOCITY * np.sqrt(3.0))
    n = (8, 6, 10)
    species = (pg.ELECTRON, (PROTON_MASS, -pg.ELECTRON_CHARGE))
    s = pg.Simulation(n, (h, h, h), dt, supercell=(1, 1, 1), species=species)
    cols = [[] for _ in range(8)]
    for i in range(n[0]):
        for j in range(n[1]):
            for k in range(n[2]):
                for p in range(2):
                    ii = n[0] - 1 - i
                    vals = ((ii + 0.2 + 0.5 * p) * h, (j + 0.35) * h, (k + 0.7 - 0.4 * p) * h,
                            0.02 * ((ii + p) % 3 - 1), 0.03 * ((j + k) % 2) - 0.01, -0.015 + 0.01 * p,
                            n0 * h * h * h / 2, p)
                    for c, v in zip(cols, vals):
                        c.append(v)
    f9 = [np.zeros(n) for _ in range(9)]
    f9[2][3, 4, 5] = 100.0
    f9[4][1, 2, 3] = -50.0
    f9[0][7, 5, 9] = 30.0
    s.upload_fields(f9)
    e = pg.FlatEnsemble(s, guard=0)
    e.add(*[np.array(c) for c in cols[:7]], np.array(cols[7], np.int32))
    if ordered:
        e.reorder()
    e.step(steps)
    return e.particles(), s.fields()


@pytest.mark.parametrize("kind", ["unordered", "ordered"])
def test_cpp_flat_host_loop_matches_python(tmp_path, kind):
    """pica's host loop over EnsembleUnordered / EnsembleOrdered with the grid-level
    CIC operators, on the C++ mirror (pushParticles), against FlatEnsemble: the same
    particles in the same array order and the same fields (FP64; the atomic current
    sums may round differently, so 1e-13)."""
    so = pg._lib.lib_path()
    pg._lib.load()
    exe = str(tmp_path / "flat_host_loop")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "flat_host_loop.cpp"), so, "-o", exe,
                    "-Wl,-rpath," + os.path.dirname(so), "-lpthread"], check=True)
    out = subprocess.run([exe, "3", kind], capture_output=True, text=True, check=True).stdout.strip().split("\n")
    m = int(out[0])
    rows = np.array([[float(v) for v in line.split()] for line in out[1:1 + m]])
    last = [float(v) for v in out[1 + m].split()[1:]]
    p, f = python_flat_loop(3, kind == "ordered")
    assert np.array_equal(rows[:, 0].astype(np.int32), p["species"])
    for c, k in enumerate(("x", "y", "z", "ux", "uy", "uz", "w")):
        assert np.max(np.abs(rows[:, 1 + c] - p[k])) <= 1e-13 * np.max(np.abs(p[k])), k
    for got, want in zip(last, (f[0][3, 4, 5], f[6][2, 2, 2], f[5][4, 4, 4])):
        assert abs(got - want) <= 1e-13 * max(abs(want), 1e-300)
