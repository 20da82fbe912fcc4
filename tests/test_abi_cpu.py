"""CPU checks of the C ABI library: it builds, loads, exports every declared
symbol, and its host-only routines (plasma generation) behave.  No device work."""
import ctypes as C
import os
import re

import numpy as np

import pica_gb300
from oracle import pic_oracle as po
from pica_gb300 import _lib, workloads

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def declared_functions():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            text = open(os.path.join(ROOT, "include", fn)).read()
            names |= set(re.findall(r"\b(pica_[a-z0-9_]+)\s*\(", text))
    return names


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    declared = declared_functions()
    assert len(declared) >= 25
    for name in declared:
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, name
    assert lib.pica_abi_version() == 1
    assert lib.pica_status_string(-5).decode().startswith("particle crossed")
    assert "bounded device wait" in lib.pica_status_string(-9).decode()   # PICA_ERR_TIMEOUT


def test_config_struct_layout_matches_header():
    # pica_config: 3 int32 + 3 int32 + 3 double + double + 4 int32 + 4 double + 4 double + double + 2 int32
    assert C.sizeof(_lib.PicaConfig) == 4 * 6 + 8 * 4 + 4 * 4 + 8 * 8 + 8 + 4 * 2
    assert C.sizeof(_lib.PicaDiag) == 8 * 8


def test_plasma_generation_is_thread_count_independent():
    spec = pica_gb300.plasma_spec((6, 5, 4), (1e-3, 1e-3, 1e-3), 9, 0.05, 2.0, seed=7)
    a = pica_gb300.generate_plasma(spec, threads=1)
    b = pica_gb300.generate_plasma(spec, threads=5)
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    assert len(a["x"]) == 6 * 5 * 4 * 9
    # positions in their cell, cell-major order
    cell = (np.floor(a["x"] / 1e-3).astype(int) * 5 + np.floor(a["y"] / 1e-3).astype(int)) * 4 + np.floor(a["z"] / 1e-3).astype(int)
    assert np.all(np.diff(cell) >= 0)
    assert abs(np.std(np.concatenate([a["ux"], a["uy"], a["uz"]])) - 0.05) < 0.01


def test_density_modulation_and_beams():
    spec = pica_gb300.plasma_spec((16, 2, 2), (1.0, 1.0, 1.0), 100, 0.01, 1.0, seed=3, density_mod=0.9, nbeams=2,
                                  drift_u=0.2, drift_axis=0)
    p = pica_gb300.generate_plasma(spec)
    per_plane = np.bincount(np.floor(p["x"]).astype(int), minlength=16) // 4
    expected = np.round(100 * (1 + 0.9 * np.cos(2 * np.pi * (np.arange(16) + 0.5) / 16))).astype(int)
    assert np.array_equal(per_plane, expected)
    assert per_plane.min() >= 10 and per_plane.max() <= 190
    assert abs(np.mean(np.abs(p["ux"])) - 0.2) < 0.01


def test_workload_sizes():
    c2 = workloads.config2()
    n = c2["sim"]["n"]
    assert n == (128, 128, 128) and c2["specs"][0].ppc == 100
    assert int(np.prod(n)) * 100 == 209715200
    members = workloads.batched_members()
    assert len(members) == 64
    edges = [m["sim"]["n"][0] for m in members]
    assert min(edges) >= 32 and max(edges) <= 96 and all(e % 4 == 0 for e in edges)


def test_supercell_ranges_cover_every_supercell_once():
    for total, n, k in ((32768, 16, 1), (32768, 16, 8), (1000, 7, 3), (5, 8, 1), (5, 1, 4)):
        r = pica_gb300.supercell_ranges(total, n, k)
        assert r[0][0] == 0 and r[-1][1] == total
        assert all(a[1] == b[0] and a[0] <= a[1] for a, b in zip(r, r[1:]))
        assert len(r) == (n + (2 * (k - 1) if n > 1 else k - 1) if k > 1 else n)
    # uniform ranges are those of pica_push_deposit_chunked: [total r / n, total (r+1) / n)
    assert pica_gb300.supercell_ranges(10, 3) == [(0, 3), (3, 6), (6, 10)]


def test_cpp_mirror_compiles_and_links_against_the_library(tmp_path):
    """The C++ header mirror and the host loops of the GPU tests compile and link
    against the library (running them needs a GPU)."""
    import subprocess
    from pica_gb300.build import NVCC
    so = _lib.lib_path()
    _lib.load()
    cuda = os.path.dirname(os.path.dirname(NVCC))
    runtime = ["-I", os.path.join(cuda, "include"), "-L", os.path.join(cuda, "lib64"), "-lcudart"]
    for src in ("host_loop.cpp", "driver_checkpoint.cpp", "host_resident_loop.cpp"):
        exe = str(tmp_path / src.replace(".cpp", ""))
        extra = runtime if src == "host_resident_loop.cpp" else []
        subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Wpedantic", "-Werror", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", src), so] + extra + ["-o", exe,
                        "-Wl,-rpath," + os.path.dirname(so), "-lpthread"], check=True)
        assert os.path.exists(exe)


def test_particle_and_constants_known_answers_of_the_cpp_mirror(tmp_path):
    """pica's Particle, Constants and YeeGrid known answers (ParticleTests.cpp:37-164,
    ConstantsTests.cpp:15-28, YeeGridTests.cpp:115-134) against the C++ mirror, host only
    (linked against the library, which a grid without a Simulation never calls)."""
    import subprocess
    so = _lib.lib_path()
    _lib.load()
    exe = str(tmp_path / "particle_known_answers")
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Wpedantic", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "particle_known_answers.cpp"), so, "-o", exe,
                    "-Wl,-rpath," + os.path.dirname(so)], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout


CONSTANT_NAMES = ("pi", "c", "lightVelocity", "electronCharge", "electronMass", "protonMass", "planck", "eV", "meV")


def _print_constants(tmp_path, name, include, namespace):
    import subprocess
    src = tmp_path / f"{name}.cpp"
    body = "".join(f'    std::printf("%.17g\\n", {namespace}::constants::{c});\n' for c in CONSTANT_NAMES)
    src.write_text(f'#include <cstdio>\n#include "{include}"\nint main() {{\n{body}    return 0;\n}}\n')
    exe = str(tmp_path / name)
    inc = po.pica_include_dir() if namespace == "pica" else os.path.join(ROOT, "include")
    subprocess.run(["g++", "-std=c++17", "-I", inc, str(src), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    return [float(v) for v in out]


def test_constants_equal_picas(tmp_path):
    """The mirror's constants table (and the Python module's) equals pica's
    math/Constants.h value for value; compiled against pica's own header when it is
    present in this checkout."""
    import pytest
    ours = _print_constants(tmp_path, "ours", "pica_gb300.hpp", "pica_gb300")
    py = dict(pi=pica_gb300.PI, c=pica_gb300.LIGHT_VELOCITY, electronCharge=pica_gb300.ELECTRON_CHARGE,
              electronMass=pica_gb300.ELECTRON_MASS)
    for name, v in py.items():
        assert ours[CONSTANT_NAMES.index(name)] == v, name
    if po.pica_include_dir() is None:
        pytest.skip("pica's headers are not in this checkout")
    theirs = _print_constants(tmp_path, "theirs", "pica/math/Constants.h", "pica")
    assert ours == theirs


def test_cpp_mirror_plumbing_against_a_host_fake_of_the_abi(tmp_path):
    """The C++ mirror's host code (field order and round trip, particle conversion,
    per-supercell selection) against tests/cpp/fake_abi.cpp, a host stand-in for the
    entry points it calls that returns the ABI's documented ensemble order."""
    import subprocess
    exe = str(tmp_path / "mirror_plumbing")
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Wpedantic", "-Werror",
                    "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp", "mirror_plumbing.cpp"),
                    os.path.join(ROOT, "tests", "cpp", "fake_abi.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout


def _config(**kw):
    c = _lib.PicaConfig()
    for d in range(3):
        c.n[d], c.sc[d], c.h[d] = 8, 2, 1e-3
    c.dt, c.form, c.shape, c.deposit, c.nspecies = 1e-14, 0, 1, 0, 1
    c.mass[0], c.charge[0] = pica_gb300.ELECTRON_MASS, pica_gb300.ELECTRON_CHARGE
    for k, v in kw.items():
        if isinstance(v, tuple):
            getattr(c, k)[v[0]] = v[1]
        else:
            setattr(c, k, v)
    return c


def test_context_creation_rejects_bad_configurations_before_touching_the_device():
    """Statuses, not exceptions, cross the ABI: every malformed configuration is
    PICA_ERR_INVALID (a grid beyond the FP32 form's packed cell index, PICA_ERR_LIMIT)
    and leaves the output handle NULL; validation runs before any CUDA call, so this
    holds on a machine without a GPU."""
    lib = _lib.load()
    bad = [dict(form=7), dict(shape=0), dict(deposit=3), dict(nspecies=0), dict(nspecies=9), dict(dt=0.0),
           dict(dt=float("nan")), dict(n=(0, 9)), dict(n=(1, 0)), dict(sc=(1, 3)), dict(sc=(2, 0)), dict(h=(2, -1.0)),
           dict(h=(0, float("nan")))]
    for kw in bad:
        out = C.c_void_p(123)
        assert lib.pica_ctx_create(C.byref(_config(**kw)), C.byref(out)) == -1, kw
        assert out.value is None, kw
    out = C.c_void_p(123)
    assert lib.pica_ctx_create(C.byref(_config(form=1, n=(0, 4096))), C.byref(out)) == -8
    assert out.value is None
    assert lib.pica_ctx_create(None, C.byref(out)) == -1


def test_context_creation_without_a_device_is_a_cuda_error():
    """With no CUDA device there is no CPU path: a valid configuration returns
    PICA_ERR_CUDA, and the Python binding raises."""
    import pytest
    lib = _lib.load()
    out = C.c_void_p(123)
    rc = lib.pica_ctx_create(C.byref(_config()), C.byref(out))
    if rc == 0:   # a GPU is present: nothing to check here
        lib.pica_ctx_destroy(out)
        pytest.skip("a CUDA device is present")
    assert rc == -2 and out.value is None
    with pytest.raises(pica_gb300.PicaError):
        pica_gb300.Simulation((8, 8, 8), (1e-3,) * 3, 1e-14, supercell=(2, 2, 2))


def test_flat_entry_points_reject_bad_arguments_before_touching_the_device():
    """pica_order_by_position / _host and pica_push_flat check their arguments first:
    bad dimensions, negative sizes and missing arrays are PICA_ERR_INVALID, and an
    empty array is a no-op, all without a device."""
    lib = _lib.load()
    x = np.zeros(4)
    order = np.zeros(4, np.int64)
    dp = x.ctypes.data_as(C.POINTER(C.c_double))
    op = order.ctypes.data_as(C.POINTER(C.c_int64))
    assert lib.pica_order_by_position(4, 0, x.ctypes.data, None, None, order.ctypes.data, None) == -1
    assert lib.pica_order_by_position(4, 4, x.ctypes.data, x.ctypes.data, x.ctypes.data, order.ctypes.data, None) == -1
    assert lib.pica_order_by_position(-1, 1, x.ctypes.data, None, None, order.ctypes.data, None) == -1
    assert lib.pica_order_by_position(4, 2, x.ctypes.data, None, None, order.ctypes.data, None) == -1
    assert lib.pica_order_by_position(0, 3, None, None, None, None, None) == 0
    assert lib.pica_order_by_position_host(4, 3, dp, dp, None, op) == -1
    assert lib.pica_order_by_position_host(0, 3, None, None, None, None) == 0
    assert lib.pica_push_flat(None, 4, *([x.ctypes.data] * 7), None, 2) == -1
