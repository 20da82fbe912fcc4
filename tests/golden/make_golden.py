"""Generate the golden fixtures of the FP64 CIC / Boris / direct-deposition step.

The outputs come from pica's own headers, driven by oracle/ref_harness.cpp (3D)
and oracle/ref_harness_1d.cpp (pica's 1D classes), built into oracle/_ref/ from
the pica sources; this script therefore runs only where those sources are
mounted.  Inputs are seeded numpy draws and are
stored in the fixture, so the GPU tests need neither the sources nor the
generator.

Usage:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..", "..")))

from oracle.pic_oracle import Oracle  # noqa: E402

C = 29979245800.0
E = -4.80320427e-10
ME = 9.10938215e-28
PI = 3.14159265358


def case(name, n, sc, ppc, steps, seed, species=((ME, E),), field_amp=0.0, u_sigma=0.05, resort_every=0):
    rng = np.random.default_rng(seed)
    n0 = 1e18
    wp = np.sqrt(4 * PI * n0 * E * E / ME)
    h = 0.05 * C / wp
    hh = (h * 1.0, h * 1.1, h * 0.9)  # non-cubic cells exercise per-dimension coefficients
    dt = 0.5 / (C * np.sqrt(sum(1.0 / v ** 2 for v in hh)))
    idx = np.indices(n).reshape(3, -1).T
    cells = np.repeat(idx, ppc, axis=0)
    pos = (cells + rng.random(cells.shape)) * np.array(hh)
    u = rng.normal(0.0, u_sigma, cells.shape)
    w = np.full(len(pos), n0 * np.prod(hh) / ppc) * (1.0 + 0.1 * rng.random(len(pos)))
    sp = rng.integers(0, len(species), len(pos)).astype(np.int32)
    f9 = [field_amp * rng.standard_normal(n) for _ in range(6)] + [np.zeros(n)] * 3
    o = Oracle(n, sc, hh, dt, species=species, kind="reference", resort_every=resort_every)
    o.load(pos[:, 0], pos[:, 1], pos[:, 2], u[:, 0], u[:, 1], u[:, 2], w, sp)
    o.set_fields(f9)
    counts, migs = [], []
    for s in range(steps):
        o.step(1)
        counts.append(o.counts())
        m = o.migrations()
        migs.append(np.concatenate([np.full((len(m), 1), s, np.int32), m], axis=1))
    p = o.particles()
    f = o.get_fields()
    out = os.path.join(HERE, name + ".npz")
    np.savez_compressed(
        out, n=np.array(n), sc=np.array(sc), h=np.array(hh), dt=dt, steps=steps, resort_every=resort_every,
        mass=np.array([m for m, _ in species]), charge=np.array([q for _, q in species]),
        in_x=pos[:, 0], in_y=pos[:, 1], in_z=pos[:, 2], in_ux=u[:, 0], in_uy=u[:, 1], in_uz=u[:, 2], in_w=w,
        in_species=sp, in_fields=np.stack(f9),
        out_x=p["x"], out_y=p["y"], out_z=p["z"], out_ux=p["ux"], out_uy=p["uy"], out_uz=p["uz"], out_w=p["w"],
        out_species=p["species"], out_supercell=p["supercell"], out_fields=np.stack(f),
        counts=np.stack(counts), migrations=np.concatenate(migs) if migs else np.zeros((0, 5), np.int32))
    print(out, len(pos), "particles,", sum(len(m) for m in migs), "migrations")


def case_1d(name, n, ppc, steps, seed, field_amp=1.0e3, u_sigma=0.1):
    """pica's YeeGrid<One> path (ref_harness_1d.cpp) on n cells: the reference of a grid one
    cell thick along y and z.  Particles keep their input order."""
    import ctypes as CT
    lib = CT.CDLL(os.path.abspath(os.path.join(HERE, "..", "..", "oracle", "_ref", "libpica_ref1d.so")))
    dp = CT.POINTER(CT.c_double)
    lib.ref1d_run.argtypes = [CT.c_int32, CT.c_double, CT.c_double, CT.c_double, CT.c_int32, dp, dp, CT.c_int64, dp,
                              dp, dp, dp, dp, CT.POINTER(CT.c_int32), dp, CT.c_int32]
    rng = np.random.default_rng(seed)
    n0 = 1e18
    h = 0.05 * C / np.sqrt(4 * PI * n0 * E * E / ME)
    dt = 0.5 * h / (C * np.sqrt(3.0))
    npart = n * ppc
    x = (np.repeat(np.arange(n), ppc) + rng.random(npart)) * h
    u = rng.normal(0.0, u_sigma, (3, npart))
    w = np.full(npart, n0 * h ** 3 / ppc) * (1.0 + 0.1 * rng.random(npart))
    sp = np.zeros(npart, np.int32)
    f = np.stack([field_amp * rng.standard_normal(n) for _ in range(6)] + [np.zeros(n)] * 3)
    mass, charge = np.array([ME]), np.array([E])
    xo, uxo, uyo, uzo, fo = x.copy(), u[0].copy(), u[1].copy(), u[2].copy(), f.copy()

    def ptr(a):
        return a.ctypes.data_as(dp)

    rc = lib.ref1d_run(n, h, h * h, dt, 1, ptr(mass), ptr(charge), npart, ptr(xo), ptr(uxo), ptr(uyo), ptr(uzo),
                       ptr(w), sp.ctypes.data_as(CT.POINTER(CT.c_int32)), ptr(fo), steps)
    assert rc == 0
    out = os.path.join(HERE, name + ".npz")
    np.savez_compressed(out, n=n, h=h, dt=dt, steps=steps, mass=mass, charge=charge, in_x=x, in_ux=u[0], in_uy=u[1],
                        in_uz=u[2], in_w=w, in_fields=f, out_x=xo, out_ux=uxo, out_uy=uyo, out_uz=uzo, out_fields=fo)
    print(out, npart, "particles")


if __name__ == "__main__":
    # The plain FP64 32^3 electron plasma reduced to 8^3 x 4 ppc x 5 steps.
    case("cic_direct_8cube", (8, 8, 8), (2, 2, 2), 4, 5, seed=1)
    # Non-cubic grid and supercell, two species, non-zero initial E and B.
    case("cic_direct_2species", (8, 12, 16), (2, 2, 4), 3, 4, seed=2,
         species=((ME, E), (ME * 4.0, -E)), field_amp=2.0e3, u_sigma=0.08, resort_every=2)
    # pica's 1D classes: 32 cells x 4 ppc x 20 steps, non-zero initial E and B.
    case_1d("pica_1d_cic_direct", 32, 4, 20, seed=3)
