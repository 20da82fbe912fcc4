"""Generate the golden fixtures of the FP64 CIC / Boris / direct-deposition step.

The outputs come from pica's own headers, driven by oracle/ref_harness.cpp (3D)
and oracle/ref_harness_1d.cpp (pica's 1D classes), built into oracle/_ref/ from
the pica sources; this script therefore runs only where those sources are
mounted.  Inputs are seeded numpy draws and are
stored in the fixture, so the GPU tests need neither the sources nor the
generator.

Usage:  python tests/golden/make_golden.py            (every fixture)
        python tests/golden/make_golden.py config1    (the 32^3 x 50 ppc run only)
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


def case_config1(name="config1_pica_100steps", steps=100, sample_every=1009):
    """The plain FP64 electron plasma at its own size (tests.helpers.config1_plasma:
    32^3 cells, 50 ppc, CIC, Boris, direct deposition, supercell 2^3) run 100 steps
    through pica's headers.  The fixture keeps checksums, not the 1.6e6 particles: per
    step the number of moves, sum of count * (s + 1) and sum over moves of src * 7 +
    slot * 3 + dst; at the end the per-supercell counts, per field component the sum,
    sum of |.| and sum of squares, per particle component the sum and sum of squares,
    and every sample_every-th particle in ensemble order."""
    from tests.helpers import config1_plasma, run_checksums
    sim, p = config1_plasma()
    o = Oracle(sim["n"], sim["supercell"], sim["h"], sim["dt"], kind="reference")
    o.load(*[p[k] for k in ("x", "y", "z", "ux", "uy", "uz", "w", "species")])
    o.set_fields([np.zeros(sim["n"])] * 9)
    nm, cs, ms = run_checksums(lambda: o.step(1), o.counts, o.migrations, steps)
    q = o.particles()
    f = o.get_fields()
    comps = ("x", "y", "z", "ux", "uy", "uz")
    idx = np.arange(0, len(q["x"]), sample_every)
    out = os.path.join(HERE, name + ".npz")
    np.savez_compressed(
        out, steps=steps, n_moves=nm, count_sums=cs, move_sums=ms, counts=o.counts().astype(np.int32),
        field_sum=np.array([np.sum(a) for a in f]), field_abs=np.array([np.sum(np.abs(a)) for a in f]),
        field_sq=np.array([np.sum(a * a) for a in f]),
        part_sum=np.array([np.sum(q[k]) for k in comps]), part_sq=np.array([np.sum(q[k] * q[k]) for k in comps]),
        sample_index=idx, sample=np.stack([q[k][idx] for k in comps], axis=1), sample_supercell=q["supercell"][idx])
    print(out, len(q["x"]), "particles,", int(nm.sum()), "moves over", steps, "steps")


if __name__ == "__main__" and sys.argv[1:] == ["config1"]:
    case_config1()
elif __name__ == "__main__":
    # The plain FP64 32^3 electron plasma reduced to 8^3 x 4 ppc x 5 steps.
    case("cic_direct_8cube", (8, 8, 8), (2, 2, 2), 4, 5, seed=1)
    # Non-cubic grid and supercell, two species, non-zero initial E and B.
    case("cic_direct_2species", (8, 12, 16), (2, 2, 4), 3, 4, seed=2,
         species=((ME, E), (ME * 4.0, -E)), field_amp=2.0e3, u_sigma=0.08, resort_every=2)
    # pica's 1D classes: 32 cells x 4 ppc x 20 steps, non-zero initial E and B.
    case_1d("pica_1d_cic_direct", 32, 4, 20, seed=3)
    # The plain FP64 32^3 x 50 ppc plasma itself, 100 steps (checksums and a sample).
    case_config1()
