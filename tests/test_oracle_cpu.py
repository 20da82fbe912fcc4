"""CPU tests of the oracle: pinned to pica's own headers and to the golden
fixtures, plus known answers for the parts pica does not have (TSC,
Esirkepov charge conservation, Boris gyration, E x B drift)."""
import os

import numpy as np
import pytest

from oracle import pic_oracle as po
from tests.helpers import C, E, ME, load_golden, rel_err, run_1d_golden, species_of, thermal_inputs

REFERENCE_AVAILABLE = po.reference_available()


def run_fixture(kind, g):
    o = po.Oracle(tuple(g["n"]), tuple(g["sc"]), tuple(g["h"]), float(g["dt"]), species=species_of(g), kind=kind,
                  resort_every=int(g["resort_every"]))
    o.load(g["in_x"], g["in_y"], g["in_z"], g["in_ux"], g["in_uy"], g["in_uz"], g["in_w"], g["in_species"])
    o.set_fields(list(g["in_fields"]))
    counts, migs = [], []
    for s in range(int(g["steps"])):
        o.step(1)
        counts.append(o.counts())
        m = o.migrations()
        migs.append(np.concatenate([np.full((len(m), 1), s, np.int32), m], axis=1))
    return o, np.stack(counts), np.concatenate(migs)


@pytest.mark.parametrize("name", ["cic_direct_8cube", "cic_direct_2species"])
def test_port_reproduces_golden_bit_exactly(name):
    g = load_golden(name)
    o, counts, migs = run_fixture("port", g)
    p = o.particles()
    for k in ("x", "y", "z", "ux", "uy", "uz", "w"):
        assert np.array_equal(p[k], g["out_" + k]), k
    assert np.array_equal(p["supercell"], g["out_supercell"])
    assert np.array_equal(p["species"], g["out_species"])
    f = o.get_fields()
    for c in range(9):
        assert np.array_equal(f[c], g["out_fields"][c]), c
    assert np.array_equal(counts, g["counts"])
    assert np.array_equal(migs, g["migrations"])


@pytest.mark.skipif(not REFERENCE_AVAILABLE, reason="pica sources not mounted here")
@pytest.mark.parametrize("n,sc,ppc,steps,resort", [((8, 8, 8), (2, 2, 2), 6, 3, 0),
                                                   ((64, 4, 4), (2, 2, 2), 2, 3, 2),  # origin m=62: trunc(m h / h) = 61
                                                   ((12, 8, 6), (3, 4, 2), 4, 5, 2)])
def test_port_matches_reference_headers(n, sc, ppc, steps, resort):
    po.build(reference=True)
    d = thermal_inputs(n, ppc, seed=11, u_sigma=0.1)
    res = []
    for kind in ("port", "reference"):
        o = po.Oracle(n, sc, d["h"], d["dt"], kind=kind, resort_every=resort)
        o.load(d["x"], d["y"], d["z"], d["ux"], d["uy"], d["uz"], d["w"])
        rng = np.random.default_rng(3)
        o.set_fields([1e3 * rng.standard_normal(n) for _ in range(6)] + [np.zeros(n)] * 3)
        o.step(steps)
        res.append((o.particles(), o.get_fields(), o.counts(), o.migrations()))
    (pa, fa, ca, ma), (pb, fb, cb, mb) = res
    for k in ("x", "y", "z", "ux", "uy", "uz", "w"):
        assert np.array_equal(pa[k], pb[k]), k
    for c in range(9):
        assert np.array_equal(fa[c], fb[c]), c
    assert np.array_equal(ca, cb) and np.array_equal(ma, mb)


@pytest.mark.skipif(not REFERENCE_AVAILABLE, reason="pica sources not mounted here")
@pytest.mark.parametrize("n,sc,ppc,steps,resort,u_sigma,hscale,nspecies,drift", [
    ((16, 12, 8), (4, 4, 4), 4, 4, 2, 0.1, (1.0, 1.0, 1.0), 2, None),            # electrons and ions, 4^3 supercells
    ((8, 8, 8), (2, 2, 2), 3, 6, 3, 0.3, (1.0, 0.7, 1.3), 1, (0.2, 0.0, -0.1)),  # hot drifting plasma, uneven cells
])
def test_port_matches_reference_headers_species_and_fast_particles(n, sc, ppc, steps, resort, u_sigma, hscale,
                                                                    nspecies, drift):
    """The restatement against the harness over pica's headers with two species (ions
    of 100 electron masses, species interleaved in the input) and with a hot drifting
    plasma on uneven cells, where many particles migrate every step: equal bit for bit,
    particles, fields, counts and migration lists."""
    po.build(reference=True)
    d = thermal_inputs(n, ppc, seed=23, u_sigma=u_sigma, hscale=hscale, nspecies=nspecies, drift=drift)
    species = ((ME, E), (100 * ME, -E))[:nspecies]   # electrons (E < 0), ions
    res = []
    for kind in ("port", "reference"):
        o = po.Oracle(n, sc, d["h"], d["dt"], kind=kind, resort_every=resort, species=species)
        o.load(d["x"], d["y"], d["z"], d["ux"], d["uy"], d["uz"], d["w"], d["species"])
        rng = np.random.default_rng(4)
        o.set_fields([2e3 * rng.standard_normal(n) for _ in range(6)] + [np.zeros(n)] * 3)
        migrated = 0
        for _ in range(steps):
            o.step(1)
            migrated += len(o.migrations())
        res.append((o.particles(), o.get_fields(), o.counts(), o.migrations(), migrated))
    (pa, fa, ca, ma, na), (pb, fb, cb, mb, nb) = res
    for k in ("x", "y", "z", "ux", "uy", "uz", "w", "species", "supercell"):
        assert np.array_equal(pa[k], pb[k]), k
    for c in range(9):
        assert np.array_equal(fa[c], fb[c]), c
    assert np.array_equal(ca, cb) and np.array_equal(ma, mb) and na == nb
    assert na > 0.02 * len(d["x"]) * steps if u_sigma >= 0.3 else na > 0


def div_faces(jx, jy, jz, h):
    return ((np.roll(jx, -1, 0) - jx) / h[0] + (np.roll(jy, -1, 1) - jy) / h[1] + (np.roll(jz, -1, 2) - jz) / h[2])


@pytest.mark.parametrize("form,tol", [(po.FORM_FP64_PLAIN, 1e-12), (po.FORM_FP32_CELL, 2e-6)])
@pytest.mark.parametrize("shape", [po.SHAPE_CIC, po.SHAPE_TSC])
def test_esirkepov_continuity(form, tol, shape):
    """(rho^{n+1} - rho^n)/dt + div J^{n+1/2} = 0 on the cell-centred lattice."""
    n = (8, 8, 8)
    d = thermal_inputs(n, 6, seed=5, u_sigma=0.2)
    o = po.Oracle(n, (4, 4, 4), d["h"], d["dt"], form=form, shape=shape, deposit=po.DEPOSIT_ESIRKEPOV)
    o.load(d["x"], d["y"], d["z"], d["ux"], d["uy"], d["uz"], d["w"])
    rng = np.random.default_rng(9)
    o.set_fields([5e3 * rng.standard_normal(n) for _ in range(6)] + [np.zeros(n)] * 3)
    for _ in range(3):
        r0 = o.charge_density()
        o.step(1)
        r1 = o.charge_density()
        f = o.get_fields()
        res = (r1 - r0) / d["dt"] + div_faces(f[6], f[7], f[8], d["h"])
        scale = np.max(np.abs(r0)) / d["dt"]
        assert np.max(np.abs(res)) / scale < tol


def single_particle(u0, e, b, steps, form=po.FORM_FP64_PLAIN, n=(8, 8, 8)):
    """One particle of negligible weight in uniform fields (self-fields ~1e-30 of the applied ones)."""
    h0 = 1e-3
    dt = 0.5 * h0 / (C * np.sqrt(3))
    o = po.Oracle(n, (4, 4, 4), (h0, h0, h0), dt, form=form, deposit=po.DEPOSIT_ESIRKEPOV, shape=po.SHAPE_TSC)
    x0 = 4.3 * h0
    o.load([x0], [x0], [x0], [u0[0]], [u0[1]], [u0[2]], [1e-30])
    o.set_fields([np.full(n, e[0]), np.full(n, e[1]), np.full(n, e[2]), np.full(n, b[0]), np.full(n, b[1]),
                  np.full(n, b[2])] + [np.zeros(n)] * 3)
    traj = []
    for _ in range(steps):
        o.step(1)
        p = o.particles()
        traj.append([p[k][0] for k in ("x", "y", "z", "ux", "uy", "uz")])
    return np.array(traj), dt, h0


def test_boris_gyration_known_answer():
    """Uniform B: |u| is conserved and the phase advances by 2 atan(|t|) per step (BorisPusher.h:33-43)."""
    b = 3.0e4
    u0 = np.array([0.1, 0.0, 0.0])
    traj, dt, _ = single_particle(u0, (0, 0, 0), (0, 0, b), 40)
    u = traj[:, 3:]
    assert np.max(np.abs(np.linalg.norm(u, axis=1) - 0.1)) < 1e-14
    gamma = np.sqrt(1 + 0.01)
    t = (E * dt / (2 * ME * C)) * b / gamma
    phase = np.unwrap(np.arctan2(u[:, 1], u[:, 0]))
    expected = -2 * np.arctan(t) * np.arange(1, 41)   # rotation sense of the Boris map for t along z
    assert np.max(np.abs(phase - expected)) < 1e-12


def test_exb_drift():
    """E x B drift c E x B / B^2 of a non-relativistic electron, averaged over whole gyro-periods."""
    b = 1.0e5
    e_y = 1.0e2   # v_d = c E/B = 3e7 cm/s << c
    traj, dt, _ = single_particle(np.zeros(3), (0, e_y, 0), (0, 0, b), 2000, n=(64, 64, 8))
    omega = abs(E) * b / (ME * C)
    period = int(round(2 * np.pi / omega / dt))
    k = (len(traj) // period) * period
    vx = np.diff(np.unwrap(traj[:k + 1, 0], period=64 * 1e-3)) / dt
    vd = C * e_y / b
    assert abs(np.mean(vx[:k]) - vd) / vd < 2e-3


@pytest.mark.parametrize("shape", [po.SHAPE_CIC, po.SHAPE_TSC])
def test_fp32_form_tracks_fp64(shape):
    """The FP32 cell form follows the FP64 form within single-precision error over a few steps."""
    n = (8, 8, 8)
    d = thermal_inputs(n, 4, seed=8)
    out = []
    for form in (po.FORM_FP64_PLAIN, po.FORM_FP32_CELL):
        o = po.Oracle(n, (4, 4, 4), d["h"], d["dt"], form=form, shape=shape, deposit=po.DEPOSIT_ESIRKEPOV)
        o.load(d["x"], d["y"], d["z"], d["ux"], d["uy"], d["uz"], d["w"])
        o.set_fields([np.zeros(n)] * 9)
        o.step(5)
        out.append((o.particles(), o.get_fields(), o.counts()))
    (p64, f64, c64), (p32, f32, c32) = out
    assert np.array_equal(c64, c32)
    assert rel_err(p32["ux"], p64["ux"]) < 1e-4
    for c in range(9):
        assert rel_err(f32[c], f64[c]) < 1e-3


def test_diagnostics_conservation():
    """Total charge is exact; field + kinetic energy of a thermal plasma drifts little over 20 steps."""
    n = (8, 8, 8)
    d = thermal_inputs(n, 8, seed=4)
    o = po.Oracle(n, (4, 4, 4), d["h"], d["dt"], shape=po.SHAPE_TSC, deposit=po.DEPOSIT_ESIRKEPOV)
    o.load(d["x"], d["y"], d["z"], d["ux"], d["uy"], d["uz"], d["w"])
    o.set_fields([np.zeros(n)] * 9)
    bg = -E * 1e18
    d0 = o.diagnostics(bg)
    o.step(20)
    d1 = o.diagnostics(bg)
    assert d1["total_charge"] == pytest.approx(d0["total_charge"], rel=1e-14)
    e0 = d0["field_energy"] + d0["kinetic_energy"]
    e1 = d1["field_energy"] + d1["kinetic_energy"]
    assert abs(e1 - e0) / e0 < 2e-2
    # Esirkepov keeps div E - 4 pi rho at its initial value.
    assert abs(d1["gauss_max"] - d0["gauss_max"]) / d0["gauss_max"] < 0.5


def test_oracle_one_cell_thick_grid_matches_pica_1d_classes():
    """A grid one cell thick along y and z against pica's own 1D path (YeeGrid<One>,
    FieldInterpolatorCIC / CurrentDepositorCIC<YeeGrid<One>>, the 1D YeeSolver; golden
    fixture from oracle/ref_harness_1d.cpp): fields and particles within 1e-12."""
    g = load_golden("pica_1d_cic_direct")

    def make(n3, sc, h3, dt):
        o = po.Oracle(n3, sc, h3, dt, form=po.FORM_FP64_PLAIN, shape=po.SHAPE_CIC, deposit=po.DEPOSIT_DIRECT)
        return o.load, o.set_fields, o.step, o.get_fields, o.particles

    f, got, ref = run_1d_golden(make, g)
    for c in range(9):
        assert rel_err(f[c], g["out_fields"][c]) <= 1e-12, c
    for k in ("x", "ux", "uy", "uz"):
        assert rel_err(got[k], ref[k]) <= 1e-12, k


@pytest.mark.parametrize("form,tol", [(po.FORM_FP64_PLAIN, 1e-11), (po.FORM_FP32_CELL, 2e-5)])
def test_yee_vacuum_plane_wave_follows_the_discrete_dispersion(form, tol):
    """A standing Ey mode cos(k x) in vacuum (pica's staggering: Ey at x = (i + 1/2) h,
    YeeGrid.h:11-14), advanced by B(dt/2), E(dt), B(dt/2) per step, keeps its shape and
    its amplitude follows cos(w n dt) with Yee's discrete dispersion
    sin(w dt / 2) = (c dt / h) sin(k h / 2), not w = c k."""
    n, m, h = (32, 2, 2), 3, 1e-3
    dt = 0.5 * h / (C * np.sqrt(3.0))
    k = 2 * np.pi * m / (n[0] * h)
    o = po.Oracle(n, (2, 2, 2), (h, h, h), dt, form=form)
    o.load(np.zeros(0), np.zeros(0), np.zeros(0), np.zeros(0), np.zeros(0), np.zeros(0), np.zeros(0))
    mode = np.broadcast_to(np.cos(k * (np.arange(n[0]) + 0.5) * h)[:, None, None], n)
    f = [np.zeros(n) for _ in range(9)]
    f[1] = 100.0 * mode
    o.set_fields(f)
    w = 2.0 / dt * np.arcsin(C * dt / h * np.sin(k * h / 2))
    assert abs(w / (C * k) - 1) > 1e-3   # the discrete frequency is measurably not c k
    steps = 40
    for s in range(1, steps + 1):
        o.step(1)
        ey = o.get_fields()[1]
        a = np.sum(ey * mode) / np.sum(mode * mode)
        assert abs(a / 100.0 - np.cos(w * s * dt)) < tol, s
        assert np.max(np.abs(ey - a * mode)) < tol * 100.0   # still the same mode


@pytest.mark.parametrize("form,shape,deposit,tol", [
    (po.FORM_FP64_PLAIN, po.SHAPE_CIC, po.DEPOSIT_DIRECT, 1e-12),
    (po.FORM_FP64_PLAIN, po.SHAPE_TSC, po.DEPOSIT_ESIRKEPOV, 1e-12),
    (po.FORM_FP32_CELL, po.SHAPE_CIC, po.DEPOSIT_ESIRKEPOV, 2e-5),
    (po.FORM_FP32_CELL, po.SHAPE_TSC, po.DEPOSIT_ESIRKEPOV, 2e-5),
])
def test_uniform_field_is_interpolated_exactly(form, shape, deposit, tol):
    """Constant-field interpolation is exact: in a uniform E with B = 0, one step
    changes every particle's normalised momentum by q E dt / (m c) (Boris without
    rotation), wherever it sits in its cell -- the CIC and TSC weights of every
    staggered component sum to one."""
    n = (8, 8, 8)
    d = thermal_inputs(n, 5, seed=31, u_sigma=0.05)
    npart = len(d["x"])
    w = np.mean(d["w"]) * (1.0 + np.arange(npart) / npart)   # unique (also in FP32): identify particles after the step
    o = po.Oracle(n, (4, 4, 4), d["h"], d["dt"], form=form, shape=shape, deposit=deposit)
    o.load(d["x"], d["y"], d["z"], d["ux"], d["uy"], d["uz"], w)
    e = (3.0e6, -1.5e6, 2.0e6)   # du ~ 1e-2, well above the rounding of u ~ 0.05
    o.set_fields([np.full(n, v) for v in e] + [np.zeros(n)] * 6)
    before = o.particles()
    o.step(1)
    after = o.particles()
    ib, ia = np.argsort(before["w"]), np.argsort(after["w"])
    assert np.array_equal(before["w"][ib], after["w"][ia])
    for c, k in enumerate(("ux", "uy", "uz")):
        du = after[k][ia] - before[k][ib]
        want = E * e[c] * d["dt"] / (ME * C)
        assert np.max(np.abs(du - want)) < tol * abs(want), k


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(po.REF_SO), "libpica_ref1d.so")),
                    reason="the harness over pica's 1D classes is not built here")
@pytest.mark.parametrize("n,sc,ppc,steps,seed,nspecies,u_sigma,field_amp", [
    (48, 4, 3, 30, 41, 2, 0.1, 2.0e3),    # electrons and ions (4 electron masses), longer run
    (20, 2, 6, 12, 42, 1, 0.25, 5.0e2),   # hot plasma, supercell edge 2
])
def test_oracle_matches_pica_1d_classes_live(n, sc, ppc, steps, seed, nspecies, u_sigma, field_amp):
    """The oracle on a grid one cell thick along y and z against pica's own 1D path
    (oracle/ref_harness_1d.cpp over YeeGrid<One>, FieldInterpolatorCIC and
    CurrentDepositorCIC of YeeGrid<One>, the 1D YeeSolver), run here on new inputs:
    fields and particles within 1e-12."""
    import ctypes as CT
    lib = CT.CDLL(os.path.join(os.path.dirname(po.REF_SO), "libpica_ref1d.so"))
    dp = CT.POINTER(CT.c_double)
    lib.ref1d_run.argtypes = [CT.c_int32, CT.c_double, CT.c_double, CT.c_double, CT.c_int32, dp, dp, CT.c_int64, dp,
                              dp, dp, dp, dp, CT.POINTER(CT.c_int32), dp, CT.c_int32]
    rng = np.random.default_rng(seed)
    h = 0.05 * C / np.sqrt(4 * np.pi * 1e18 * E * E / ME)
    dt = 0.5 * h / (C * np.sqrt(3.0))
    npart = n * ppc
    x = (np.repeat(np.arange(n), ppc) + rng.random(npart)) * h
    u = rng.normal(0.0, u_sigma, (3, npart))
    w = np.full(npart, 1e18 * h ** 3 / ppc) * (1.0 + 0.1 * rng.random(npart))
    sp = rng.integers(0, nspecies, npart).astype(np.int32)
    f = np.stack([field_amp * rng.standard_normal(n) for _ in range(6)] + [np.zeros(n)] * 3)
    mass, charge = np.array([ME, 4 * ME][:nspecies]), np.array([E, -E][:nspecies])
    xo, uo, fo = x.copy(), u.copy(), f.copy()

    def ptr(a):
        return a.ctypes.data_as(dp)

    ux, uy, uz = (np.ascontiguousarray(uo[i]) for i in range(3))
    assert lib.ref1d_run(n, h, h * h, dt, nspecies, ptr(mass), ptr(charge), npart, ptr(xo), ptr(ux), ptr(uy), ptr(uz),
                         ptr(w), sp.ctypes.data_as(CT.POINTER(CT.c_int32)), ptr(fo), steps) == 0

    o = po.Oracle((n, 1, 1), (sc, 1, 1), (h, h, h), dt, form=po.FORM_FP64_PLAIN, shape=po.SHAPE_CIC,
                  deposit=po.DEPOSIT_DIRECT, species=tuple(zip(mass, charge)))
    yz = np.full(npart, 0.5 * h)
    o.load(x, yz, yz, u[0], u[1], u[2], w, sp)
    o.set_fields([a.reshape(n, 1, 1) for a in f[:6]] + [np.zeros((n, 1, 1))] * 3)
    o.step(steps)
    got = o.get_fields()
    for c in range(9):
        assert rel_err(got[c].reshape(-1), fo[c]) <= 1e-12, c
    p = o.particles()
    mine, theirs = np.argsort(p["x"]), np.argsort(xo)
    for k, ref in (("x", xo), ("ux", ux), ("uy", uy), ("uz", uz)):
        assert rel_err(p[k][mine], ref[theirs]) <= 1e-12, k
    assert np.array_equal(p["species"][mine], sp[theirs])


def run_config1(kind, steps=100):
    from tests.helpers import config1_plasma, run_checksums
    sim, p = config1_plasma()
    o = po.Oracle(sim["n"], sim["supercell"], sim["h"], sim["dt"], kind=kind)
    o.load(*[p[k] for k in ("x", "y", "z", "ux", "uy", "uz", "w", "species")])
    o.set_fields([np.zeros(sim["n"])] * 9)
    return o, run_checksums(lambda: o.step(1), o.counts, o.migrations, steps)


def test_config1_restatement_reproduces_pica_fixture():
    """The plain FP64 32^3 x 50 ppc plasma, 100 steps, through the restatement: every
    checksum of tests/golden/config1_pica_100steps.npz (made by pica's own headers)
    equal bit for bit -- moves, counts and move lists every step, and the final
    counts, fields, particle sums and particle sample."""
    g = load_golden("config1_pica_100steps")
    o, (nm, cs, ms) = run_config1("port", int(g["steps"]))
    assert np.array_equal(nm, g["n_moves"]) and np.array_equal(cs, g["count_sums"])
    assert np.array_equal(ms, g["move_sums"])
    assert np.array_equal(o.counts(), g["counts"])
    q, f = o.particles(), o.get_fields()
    comps = ("x", "y", "z", "ux", "uy", "uz")
    assert np.array_equal([np.sum(a) for a in f], g["field_sum"])
    assert np.array_equal([np.sum(a * a) for a in f], g["field_sq"])
    assert np.array_equal([np.sum(q[k]) for k in comps], g["part_sum"])
    idx = g["sample_index"]
    assert np.array_equal(np.stack([q[k][idx] for k in comps], axis=1), g["sample"])
    assert np.array_equal(q["supercell"][idx], g["sample_supercell"])


@pytest.mark.skipif(not REFERENCE_AVAILABLE, reason="pica sources not mounted here")
def test_config1_restatement_matches_pica_headers_every_step():
    """The same 100 steps side by side, the restatement against the harness over pica's
    headers: per-supercell counts and migration lists equal after every step, particles
    and fields equal bit for bit at the end."""
    from tests.helpers import config1_plasma
    po.build(reference=True)
    sim, p = config1_plasma()
    pair = []
    for kind in ("port", "reference"):
        o = po.Oracle(sim["n"], sim["supercell"], sim["h"], sim["dt"], kind=kind)
        o.load(*[p[k] for k in ("x", "y", "z", "ux", "uy", "uz", "w", "species")])
        o.set_fields([np.zeros(sim["n"])] * 9)
        pair.append(o)
    a, b = pair
    for st in range(100):
        a.step(1)
        b.step(1)
        assert np.array_equal(a.counts(), b.counts()), st
        assert np.array_equal(a.migrations(), b.migrations()), st
    pa, pb = a.particles(), b.particles()
    for k in ("x", "y", "z", "ux", "uy", "uz", "w", "supercell"):
        assert np.array_equal(pa[k], pb[k]), k
    fa, fb = a.get_fields(), b.get_fields()
    for c in range(9):
        assert np.array_equal(fa[c], fb[c]), c
