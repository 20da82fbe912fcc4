"""GPU parity tests: the CUDA library (through the C ABI) against the golden
fixtures made by pica's own headers and against the oracle restatement.

Tolerances (written per test): FP64 plain form within 1e-12 relative (the only
difference is the order of the J sums: shared-memory and global atomics);
integer results (per-supercell counts, migration order, supercell of every
particle) exactly equal.  FP32 form against the FP32 oracle: 1e-4 on
particle momenta and fields (FMA contraction and atomic order differ)."""
import numpy as np
import pytest

import pica_gb300 as pg
from oracle import pic_oracle as po
from tests.helpers import elem_err, load_golden, particle_args, periodic_err, rel_err, run_1d_golden, species_of, thermal_inputs

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12


def gpu_sim(n, sc, h, dt, **kw):
    return pg.Simulation(n, h, dt, supercell=sc, **kw)


def compare_particles(pg_, po_, L, tol_x, tol_u):
    assert np.array_equal(pg_["supercell"], po_["supercell"])
    assert np.array_equal(pg_["species"], po_["species"])
    for d, k in enumerate(("x", "y", "z")):
        assert periodic_err(pg_[k], po_[k], L[d]) < tol_x, k
    for k in ("ux", "uy", "uz"):
        assert rel_err(pg_[k], po_[k]) < tol_u, k
    assert np.array_equal(pg_["w"], po_["w"]) or rel_err(pg_["w"], po_["w"]) < 1e-7


@pytest.mark.parametrize("name", ["cic_direct_8cube", "cic_direct_2species"])
def test_fp64_matches_reference_golden(name):
    g = load_golden(name)
    n, sc, h = tuple(g["n"]), tuple(g["sc"]), tuple(g["h"])
    s = gpu_sim(n, sc, h, float(g["dt"]), species=species_of(g), resort_every=int(g["resort_every"]))
    s.upload_particles(g["in_x"], g["in_y"], g["in_z"], g["in_ux"], g["in_uy"], g["in_uz"], g["in_w"], g["in_species"])
    s.upload_fields(list(g["in_fields"]))
    for st in range(int(g["steps"])):
        s.step(1)
        assert np.array_equal(s.counts(), g["counts"][st]), st
    p = s.particles()
    ref = {k: g["out_" + k] for k in ("x", "y", "z", "ux", "uy", "uz", "w", "species", "supercell")}
    L = [n[d] * h[d] for d in range(3)]
    compare_particles(p, ref, L, FP64_TOL, FP64_TOL)
    f = s.fields()
    for c in range(9):
        assert rel_err(f[c], g["out_fields"][c]) < FP64_TOL, c


def run_pair(n, sc, d, steps, form, shape, deposit, species=(pg.ELECTRON,), fields=None, slack=0.15, resort_every=0):
    s = gpu_sim(n, sc, d["h"], d["dt"], form=form, shape=shape, deposit=deposit, species=species, slack=slack,
                resort_every=resort_every)
    o = po.Oracle(n, sc, d["h"], d["dt"], form=form, shape=shape, deposit=deposit, species=species,
                  resort_every=resort_every)
    s.upload_particles(*particle_args(d))
    o.load(*particle_args(d))
    f9 = fields if fields is not None else [np.zeros(n)] * 9
    s.upload_fields(f9)
    o.set_fields(f9)
    s.record_migrations(True)
    for st in range(steps):
        s.step(1)
        o.step(1)
        assert np.array_equal(s.counts(), o.counts()), st
        assert np.array_equal(s.migrations(), o.migrations()), st
    return s, o


@pytest.mark.parametrize("shape,deposit", [(pg.SHAPE_CIC, pg.DEPOSIT_DIRECT), (pg.SHAPE_CIC, pg.DEPOSIT_ESIRKEPOV),
                                           (pg.SHAPE_TSC, pg.DEPOSIT_DIRECT), (pg.SHAPE_TSC, pg.DEPOSIT_ESIRKEPOV)])
def test_fp64_forms_match_oracle(shape, deposit):
    n, sc = (12, 8, 16), (4, 2, 4)
    d = thermal_inputs(n, 5, seed=21, u_sigma=0.1, hscale=(1.0, 1.2, 0.8), nspecies=2)
    rng = np.random.default_rng(2)
    fields = [2e3 * rng.standard_normal(n) for _ in range(6)] + [np.zeros(n)] * 3
    species = (pg.ELECTRON, (pg.ELECTRON_MASS * 100.0, -pg.ELECTRON_CHARGE))
    s, o = run_pair(n, sc, d, 6, pg.FORM_FP64_PLAIN, shape, deposit, species=species, fields=fields)
    L = [n[k] * d["h"][k] for k in range(3)]
    compare_particles(s.particles(), o.particles(), L, FP64_TOL, FP64_TOL)
    fs, fo = s.fields(), o.get_fields()
    for c in range(9):
        assert rel_err(fs[c], fo[c]) < FP64_TOL, c


def test_fp64_thermal_32cube_100_steps():
    """The plain FP64 32^3 x 50 ppc electron plasma (CIC, Boris, direct, supercell 2^3) for 100 steps:
    per-supercell counts and the migration list (species, source supercell, source slot,
    destination) exactly equal after every step; particles and fields within 1e-12."""
    from pica_gb300 import workloads
    wl = workloads.config1()
    p = pg.generate_plasma(wl["specs"][0])
    sim = wl["sim"]
    s = pg.Simulation(**sim)
    o = po.Oracle(sim["n"], sim["supercell"], sim["h"], sim["dt"])
    args = [p[k] for k in ("x", "y", "z", "ux", "uy", "uz", "w")] + [p["species"]]
    s.upload_particles(*args)
    o.load(*args)
    zeros = [np.zeros(sim["n"])] * 9
    s.upload_fields(zeros)
    o.set_fields(zeros)
    s.record_migrations(True)
    moved = 0
    for st in range(100):
        s.step(1)
        o.step(1)
        assert np.array_equal(s.counts(), o.counts()), st
        m = s.migrations()
        assert np.array_equal(m, o.migrations()), st
        moved += len(m)
    assert moved > 0
    L = [sim["n"][k] * sim["h"][k] for k in range(3)]
    ps, po_ = s.particles(), o.particles()
    compare_particles(ps, po_, L, FP64_TOL, FP64_TOL)
    for k in ("ux", "uy", "uz"):   # also element by element, floor 1e-3 of the largest |u|
        assert elem_err(ps[k], po_[k]) < FP64_TOL, k
    fs, fo = s.fields(), o.get_fields()
    for c in range(9):
        assert rel_err(fs[c], fo[c]) < FP64_TOL, c


@pytest.mark.parametrize("shape,deposit", [(pg.SHAPE_CIC, pg.DEPOSIT_DIRECT), (pg.SHAPE_CIC, pg.DEPOSIT_ESIRKEPOV),
                                           (pg.SHAPE_TSC, pg.DEPOSIT_DIRECT), (pg.SHAPE_TSC, pg.DEPOSIT_ESIRKEPOV)])
def test_fp32_cell_form_matches_oracle(shape, deposit):
    n, sc = (16, 8, 8), (4, 4, 2)
    d = thermal_inputs(n, 6, seed=31, u_sigma=0.1)
    s, o = run_pair(n, sc, d, 5, pg.FORM_FP32_CELL, shape, deposit)
    ps, pr = s.particles(), o.particles()
    L = [n[k] * d["h"][k] for k in range(3)]
    assert np.array_equal(ps["supercell"], pr["supercell"])
    for k, key in enumerate(("x", "y", "z")):
        assert periodic_err(ps[key], pr[key], L[k]) < 1e-6
    for key in ("ux", "uy", "uz"):
        assert rel_err(ps[key], pr[key]) < 1e-4
    fs, fo = s.fields(), o.get_fields()
    for c in range(9):
        assert rel_err(fs[c], fo[c]) < 1e-4, c


def test_fp64_yee_update_bit_exact():
    """With no particles the step is YeeSolver only: bit-exact against the oracle."""
    n = (8, 12, 6)
    d = thermal_inputs(n, 1, seed=1)
    rng = np.random.default_rng(4)
    f9 = [rng.standard_normal(n) for _ in range(6)] + [np.zeros(n)] * 3
    s = gpu_sim(n, (2, 2, 2), d["h"], d["dt"])
    o = po.Oracle(n, (2, 2, 2), d["h"], d["dt"])
    s.upload_fields(f9)
    o.set_fields(f9)
    s.step(3)
    o.step(3)
    fs, fo = s.fields(), o.get_fields()
    for c in range(9):
        assert np.array_equal(fs[c], fo[c]), c


def test_migration_overflow_rebuild_keeps_order():
    """A cold beam concentrates particles into a supercell with no spare room: the
    in-place append overflows, the layout is rebuilt, and the order stays canonical."""
    n, sc = (16, 4, 4), (2, 2, 2)
    d = thermal_inputs(n, 2, seed=41, u_sigma=1e-4)
    # Pack 120 particles near the +x face of supercell x=0 moving +x fast: supercell x=1 gets all.
    h = d["h"]
    m = 120
    rng = np.random.default_rng(5)
    x = np.concatenate([d["x"], (1.97 + 0.02 * rng.random(m)) * h[0]])
    y = np.concatenate([d["y"], 0.5 * h[1] + 0 * rng.random(m)])
    z = np.concatenate([d["z"], 0.5 * h[2] + rng.random(m) * h[2]])
    ux = np.concatenate([d["ux"], np.full(m, 3.0)])
    uy = np.concatenate([d["uy"], np.zeros(m)])
    uz = np.concatenate([d["uz"], np.zeros(m)])
    w = np.concatenate([d["w"], np.full(m, d["w"][0])])
    sp = np.zeros(len(x), np.int32)
    dd = dict(h=h, dt=d["dt"], x=x, y=y, z=z, ux=ux, uy=uy, uz=uz, w=w, species=sp)
    s, o = run_pair(n, sc, dd, 4, pg.FORM_FP64_PLAIN, pg.SHAPE_CIC, pg.DEPOSIT_DIRECT, slack=1e-9)
    L = [n[k] * h[k] for k in range(3)]
    compare_particles(s.particles(), o.particles(), L, FP64_TOL, FP64_TOL)


@pytest.mark.parametrize("form", [pg.FORM_FP64_PLAIN, pg.FORM_FP32_CELL])
def test_resort_cadence_matches_oracle_order(form):
    """With a resort every 2 steps (compact + sort each supercell by cell) the GPU
    keeps the oracle's exact ensemble order; without it the order differs but the
    particles are the same.  FP32: each lane pre-sums its particles' window
    contributions in FP32 before the exact fixed-point deposit, so the in-supercell
    order moves results by FP32 rounding (checked to 1e-6); for a given order the
    results are bit-reproducible (test_fp32_deposit_is_deterministic)."""
    n, sc = (8, 8, 8), (2, 2, 2)
    d = thermal_inputs(n, 4, seed=12, u_sigma=0.2)
    tol = 1e-12 if form == pg.FORM_FP64_PLAIN else 1e-5
    runs = []
    for every in (0, 2):
        s, o = run_pair(n, sc, d, 5, form, pg.SHAPE_CIC, pg.DEPOSIT_ESIRKEPOV, resort_every=every)
        ps, pr = s.particles(), o.particles()
        assert np.array_equal(ps["supercell"], pr["supercell"])
        assert rel_err(ps["ux"], pr["ux"]) < tol
        runs.append(ps)
    key = lambda p: np.lexsort((p["uz"], p["uy"], p["ux"], p["supercell"]))
    a, b = runs[0], runs[1]
    ia, ib = key(a), key(b)
    for k in ("x", "ux", "w"):
        if form == pg.FORM_FP32_CELL:
            assert rel_err(a[k][ia], b[k][ib]) < 1e-6, k
        else:
            assert rel_err(a[k][ia], b[k][ib]) < 1e-12, k


def test_fp32_deposit_is_deterministic():
    """Two identical FP32 runs agree bit for bit (the J sums are exact integers)."""
    n, sc = (8, 8, 8), (4, 4, 4)
    d = thermal_inputs(n, 8, seed=13, u_sigma=0.2)
    out = []
    for _ in range(2):
        s = gpu_sim(n, sc, d["h"], d["dt"], form=pg.FORM_FP32_CELL, shape=pg.SHAPE_TSC, deposit=pg.DEPOSIT_ESIRKEPOV)
        s.upload_particles(*particle_args(d))
        s.upload_fields([np.zeros(n)] * 9)
        s.step(4)
        out.append((s.particles(), s.fields()))
    for k in ("x", "y", "z", "ux", "uy", "uz"):
        assert np.array_equal(out[0][0][k], out[1][0][k]), k
    for c in range(9):
        assert np.array_equal(out[0][1][c], out[1][1][c]), c


def test_diagnostics_match_oracle():
    n, sc = (8, 8, 8), (4, 4, 4)
    d = thermal_inputs(n, 6, seed=7)
    for form in (pg.FORM_FP64_PLAIN, pg.FORM_FP32_CELL):
        s, o = run_pair(n, sc, d, 3, form, pg.SHAPE_TSC, pg.DEPOSIT_ESIRKEPOV)
        bg = 4.80320427e-10 * 1e18
        ds, do = s.diagnostics(bg), o.diagnostics(bg)
        tol = 1e-12 if form == pg.FORM_FP64_PLAIN else 1e-4
        for k in ("field_energy", "kinetic_energy", "total_charge", "gauss_max", "rho_max"):
            assert abs(ds[k] - do[k]) <= tol * abs(do[k]), (form, k, ds[k], do[k])
        assert rel_err(s.charge_density(), o.charge_density()) < tol


def test_upload_download_roundtrip_and_order():
    n, sc = (8, 8, 8), (2, 4, 2)
    d = thermal_inputs(n, 3, seed=17, nspecies=2)
    s = gpu_sim(n, sc, d["h"], d["dt"], species=(pg.ELECTRON, pg.ELECTRON))
    o = po.Oracle(n, sc, d["h"], d["dt"], species=(pg.ELECTRON, pg.ELECTRON))
    s.upload_particles(*particle_args(d))
    o.load(*particle_args(d))
    p, q = s.particles(), o.particles()
    for k in ("x", "y", "z", "ux", "uy", "uz", "w", "species", "supercell"):
        assert np.array_equal(p[k], q[k]), k
    assert np.array_equal(s.counts(), o.counts())


def test_error_paths_do_not_fault():
    n = (8, 8, 8)
    d = thermal_inputs(n, 2, seed=3)
    s = gpu_sim(n, (2, 2, 2), d["h"], d["dt"])
    s.upload_particles(*particle_args(d))
    s.push_deposit()
    with pytest.raises(pg.PicaError) as e:
        s.push_deposit()
    assert e.value.status == -6
    s.migrate()
    # A time step far above the Courant limit moves a relativistic particle across
    # more than one supercell: reported as an error, no device fault.
    s2 = gpu_sim(n, (1, 1, 1), d["h"], 40 * d["h"][0] / 2.9979e10)
    s2.upload_particles([0.5 * d["h"][0]], [0.5 * d["h"][1]], [0.5 * d["h"][2]], [50.0], [0.0], [0.0], [1.0])
    with pytest.raises(pg.PicaError) as e:
        s2.step(1)
    assert e.value.status == -5
    # The context stays usable.
    s.step(2)
    assert s.num_particles() == len(d["x"])


@pytest.mark.parametrize("n", [(16, 8, 8), (16, 16, 24)])
@pytest.mark.parametrize("shape", [pg.SHAPE_CIC, pg.SHAPE_TSC])
def test_push_variants_give_identical_results(shape, n):
    """Every launch variant of the FP32 charge-conserving push kernel gives the same
    particles and fields bit for bit (the J sums are exact integers), from random
    E and B.  On the 16 x 16 x 24 grid the TMA variant (4) copies the E/B tile of
    the interior supercells (2 x 2 x 4 of 4 x 4 x 6) and loads the others; on the
    16 x 8 x 8 grid it has no tensor maps and launches as variant 0."""
    sc = (4, 4, 4)
    d = thermal_inputs(n, 10, seed=77, u_sigma=0.2)
    rng = np.random.default_rng(9)
    f9 = [1e3 * rng.standard_normal(n) for _ in range(6)] + [np.zeros(n)] * 3
    out = []
    _, count = gpu_sim(n, sc, d["h"], d["dt"], form=pg.FORM_FP32_CELL).variant()
    assert count == 5
    for v in range(count):
        s = gpu_sim(n, sc, d["h"], d["dt"], form=pg.FORM_FP32_CELL, shape=shape, deposit=pg.DEPOSIT_ESIRKEPOV,
                    resort_every=3)
        s.set_variant(v)
        s.upload_particles(*particle_args(d))
        s.upload_fields(f9)
        s.step(6)
        out.append((s.particles(), s.fields()))
    for p, f in out[1:]:
        for k in ("x", "y", "z", "ux", "uy", "uz", "w", "supercell"):
            assert np.array_equal(p[k], out[0][0][k]), k
        for c in range(9):
            assert np.array_equal(f[c], out[0][1][c]), c


def test_autotune_picks_a_variant():
    from pica_gb300 import autotune
    n = (16, 16, 16)
    d = thermal_inputs(n, 8, seed=5)
    s = gpu_sim(n, (4, 4, 4), d["h"], d["dt"], form=pg.FORM_FP32_CELL, shape=pg.SHAPE_TSC,
                deposit=pg.DEPOSIT_ESIRKEPOV, resort_every=4)
    s.upload_particles(*particle_args(d))
    s.upload_fields([np.zeros(n)] * 9)
    times = autotune.tune_variant(s, steps=1)
    assert len(times) == s.variant()[1]
    assert s.variant()[0] == min(times, key=times.get)
    assert s.num_particles() == len(d["x"])


def test_fp64_one_cell_thick_grid_matches_pica_1d_classes():
    """The FP64 plain form on a grid one cell thick along y and z against pica's own 1D
    path (golden fixture from oracle/ref_harness_1d.cpp): fields and particles within
    FP64_TOL."""
    g = load_golden("pica_1d_cic_direct")
    sims = []

    def make(n3, sc, h3, dt):
        s = gpu_sim(n3, sc, h3, dt)
        sims.append(s)
        return s.upload_particles, s.upload_fields, s.step, s.fields, s.particles

    f, got, ref = run_1d_golden(make, g)
    for c in range(9):
        assert rel_err(f[c], g["out_fields"][c]) <= FP64_TOL, c
    for k in ("x", "ux", "uy", "uz"):
        assert rel_err(got[k], ref[k]) <= FP64_TOL, k
    sims[0].close()


def test_fp64_config1_matches_pica_headers_fixture():
    """The plain FP64 32^3 x 50 ppc plasma (CIC, Boris, direct, supercell 2^3) for 100
    steps on the GPU against tests/golden/config1_pica_100steps.npz, which pica's own
    headers made from the same plasma: number of moves, count checksum and move-list
    checksum equal after every step, final per-supercell counts and the supercell of
    every sampled particle equal; field and particle sums and the particle sample
    within 1e-12 (norm-wise; only the order of the FP64 current sums differs)."""
    from tests.helpers import config1_plasma, run_checksums
    g = load_golden("config1_pica_100steps")
    sim, p = config1_plasma()
    s = pg.Simulation(**sim)
    s.upload_particles(*[p[k] for k in ("x", "y", "z", "ux", "uy", "uz", "w", "species")])
    s.upload_fields([np.zeros(sim["n"])] * 9)
    s.record_migrations(True)
    nm, cs, ms = run_checksums(lambda: s.step(1), s.counts, s.migrations, int(g["steps"]))
    assert np.array_equal(nm, g["n_moves"])
    assert np.array_equal(cs, g["count_sums"])
    assert np.array_equal(ms, g["move_sums"])
    assert np.array_equal(s.counts(), g["counts"])
    q, f = s.particles(), s.fields()
    comps = ("x", "y", "z", "ux", "uy", "uz")
    # Sums are compared against the sum of magnitudes (a mean field or momentum near
    # zero cancels, and its sum carries the rounding of the terms, not of the total).
    fabs = [np.sum(np.abs(a)) for a in f]
    pabs = [np.sum(np.abs(q[k])) for k in comps]
    for name, got, want, scale in (("field_sum", [np.sum(a) for a in f], g["field_sum"], fabs),
                                   ("field_abs", fabs, g["field_abs"], fabs),
                                   ("field_sq", [np.sum(a * a) for a in f], g["field_sq"], g["field_sq"]),
                                   ("part_sum", [np.sum(q[k]) for k in comps], g["part_sum"], pabs),
                                   ("part_sq", [np.sum(q[k] * q[k]) for k in comps], g["part_sq"], g["part_sq"])):
        for c, (a, b, sc) in enumerate(zip(got, want, scale)):
            assert abs(a - b) <= FP64_TOL * abs(sc) or a == b, (name, c)
    idx = g["sample_index"]
    assert np.array_equal(q["supercell"][idx], g["sample_supercell"])
    for c, k in enumerate(comps):
        assert rel_err(q[k][idx], g["sample"][:, c]) < FP64_TOL, k
