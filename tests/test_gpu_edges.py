"""Edge cases against the oracle (GPU): no particles, a single particle, the
smallest and largest supercells, odd and ragged grids, a species with no
particles, supercells left empty by a cold beam."""
import numpy as np
import pytest

import pica_gb300 as pg
from oracle import pic_oracle as po
from tests.helpers import ME, E, particle_args, periodic_err, rel_err, thermal_inputs

pytestmark = pytest.mark.gpu


def run_both(n, sc, d, steps, form, shape, deposit, species=(pg.ELECTRON,), fields=None, resort_every=0):
    s = pg.Simulation(n, d["h"], d["dt"], supercell=sc, form=form, shape=shape, deposit=deposit, species=species,
                      resort_every=resort_every)
    o = po.Oracle(n, sc, d["h"], d["dt"], form=form, shape=shape, deposit=deposit, species=species,
                  resort_every=resort_every)
    s.upload_particles(*particle_args(d))
    o.load(*particle_args(d))
    f9 = fields if fields is not None else [np.zeros(n)] * 9
    s.upload_fields(f9)
    o.set_fields(f9)
    for st in range(steps):
        s.step(1)
        o.step(1)
        assert np.array_equal(s.counts(), o.counts()), st
    return s, o


def check(s, o, n, h, form):
    tol_x, tol = (1e-12, 1e-12) if form == pg.FORM_FP64_PLAIN else (1e-6, 1e-4)
    ps, pr = s.particles(), o.particles()
    assert np.array_equal(ps["supercell"], pr["supercell"])
    L = [n[k] * h[k] for k in range(3)]
    for k, key in enumerate(("x", "y", "z")):
        assert periodic_err(ps[key], pr[key], L[k]) <= tol_x, key
    for key in ("ux", "uy", "uz"):
        assert rel_err(ps[key], pr[key]) <= tol, key
    fs, fo = s.fields(), o.get_fields()
    for c in range(9):
        assert rel_err(fs[c], fo[c]) <= tol, c


def subset(d, idx):
    out = dict(d)
    for k in ("x", "y", "z", "ux", "uy", "uz", "w", "species"):
        out[k] = d[k][idx]
    return out


FORMS = [(pg.FORM_FP64_PLAIN, pg.SHAPE_CIC, pg.DEPOSIT_DIRECT), (pg.FORM_FP32_CELL, pg.SHAPE_TSC, pg.DEPOSIT_ESIRKEPOV),
         (pg.FORM_FP32_CELL, pg.SHAPE_CIC, pg.DEPOSIT_ESIRKEPOV)]


@pytest.mark.parametrize("form,shape,dep", FORMS)
def test_no_particles_is_the_field_solver(form, shape, dep):
    n, sc = (8, 8, 8), (4, 4, 4)
    d = subset(thermal_inputs(n, 1, seed=61), np.arange(0))
    rng = np.random.default_rng(62)
    f9 = [rng.standard_normal(n) for _ in range(6)] + [np.zeros(n)] * 3
    s, o = run_both(n, sc, d, 3, form, shape, dep, fields=f9)
    assert s.num_particles() == 0
    check(s, o, n, d["h"], form)


@pytest.mark.parametrize("form,shape,dep", FORMS)
def test_single_particle(form, shape, dep):
    n, sc = (8, 8, 8), (4, 4, 4)
    d = subset(thermal_inputs(n, 1, seed=63, u_sigma=0.3), np.array([137]))
    s, o = run_both(n, sc, d, 6, form, shape, dep)
    assert s.num_particles() == 1
    check(s, o, n, d["h"], form)


@pytest.mark.parametrize("form,shape,dep", FORMS)
@pytest.mark.parametrize("n,sc", [((4, 4, 4), (1, 1, 1)), ((16, 16, 16), (8, 8, 8)), ((6, 10, 14), (2, 2, 2)),
                                  ((12, 8, 4), (3, 4, 2))])
def test_supercell_sizes_and_ragged_grids(n, sc, form, shape, dep):
    d = thermal_inputs(n, 3, seed=64, u_sigma=0.15)
    s, o = run_both(n, sc, d, 4, form, shape, dep, resort_every=2)
    check(s, o, n, d["h"], form)


@pytest.mark.parametrize("form,shape,dep", FORMS)
def test_species_without_particles_and_empty_supercells(form, shape, dep):
    """Two species, all particles in the first; a cold beam fills one x-slab only, so
    most supercells stay empty while the beam crosses into them."""
    n, sc = (16, 8, 8), (4, 4, 4)
    d = thermal_inputs(n, 2, seed=65, u_sigma=0.01, drift=(0.3, 0.0, 0.0))
    keep = np.nonzero(d["x"] < 3.0 * d["h"][0])[0]
    d = subset(d, keep)
    d["species"] = np.zeros(len(keep), np.int32)
    ion = (100.0 * ME, -E)
    s, o = run_both(n, sc, d, 8, form, shape, dep, species=((ME, E), ion))
    assert s.counts()[1].sum() == 0
    check(s, o, n, d["h"], form)


@pytest.mark.parametrize("form,shape,dep", FORMS)
@pytest.mark.parametrize("n,sc", [((16, 8, 1), (4, 4, 1)), ((32, 1, 1), (4, 1, 1))])
def test_two_and_one_dimensional_grids(n, sc, form, shape, dep):
    """A grid one cell thick along z (2D) or along y and z (1D), periodic: the 3D step
    reduces to the 2D / 1D one (the derivatives along a one-cell periodic axis are exact
    zeros, and the gather and deposit along it sum their weights on the single node).
    Against the oracle on the same grid."""
    d = thermal_inputs(n, 6, seed=66, u_sigma=0.15)
    rng = np.random.default_rng(67)
    f9 = [1e3 * rng.standard_normal(n) for _ in range(6)] + [np.zeros(n)] * 3
    s, o = run_both(n, sc, d, 5, form, shape, dep, fields=f9, resort_every=2)
    check(s, o, n, d["h"], form)


@pytest.mark.parametrize("form,shape,dep", FORMS)
def test_reorder_sorts_each_supercell_like_the_oracle_load(form, shape, dep):
    """pica_reorder (EnsembleOrdered::reorder's role): after steps without a resort the
    particles are out of cell order; reordering gives each supercell its live particles
    by (cell, slot), the order the oracle's stable load of the same particles gives."""
    n, sc = (8, 8, 8), (4, 4, 4)
    d = thermal_inputs(n, 6, seed=68, u_sigma=0.3)
    s = pg.Simulation(n, d["h"], d["dt"], supercell=sc, form=form, shape=shape, deposit=dep)
    s.upload_particles(*particle_args(d))
    s.upload_fields([np.zeros(n)] * 9)
    s.step(4)
    before = s.particles()
    s.reorder()
    after = s.particles()
    o = po.Oracle(n, sc, d["h"], d["dt"], form=form, shape=shape, deposit=dep)
    o.load(*[before[k] for k in ("x", "y", "z", "ux", "uy", "uz", "w", "species")])
    ref = o.particles()
    assert np.array_equal(s.counts(), o.counts())
    for k in ("species", "supercell", "ux", "uy", "uz", "w"):
        assert np.array_equal(after[k], ref[k]), k
    # Positions pass through the oracle's load (FP32 form: back to cell + offset), so to
    # the rounding of that conversion; an order difference would show as O(h).
    for k in ("x", "y", "z"):
        assert np.max(np.abs(after[k] - ref[k])) <= 1e-9 * d["h"][0], k
    s.step(1)   # the context steps on from the new order
    assert s.num_particles() == len(before["x"])
    s.close()
