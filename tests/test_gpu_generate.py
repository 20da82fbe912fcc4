"""Device plasma generator (pica_generate_plasma) against the host generator
followed by pica_upload_particles, and the generated state stepped against the
oracle.  Counts, supercells, species and weights equal exactly; offsets within
one FP32 ulp of the cell (the device rounds the uniform draw, the host x/h - i);
momenta within one FP32 ulp (device log and cos)."""
import numpy as np
import pytest

import pica_gb300 as pg
from oracle import pic_oracle as po
from pica_gb300 import workloads
from tests.helpers import ME, E, periodic_err, rel_err

pytestmark = pytest.mark.gpu

ION = (100.0 * ME, -E)


def populations(n):
    """Two electron populations (a modulated two-beam plasma and a drifting thermal one)
    and one ion population, as in the two-stream and Weibel workloads."""
    h = workloads.cell_size()
    hh = (h, h, h)
    w = workloads.N0 * h ** 3 / 8
    return hh, [pg.plasma_spec(n, hh, 6, 0.05, w, 901, species=0, density_mod=0.5, nbeams=2, drift_u=0.2,
                               drift_axis=0),
                pg.plasma_spec(n, hh, 3, 0.02, 2 * w, 902, species=0, drift_u=-0.1, drift_axis=2),
                pg.plasma_spec(n, hh, 4, 0.002, w, 903, species=1, nbeams=2, drift_u=0.3, drift_axis=1)]


def host_upload(sim, specs):
    parts = [pg.generate_plasma(s) for s in specs]
    args = [np.concatenate([p[k] for p in parts]) for k in ("x", "y", "z", "ux", "uy", "uz", "w", "species")]
    sim.upload_particles(*args)


def make(n, hh, shape=pg.SHAPE_TSC):
    return pg.Simulation(n, hh, workloads.time_step(hh[0]), supercell=(4, 4, 4), form=pg.FORM_FP32_CELL, shape=shape,
                         deposit=pg.DEPOSIT_ESIRKEPOV, species=(pg.ELECTRON, ION), resort_every=2)


def test_device_generator_equals_host_generator_and_upload():
    n = (16, 8, 12)
    hh, specs = populations(n)
    dev, host = make(n, hh), make(n, hh)
    dev.generate_plasma(specs)
    host_upload(host, specs)
    assert np.array_equal(dev.counts(), host.counts())
    expect = [sum(int(dev.lib.pica_plasma_count(s)) for s in specs if s.species == q) for q in range(2)]
    assert dev.counts().sum(axis=1).tolist() == expect
    pd, ph = dev.particles(), host.particles()
    for k in ("species", "supercell", "w"):
        assert np.array_equal(pd[k], ph[k]), k
    h = hh[0]
    for k in ("x", "y", "z"):
        assert np.max(np.abs(pd[k] - ph[k])) <= 1.2e-7 * h, k
    for k in ("ux", "uy", "uz"):
        assert np.all(np.abs(pd[k] - ph[k]) <= 1.2e-7 * np.abs(ph[k])), k
    assert dev.step_count() == 0
    dev.close()
    host.close()


@pytest.mark.parametrize("shape", [pg.SHAPE_CIC, pg.SHAPE_TSC])
def test_generated_state_steps_like_the_oracle(shape):
    n = (8, 8, 8)
    hh, specs = populations(n)
    s = make(n, hh, shape)
    s.generate_plasma(specs)
    p = s.particles()
    o = po.Oracle(n, (4, 4, 4), hh, s.dt, form=pg.FORM_FP32_CELL, shape=shape, deposit=pg.DEPOSIT_ESIRKEPOV,
                  species=(pg.ELECTRON, ION), resort_every=2)
    o.load(p["x"], p["y"], p["z"], p["ux"], p["uy"], p["uz"], p["w"], p["species"])
    zeros = [np.zeros(n)] * 9
    s.upload_fields(zeros)
    o.set_fields(zeros)
    for st in range(5):
        s.step(1)
        o.step(1)
        assert np.array_equal(s.counts(), o.counts()), st
    ps, pr = s.particles(), o.particles()
    assert np.array_equal(ps["supercell"], pr["supercell"])
    L = [n[k] * hh[k] for k in range(3)]
    for k, key in enumerate(("x", "y", "z")):
        assert periodic_err(ps[key], pr[key], L[k]) <= 1e-6, key
    for key in ("ux", "uy", "uz"):
        assert rel_err(ps[key], pr[key]) <= 1e-4, key
    fs, fo = s.fields(), o.get_fields()
    for c in range(9):
        assert rel_err(fs[c], fo[c]) <= 1e-4, c
    s.close()


def test_generator_rejects_bad_requests():
    n = (8, 8, 8)
    hh, specs = populations(n)
    s = make(n, hh)
    with pytest.raises(pg.PicaError):
        s.generate_plasma([])
    with pytest.raises(pg.PicaError):   # another grid
        s.generate_plasma(pg.plasma_spec((8, 8, 4), hh, 2, 0.05, 1.0, 1))
    with pytest.raises(pg.PicaError):   # species the context does not have
        s.generate_plasma(pg.plasma_spec(n, hh, 2, 0.05, 1.0, 1, species=2))
    with pytest.raises(pg.PicaError):   # three beams
        s.generate_plasma(pg.plasma_spec(n, hh, 2, 0.05, 1.0, 1, nbeams=3))
    with pytest.raises(pg.PicaError):   # nine populations of one species
        s.generate_plasma([pg.plasma_spec(n, hh, 1, 0.05, 1.0, k) for k in range(9)])
    s.generate_plasma(specs)            # the context stays usable
    assert s.num_particles() > 0
    s.close()
    f64 = pg.Simulation(n, hh, workloads.time_step(hh[0]), supercell=(4, 4, 4), form=pg.FORM_FP64_PLAIN)
    with pytest.raises(pg.PicaError):
        f64.generate_plasma(pg.plasma_spec(n, hh, 2, 0.05, 1.0, 1))
    f64.close()
