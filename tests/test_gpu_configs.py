"""Parity cases shaped like the two-stream and Weibel workloads, at sizes the
oracle finishes in seconds: GPU (through the C ABI) against the oracle from the
same generated plasma.  FP64 plain form within 1e-12; FP32 cell form within
1e-4 (momenta, fields) and 1e-6 of the box (positions); per-supercell counts and
the supercell of every particle exactly equal."""
import math

import numpy as np
import pytest

import pica_gb300 as pg
from oracle import pic_oracle as po
from pica_gb300 import workloads
from tests.helpers import periodic_err, rel_err

pytestmark = pytest.mark.gpu


def beta_u(beta):
    return beta / math.sqrt(1.0 - beta * beta)


def two_stream_case():
    """Two electron beams at +-0.2c along x, thermal 0.01, density 1 + 0.9 cos(2 pi x / Lx)
    (cell counts round(8 (1 + 0.9 cos)) split between the beams), CIC, Esirkepov, resort every 4."""
    n = (16, 8, 8)
    h = workloads.cell_size()
    hh = (h, h, h)
    spec = pg.plasma_spec(n, hh, 8, 0.01, workloads.N0 * h ** 3 / 8, 77, density_mod=0.9, nbeams=2,
                          drift_u=beta_u(0.2), drift_axis=0)
    parts = [pg.generate_plasma(spec)]
    sim = dict(n=n, h=hh, dt=workloads.time_step(h), supercell=(4, 4, 4), shape=pg.SHAPE_CIC,
               deposit=pg.DEPOSIT_ESIRKEPOV, species=(pg.ELECTRON,), resort_every=4)
    return sim, parts, 12


def weibel_case():
    """Counter-streaming electrons and mobile ions (m_i = 100 m_e), beams +-0.3c along z,
    thermal 0.01 (ions 0.001), 2 x 2 particles per cell per species, TSC, Esirkepov."""
    n = (8, 8, 12)
    h = workloads.cell_size()
    hh = (h, h, h)
    ion = (pg.ELECTRON_MASS * 100.0, -pg.ELECTRON_CHARGE)
    w = workloads.N0 * h ** 3 / 4
    specs = [pg.plasma_spec(n, hh, 4, 0.01, w, 78, species=0, nbeams=2, drift_u=beta_u(0.3), drift_axis=2),
             pg.plasma_spec(n, hh, 4, 0.001, w, 79, species=1, nbeams=2, drift_u=beta_u(0.3), drift_axis=2)]
    parts = [pg.generate_plasma(s) for s in specs]
    sim = dict(n=n, h=hh, dt=workloads.time_step(h), supercell=(4, 4, 4), shape=pg.SHAPE_TSC,
               deposit=pg.DEPOSIT_ESIRKEPOV, species=(pg.ELECTRON, ion), resort_every=3)
    return sim, parts, 10


def joined(parts):
    return [np.concatenate([p[k] for p in parts]) for k in ("x", "y", "z", "ux", "uy", "uz", "w", "species")]


@pytest.mark.parametrize("form", [pg.FORM_FP64_PLAIN, pg.FORM_FP32_CELL])
@pytest.mark.parametrize("case", [two_stream_case, weibel_case])
def test_config_shaped_case_matches_oracle(case, form):
    sim, parts, steps = case()
    args = joined(parts)
    s = pg.Simulation(form=form, **sim)
    o = po.Oracle(sim["n"], sim["supercell"], sim["h"], sim["dt"], form=form, shape=sim["shape"],
                  deposit=sim["deposit"], species=sim["species"], resort_every=sim["resort_every"])
    s.upload_particles(*args)
    o.load(*args)
    zeros = [np.zeros(sim["n"])] * 9
    s.upload_fields(zeros)
    o.set_fields(zeros)
    for st in range(steps):
        s.step(1)
        o.step(1)
        assert np.array_equal(s.counts(), o.counts()), st
    ps, pr = s.particles(), o.particles()
    assert np.array_equal(ps["supercell"], pr["supercell"])
    assert np.array_equal(ps["species"], pr["species"])
    L = [sim["n"][k] * sim["h"][k] for k in range(3)]
    tol_x, tol = (1e-12, 1e-12) if form == pg.FORM_FP64_PLAIN else (1e-6, 1e-4)
    for k, key in enumerate(("x", "y", "z")):
        assert periodic_err(ps[key], pr[key], L[k]) < tol_x, key
    for key in ("ux", "uy", "uz"):
        assert rel_err(ps[key], pr[key]) < tol, key
    fs, fo = s.fields(), o.get_fields()
    for c in range(9):
        assert rel_err(fs[c], fo[c]) < tol, c
    s.close()
