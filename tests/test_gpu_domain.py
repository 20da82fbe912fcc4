"""Domain decomposition on the GPU: one plasma as 2 or 3 slab contexts on this GPU
(pica_gb300.domain: halo, current fold, particle exchange between the contexts)
against the same plasma in one context.

Checked after every step: the number of particles of every global supercell,
exactly.  At the end: the fields of every global cell and the particles (sorted
by global supercell and position), FP64 plain form (CIC, direct) within 1e-12,
FP32 cell form (TSC, Esirkepov) within 1e-5 for fields and 1e-6 of the box /
1e-4 for particles (norm-wise; the two runs sum the current of a face cell in a
different order: exact fixed point within a slab, one more FP32 addition across
its face; and FP64 positions move between frames by whole cells, one rounding).
"""
import numpy as np
import pytest

import pica_gb300 as pg
from pica_gb300 import domain
from tests.helpers import periodic_err, rel_err, thermal_inputs

pytestmark = pytest.mark.gpu


def global_counts(plan, doms, nsc_global):
    out = np.zeros((doms[0].nspecies, int(np.prod(nsc_global))), np.int32)
    S, G = plan.S, plan.G
    for r, d in enumerate(doms):
        c = d.sim.counts().reshape(d.nspecies, -1, nsc_global[1], nsc_global[2])
        own = c[:, G // S:(G + plan.w[r]) // S]
        gx0 = plan.x0[r] // S
        out.reshape(d.nspecies, nsc_global[0], nsc_global[1], nsc_global[2])[:, gx0:gx0 + own.shape[1]] = own
    return out


def gathered_particles(plan, doms, h0, L):
    keys = ("x", "y", "z", "ux", "uy", "uz", "w", "species")
    parts = []
    for r, d in enumerate(doms):
        p = d.sim.particles()
        p = {k: p[k] for k in keys}
        p["x"] = np.mod(p["x"] - (plan.G - plan.x0[r]) * h0, L[0])
        parts.append(p)
    return {k: np.concatenate([p[k] for p in parts]) for k in keys}


def canonical(p, h, nsc_global, S):
    sc = (np.floor(p["x"] / (S * h[0])).astype(np.int64) * nsc_global[1] +
          np.floor(p["y"] / (S * h[1])).astype(np.int64)) * nsc_global[2] + np.floor(p["z"] / (S * h[2])).astype(np.int64)
    order = np.lexsort((p["z"], p["y"], p["x"], sc, p["species"]))
    return {k: v[order] for k, v in p.items()}


@pytest.mark.parametrize("slabs", [2, 3])
@pytest.mark.parametrize("form", [pg.FORM_FP64_PLAIN, pg.FORM_FP32_CELL])
def test_slabs_equal_one_context(slabs, form):
    n, S = (32, 8, 8), 4
    d = thermal_inputs(n, 6, seed=41, u_sigma=0.15, nspecies=2)
    species = (pg.ELECTRON, (pg.ELECTRON_MASS * 100.0, -pg.ELECTRON_CHARGE))
    shape, dep = (pg.SHAPE_CIC, pg.DEPOSIT_DIRECT) if form == pg.FORM_FP64_PLAIN else (pg.SHAPE_TSC,
                                                                                      pg.DEPOSIT_ESIRKEPOV)
    rng = np.random.default_rng(5)
    f9 = [1e3 * rng.standard_normal(n) for _ in range(6)] + [np.zeros(n)] * 3
    kw = dict(form=form, shape=shape, deposit=dep, species=species)
    one = pg.Simulation(n, d["h"], d["dt"], supercell=(S, S, S), **kw)
    keys = ("x", "y", "z", "ux", "uy", "uz", "w")
    one.upload_particles(*[d[k] for k in keys], d["species"])
    one.upload_fields(f9)
    dec = domain.local_decomposition(n, d["h"], d["dt"], (S, S, S), slabs, **kw)
    plan = dec.plan
    p = {k: d[k] for k in keys + ("species",)}
    for dom, part, f in zip(dec.domains, domain.split_particles(plan, p, d["h"][0]), domain.split_fields(plan, f9)):
        dom.sim.upload_particles(*[part[k] for k in keys], part["species"])
        dom.sim.upload_fields(f)
    nsc = tuple(n[k] // S for k in range(3))
    assert np.array_equal(global_counts(plan, dec.domains, nsc), one.counts())
    for st in range(8):
        one.step(1)
        dec.step(1)
        assert np.array_equal(global_counts(plan, dec.domains, nsc), one.counts()), st
    fp64 = form == pg.FORM_FP64_PLAIN
    tol_f, tol_x, tol_u = (1e-12, 1e-12, 1e-12) if fp64 else (1e-5, 1e-6, 1e-4)
    fd = domain.gather_fields(plan, [dom.sim.fields() for dom in dec.domains])
    fo = one.fields()
    for c in range(9):
        assert rel_err(fd[c], fo[c]) < tol_f, c
    L = [n[k] * d["h"][k] for k in range(3)]
    a = canonical(gathered_particles(plan, dec.domains, d["h"][0], L), d["h"], nsc, S)
    b = canonical({k: v for k, v in one.particles().items() if k in keys + ("species",)}, d["h"], nsc, S)
    assert np.array_equal(a["species"], b["species"])
    for k, key in enumerate(("x", "y", "z")):
        assert periodic_err(a[key], b[key], L[k]) < tol_x, key
    for key in ("ux", "uy", "uz"):
        assert rel_err(a[key], b[key]) < tol_u, key
    one.close()
