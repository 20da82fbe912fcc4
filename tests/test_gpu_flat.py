"""Flat particle arrays on the GPU (pica's EnsembleOrdered / EnsembleUnordered):
pica_order_by_position and pica_push_flat against the oracle, which the CPU tests
pin to pica's own classes.

* order: exactly the oracle's stable lexicographic order, for sizes around the sort
  tile (4096), with ties, negative values and -0.0 / +0.0, over 1, 2 or 3 coordinates.
* push: positions and momenta bit for bit (the per-particle arithmetic is pica's,
  compiled without contraction); J within 1e-12 of its largest value (FP64 global
  atomics add in an order that varies from run to run); CIC and TSC; pica grids with
  2 and 3 guard layers; two species.
* FlatEnsemble: a few steps (push and Yee updates) equal the oracle's pushes with the
  fields the product's own Yee update gives, and reorder() sorts the array by position.
"""
import numpy as np
import pytest
import torch

import pica_gb300 as pg
from oracle import pic_oracle as po
from tests.helpers import rel_err
from tests.test_flat_cpu import SPECIES, flat_inputs

pytestmark = pytest.mark.gpu


def cuda(a, dtype=torch.float64):
    return torch.as_tensor(np.ascontiguousarray(a)).to(device="cuda", dtype=dtype)


@pytest.mark.parametrize("n", [0, 1, 4095, 4096, 4097, 100003])
@pytest.mark.parametrize("dims", [1, 2, 3])
def test_order_by_position_equals_oracle(n, dims):
    rng = np.random.default_rng(n + dims)
    k = [np.round(rng.uniform(-3, 3, n), 2) for _ in range(3)]
    if n > 40:
        k[0][:20] = -0.0
        k[0][20:40] = 0.0
        k[1][:40] = 1e-300
    got = pg.order_by_position(*[cuda(a) for a in k[:dims]]).cpu().numpy()
    want = po.order_by_position(*k[:dims])
    assert np.array_equal(got, want)


@pytest.mark.parametrize("shape", [pg.SHAPE_CIC, pg.SHAPE_TSC])
@pytest.mark.parametrize("guard", [2, 3])
def test_push_flat_equals_oracle(shape, guard):
    n = (8, 6, 12)
    h, dt, p, f6 = flat_inputs(n, 20000, 7)
    s = pg.Simulation(n, h, dt, supercell=(1, 1, 1), form=pg.FORM_FP64_PLAIN, shape=shape, species=SPECIES)
    s.upload_fields(f6 + [np.zeros(n)] * 3)
    t = {k: cuda(p[k]) for k in ("x", "y", "z", "ux", "uy", "uz", "w")}
    sp = cuda(p["species"], torch.int32)
    s.push_flat(t["x"], t["y"], t["z"], t["ux"], t["uy"], t["uz"], t["w"], sp, guard=guard)
    want, j = po.push_flat(n, h, dt, p, f6, shape=shape, species=SPECIES, guard=guard)
    for k in ("x", "y", "z", "ux", "uy", "uz"):
        assert np.array_equal(t[k].cpu().numpy(), want[k]), k
    f = s.fields()
    for c in range(3):
        assert rel_err(f[6 + c], j[c]) < 1e-12, c
    for c in range(6):
        assert np.array_equal(f[c], f6[c]), c
    s.close()


def test_push_flat_rejects_what_it_does_not_build():
    n = (4, 4, 4)
    h, dt, p, _ = flat_inputs(n, 10, 1)
    t = [cuda(p[k]) for k in ("x", "y", "z", "ux", "uy", "uz", "w")]
    s32 = pg.Simulation(n, h, dt, supercell=(2, 2, 2), form=pg.FORM_FP32_CELL, shape=pg.SHAPE_TSC,
                        deposit=pg.DEPOSIT_ESIRKEPOV)
    with pytest.raises(pg.PicaError):
        s32.push_flat(*t)
    s = pg.Simulation(n, h, dt, supercell=(2, 2, 2), form=pg.FORM_FP64_PLAIN, species=SPECIES[:1])
    with pytest.raises(pg.PicaError):
        s.push_flat(*t, cuda(np.full(10, 1, np.int32), torch.int32))   # species 1 of a 1-species table
    s.push_flat(*t)   # the context stays usable
    s32.close()
    s.close()


def test_flat_ensemble_steps_and_reorder():
    n = (8, 8, 8)
    h, dt, p, f6 = flat_inputs(n, 6000, 11)
    s = pg.Simulation(n, h, dt, supercell=(1, 1, 1), form=pg.FORM_FP64_PLAIN, species=SPECIES)
    s.upload_fields(f6 + [np.zeros(n)] * 3)
    e = pg.FlatEnsemble(s)
    e.add(*[p[k] for k in ("x", "y", "z", "ux", "uy", "uz", "w")], p["species"])
    assert e.size() == 6000
    ref = {k: p[k].copy() for k in p}
    for _ in range(3):
        f = s.fields()
        ref, _ = po.push_flat(n, h, dt, ref, f[:6], species=SPECIES)
        e.step(1)
    got = e.particles()
    for k in ("x", "y", "z", "ux", "uy", "uz"):
        assert np.array_equal(got[k], ref[k]), k
    order = e.reorder().cpu().numpy()
    assert np.array_equal(order, po.order_by_position(got["x"], got["y"], got["z"]))
    after = e.particles()
    for k in ("x", "y", "z", "ux", "w"):
        assert np.array_equal(after[k], got[k][order]), k
    assert np.array_equal(after["species"], got["species"][order])
    s.close()
