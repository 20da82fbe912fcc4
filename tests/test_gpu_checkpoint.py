"""Checkpoints (pica_checkpoint_save / _load) and the Driver host loop (GPU).

A context loaded from a checkpoint continues like the original: the checkpoint
holds the slot layout and particle buffers as they are, the step counter (which
drives the resort cadence) and the fixed-point scale.  FP32 form: bit for bit
(exact integer current sums).  FP64 form: the current is summed with FP64
atomics, whose order differs from run to run, so two runs agree to 1e-12 (the
ensemble order and counts exactly)."""
import numpy as np
import pytest

import pica_gb300 as pg

from helpers import particle_args, rel_err, thermal_inputs

pytestmark = pytest.mark.gpu

CASES = [
    dict(form=pg.FORM_FP64_PLAIN, shape=pg.SHAPE_CIC, deposit=pg.DEPOSIT_DIRECT, supercell=(2, 2, 2), resort_every=2),
    dict(form=pg.FORM_FP32_CELL, shape=pg.SHAPE_TSC, deposit=pg.DEPOSIT_ESIRKEPOV, supercell=(4, 4, 4), resort_every=3),
]


def make(case, d, n):
    s = pg.Simulation(n, d["h"], d["dt"], **case)
    return s


def state(s):
    return s.particles(), s.fields(), s.counts(), s.step_count()


def assert_same(a, b, exact=True):
    pa, fa, ca, na = a
    pb, fb, cb, nb = b
    assert na == nb
    assert np.array_equal(ca, cb)
    for k in ("species", "supercell", "w"):
        assert np.array_equal(pa[k], pb[k]), k
    for k in ("x", "y", "z", "ux", "uy", "uz"):
        assert np.array_equal(pa[k], pb[k]) if exact else rel_err(pa[k], pb[k]) < 1e-12, k
    for c in range(9):
        assert np.array_equal(fa[c], fb[c]) if exact else rel_err(fa[c], fb[c]) < 1e-12, c


@pytest.mark.parametrize("case", CASES)
def test_checkpoint_continues_bit_for_bit(case, tmp_path):
    n = (8, 8, 8)
    d = thermal_inputs(n, 6, seed=51, u_sigma=0.2)
    a = make(case, d, n)
    a.upload_particles(*particle_args(d))
    rng = np.random.default_rng(52)
    a.upload_fields([1e3 * rng.standard_normal(n) for _ in range(6)] + [np.zeros(n)] * 3)
    a.step(4)
    path = tmp_path / "state.ckpt"
    a.save_checkpoint(path)
    a.step(5)
    b = make(case, d, n)
    b.load_checkpoint(path)
    assert b.step_count() == 4
    b.step(5)
    assert_same(state(a), state(b), exact=case["form"] == pg.FORM_FP32_CELL)


def test_checkpoint_rejects_other_configuration(tmp_path):
    n = (8, 8, 8)
    d = thermal_inputs(n, 2, seed=53)
    a = make(CASES[0], d, n)
    a.upload_particles(*particle_args(d))
    path = tmp_path / "a.ckpt"
    a.save_checkpoint(path)
    b = make(dict(CASES[0], resort_every=5), d, n)
    with pytest.raises(pg.PicaError):
        b.load_checkpoint(path)
    with pytest.raises(pg.PicaError):
        b.load_checkpoint(tmp_path / "missing.ckpt")


def test_driver_diagnostics_and_checkpoint_cadence(tmp_path):
    n = (8, 8, 8)
    d = thermal_inputs(n, 6, seed=54, u_sigma=0.1)
    case = CASES[1]
    s = make(case, d, n)
    s.upload_particles(*particle_args(d))
    s.upload_fields([np.zeros(n)] * 9)
    seen = []
    drv = pg.Driver(s, diag_every=2, checkpoint_every=3, checkpoint_path=str(tmp_path / "ck{step}.bin"),
                    on_diag=lambda st, dd: seen.append(st))
    records = drv.run(7)
    assert [r[0] for r in records] == [0, 2, 4, 6]
    assert seen == [2, 4, 6]
    assert [p.split("ck")[-1] for p in drv.checkpoints] == ["3.bin", "6.bin"]
    assert drv.step == 7
    for _, dd in records:
        assert np.isfinite(dd["kinetic_energy"]) and dd["kinetic_energy"] > 0
    r = make(case, d, n)
    r.load_checkpoint(drv.checkpoints[-1])
    r.step(1)
    assert_same(state(s), state(r))
