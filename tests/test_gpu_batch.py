"""Batching form (pica_batch_*): members advanced together equal the same plasmas
stepped one by one with pica_step, bit for bit (the same push code per
supercell, exact integer current sums), with and without the captured graph."""
import numpy as np
import pytest

import pica_gb300 as pg

from helpers import ME, E, particle_args, thermal_inputs

pytestmark = pytest.mark.gpu

ION = (100.0 * ME, -E)


def member_cases(shape):
    """Uneven members: grid, particles per cell, species, resort cadence, slack."""
    return [
        dict(n=(8, 8, 8), ppc=6, seed=31, sigma=0.2, species=((ME, E),), resort_every=2, slack=0.15),
        dict(n=(12, 8, 16), ppc=3, seed=32, sigma=0.1, species=((ME, E),), resort_every=0, slack=1e-9),
        dict(n=(16, 16, 8), ppc=4, seed=33, sigma=0.3, species=((ME, E), ION), resort_every=3, slack=0.15),
    ]


def inputs_of(case):
    d = thermal_inputs(case["n"], case["ppc"], seed=case["seed"], u_sigma=case["sigma"],
                       nspecies=len(case["species"]))
    rng = np.random.default_rng(case["seed"] + 100)
    fields = [2e3 * rng.standard_normal(case["n"]) for _ in range(6)] + [np.zeros(case["n"])] * 3
    return d, fields


def sim_kwargs(case, d, shape):
    return dict(n=case["n"], h=d["h"], dt=d["dt"], supercell=(4, 4, 4), form=pg.FORM_FP32_CELL, shape=shape,
                deposit=pg.DEPOSIT_ESIRKEPOV, species=case["species"], slack=case["slack"],
                resort_every=case["resort_every"])


def run_alone(case, shape, steps):
    d, fields = inputs_of(case)
    s = pg.Simulation(**sim_kwargs(case, d, shape))
    s.upload_particles(*particle_args(d))
    s.upload_fields(fields)
    s.step(steps)
    out = (s.particles(), s.fields(), s.counts())
    s.close()
    return out


def run_batch(cases, shape, steps, use_graph):
    kws, data = [], []
    for c in cases:
        d, fields = inputs_of(c)
        kws.append(sim_kwargs(c, d, shape))
        data.append((d, fields))
    b = pg.Batch(kws)
    b.set_options(use_graph=use_graph)
    for m, (d, fields) in zip(b.members, data):
        m.upload_particles(*particle_args(d))
        m.upload_fields(fields)
    b.step(steps)
    out = [(m.particles(), m.fields(), m.counts()) for m in b.members]
    stats = b.stats()
    b.close()
    return out, stats


@pytest.mark.parametrize("use_graph", [True, False])
@pytest.mark.parametrize("shape", [pg.SHAPE_CIC, pg.SHAPE_TSC])
def test_batch_members_equal_standalone_runs(shape, use_graph):
    cases = member_cases(shape)
    steps = 6
    got, stats = run_batch(cases, shape, steps, use_graph)
    for case, (p, f, c) in zip(cases, got):
        pa, fa, ca = run_alone(case, shape, steps)
        assert np.array_equal(c, ca)
        for k in ("x", "y", "z", "ux", "uy", "uz", "w", "species", "supercell"):
            assert np.array_equal(p[k], pa[k]), k
        for comp in range(9):
            assert np.array_equal(f[comp], fa[comp]), comp
    assert stats["steps"] == steps
    if use_graph:
        assert stats["graph_launches"] == steps
        assert 1 <= stats["captures"] <= steps
    else:
        assert stats["graph_launches"] == 0 and stats["captures"] == 0
    assert stats["kernel_launches"] >= steps * (1 + 7 * len(cases))


def test_batch_rejects_mixed_forms():
    d = thermal_inputs((8, 8, 8), 2, seed=1)
    ok = dict(n=(8, 8, 8), h=d["h"], dt=d["dt"], supercell=(4, 4, 4))
    with pytest.raises(pg.PicaError):
        pg.Batch([ok, dict(ok, form=pg.FORM_FP64_PLAIN)])
    with pytest.raises(pg.PicaError):
        pg.Batch([ok, dict(ok, supercell=(2, 2, 2))])


def test_batch_config_tuner_picks_a_measured_combination():
    """autotune.tune_batch_config on a small sample: every (supercell edge, cadence)
    combination is built and timed, the choice is the fastest of them, and a batch
    built with the choice steps."""
    from pica_gb300 import autotune, workloads

    def make(sc, every):
        ms = workloads.batched_members(count=3, half=True, resort_every=every, supercell=sc)
        b = pg.Batch([m["sim"] for m in ms])
        for sim, wl in zip(b.members, ms):
            sim.generate_plasma(wl["specs"])
            sim.upload_fields([np.zeros(wl["sim"]["n"])] * 9)
        return b

    best = autotune.tune_batch_config(make, supercells=((4, 4, 4), (2, 2, 2)), cadences=(2, 4), steps=2)
    assert set(best["tried"]) == {"4x4x4/every2", "4x4x4/every4", "2x2x2/every2", "2x2x2/every4"}
    assert best["s_per_step"] == min(best["tried"].values())
    b = make(tuple(best["supercell"]), best["resort_every"])
    n0 = b.num_particles()
    b.set_options(use_graph=True, variant=best["variant"])
    b.step(3)
    assert b.num_particles() == n0
    b.close()
