"""The workloads at full size, generated on the device: thermal 128^3 x 100 ppc
(2.1e8 electrons, TSC), two-stream 256x256x128 with 10-190 ppc (8.4e8
electrons, CIC), Weibel 256^3 with electrons and ions (2.1e9 particles, TSC;
about 200 GB of device memory), and the 64-plasma batch (grids 32^3-96^3,
16-128 ppc, 1.9e9 particles in all, batching form).  Too large for the oracle,
so they are checked through properties that hold at any size:

* particle number per species, exactly, after every checked step;
* charge conservation over one step: max |(rho^{n+1} - rho^n)/dt + div J| at most
  1e-6 of max |rho| / dt;
* the Gauss residual max |div E - 4 pi (rho + bg)| is carried unchanged by the step
  (charge-conserving deposit), to 1e-4;
* the total charge sum Q = sum q w, to 1e-12 of sum |q| w (electrons and ions
  cancel in Q);
* determinism: a second run of the same steps gives the same fields and counts,
  bit for bit (fixed-point current sums).
"""
import numpy as np
import pytest

import pica_gb300 as pg
from pica_gb300 import validate, workloads

pytestmark = pytest.mark.gpu

STEPS = 4
CASES = {
    "thermal_128": lambda: workloads.config2(),
    "two_stream_256x256x128": workloads.config3,
    "weibel_256": workloads.config5,
}


def expected_counts(sim, wl):
    return [sum(int(sim.lib.pica_plasma_count(s)) for s in wl["specs"] if s.species == q)
            for q in range(sim.nspecies)]


def charge_scale(sim, wl):
    """sum over particles of |q| w."""
    species = wl["sim"].get("species", (pg.ELECTRON,))
    return sum(int(sim.lib.pica_plasma_count(s)) * abs(species[s.species][1]) * s.weight for s in wl["specs"])


def run(wl, check):
    sim = pg.Simulation(**wl["sim"])
    sim.generate_plasma(wl["specs"])
    expect = expected_counts(sim, wl)
    assert sim.counts().sum(axis=1).tolist() == expect
    if check:
        d0 = sim.diagnostics(wl["bg"])
        res, _ = validate.charge_residual(sim)   # one step
        assert res <= 1e-6, res
        assert sim.counts().sum(axis=1).tolist() == expect
        sim.step(STEPS - 1)
        d1 = sim.diagnostics(wl["bg"])
        assert abs(d1["total_charge"] - d0["total_charge"]) <= 1e-12 * charge_scale(sim, wl)
        assert abs(d1["gauss_max"] - d0["gauss_max"]) <= 1e-4 * d0["gauss_max"]
    else:
        sim.step(STEPS)
    assert sim.step_count() == STEPS
    counts = sim.counts()
    assert counts.sum(axis=1).tolist() == expect
    fields = sim.fields()
    sim.close()
    return counts, fields


@pytest.mark.parametrize("name", list(CASES))
def test_full_size_workload_properties(name):
    wl = CASES[name]()
    c1, f1 = run(wl, check=True)
    c2, f2 = run(wl, check=False)
    assert np.array_equal(c1, c2)
    for c in range(9):
        assert np.array_equal(f1[c], f2[c]), c


def run_batch(members, steps):
    b = pg.Batch([m["sim"] for m in members])
    for sim, wl in zip(b.members, members):
        sim.generate_plasma(wl["specs"])
        sim.upload_fields([np.zeros(wl["sim"]["n"])] * 9)
    b.reorder()
    expect = [expected_counts(sim, wl) for sim, wl in zip(b.members, members)]
    b.step(steps)
    counts = [sim.counts() for sim in b.members]
    for c, e in zip(counts, expect):
        assert c.sum(axis=1).tolist() == e
    # Field energy and the J components of every member (a checksum per member).
    sums = [(sim.field_energy(), [float(np.sum(f)) for f in sim.fields()[6:]]) for sim in b.members]
    stats = b.stats()
    b.close()
    return counts, sums, stats


def test_full_size_batch_properties():
    """The 64-plasma batch at full member sizes: particle numbers conserved per member,
    and a second run equal to the first (counts, field energy and current sums of every
    member, bit for bit)."""
    members = workloads.batched_members(count=64)
    steps = 5
    c1, s1, st = run_batch(members, steps)
    assert st["steps"] == steps
    c2, s2, _ = run_batch(members, steps)
    for a, b in zip(c1, c2):
        assert np.array_equal(a, b)
    assert s1 == s2
