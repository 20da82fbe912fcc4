"""The FP32 workloads at their own sizes against the oracle, from the same plasma.

The headline plasma (128^3 cells x 100 electrons per cell, 2.1e8 particles, TSC,
Esirkepov, supercell 4^3, resort every 2 steps) runs 3 steps on the GPU and in the
oracle restatement on all host cores; the two-stream plasma on a 128x128x64 block
(1.05e8 particles, CIC, resort every 4) runs 5 steps, and the Weibel plasma on a
64^3 block with both species (3.4e7 electrons and ions, TSC, resort every step)
runs 3 steps.  Each covers at least one resort.

Checked, after every step: the per-supercell counts of every species and the
migration list (species, source supercell, source slot, destination supercell)
exactly equal.  At the end: the supercell and species of every particle exactly
equal (so the ensemble order is the same); positions within 1e-6 of the box edge;
momenta and all nine fields within 1e-4 norm-wise relative error (max |a - b| /
max |b|).  The two sides differ only in FP32 rounding: the GPU contracts a*b + c
into fused multiply-adds, takes 1/sqrt from the hardware and sums currents in
exact fixed point, the oracle rounds every operation and sums currents in FP32.

One rounding difference is allowed to move a particle, not to change it: an
offset that rounds to the cell face (1.0) on one side and just below it on the
other (a tie) puts the particle in neighbouring cells.  Measured on the two-stream
block (1.05e8 particles): one such particle in its fifth step, x = 99.99999994
cells on the GPU and 100.0 in the oracle, which is also a supercell face.  So:
  * counts and migration lists are compared exactly until a step where the counts
    differ; a difference must be a tie: supercells that differ come in pairs of
    +1 / -1, at most TIES of them over the run;
  * after the first tie, the migration lists are compared as the number of moves
    per (species, source, destination), with the same budget;
  * particles are compared slot by slot; where a supercell's slots disagree (a tie
    particle, or the slots a later resort shifted around it), its particles and
    those of the supercells around it are matched one to one by nearest neighbour in
    (position, momentum) instead, every match within the tolerances above.
"""
import os

import numpy as np
import pytest

import pica_gb300 as pg
from oracle import pic_oracle as po
from pica_gb300 import workloads
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu

CASES = {
    "thermal_128": (lambda: workloads.config2(), 2, 3),
    "two_stream_128x128x64": (lambda: workloads.two_stream(n=(128, 128, 64)), 4, 5),
    "weibel_64": (lambda: workloads.weibel(n=(64, 64, 64)), 1, 3),
}


def host_plasma(specs):
    parts = [pg.generate_plasma(s) for s in specs]
    return [np.concatenate([p[k] for p in parts]) for k in ("x", "y", "z", "ux", "uy", "uz", "w", "species")]


TOL_X, TOL_U = 1e-6, 1e-4
TIES = 8   # face ties allowed over a run (measured: 0 or 1)


def compare_ensembles(ps, pr, L, nsc3):
    """Slot by slot within each (species, supercell); the supercells whose particles
    disagree (a different count after a tie, or slots shifted around a tie particle)
    are matched one to one by nearest neighbour instead, together with their
    neighbours (see the module docstring).  Returns the number of such supercells."""
    comps = ("x", "y", "z", "ux", "uy", "uz")
    umax = [max(np.max(np.abs(pr[k])), 1e-300) for k in ("ux", "uy", "uz")]
    nsc = int(np.prod(nsc3))
    nsp = int(max(ps["species"].max(initial=0), pr["species"].max(initial=0))) + 1
    ks = ps["species"].astype(np.int64) * nsc + ps["supercell"]
    kr = pr["species"].astype(np.int64) * nsc + pr["supercell"]
    cs, cr = np.bincount(ks, minlength=nsp * nsc), np.bincount(kr, minlength=nsp * nsc)
    ss, sr = np.cumsum(cs) - cs, np.cumsum(cr) - cr
    ir = np.nonzero(cs[kr] == cr[kr])[0]            # particles of supercells with equal counts
    ia = ss[kr[ir]] + (ir - sr[kr[ir]])             # the same slot on the other side
    bad = np.zeros(len(ir), bool)
    for d, k in enumerate(("x", "y", "z")):
        dd = np.abs(ps[k][ia] - pr[k][ir])
        bad |= np.minimum(dd, L[d] - dd) >= TOL_X * L[d]
    for k, m in zip(("ux", "uy", "uz"), umax):
        bad |= np.abs(ps[k][ia] - pr[k][ir]) >= TOL_U * m
    groups = np.union1d(np.nonzero(cs != cr)[0], kr[ir[bad]])
    if len(groups) == 0:
        return 0
    assert len(groups) <= max(8, 1e-3 * nsc), f"{len(groups)} supercells disagree slot by slot"
    # the disagreeing supercells and their 26 neighbours (a tie particle sits across a face)
    sx, sy, sz = np.unravel_index(groups % nsc, nsc3)
    near = set()
    for dx in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dz in (-1, 0, 1):
                near.update(np.ravel_multi_index(((sx + dx) % nsc3[0], (sy + dy) % nsc3[1], (sz + dz) % nsc3[2]),
                                                 nsc3).tolist())
    near = np.array(sorted(near))
    from scipy.spatial import cKDTree
    scale = np.array([TOL_X * L[0], TOL_X * L[1], TOL_X * L[2]] + [TOL_U * m for m in umax])
    # In tolerance units (every component of a match below 1); positions periodic
    # (a tie at a domain face puts the particle at L - eps on one side, 0 on the other).
    box = np.array([1.0 / TOL_X] * 3 + [1e12] * 3)
    shift = np.array([0.0] * 3 + [0.5e12] * 3)
    for q in range(nsp):
        ja = np.nonzero(np.isin(ps["supercell"], near) & (ps["species"] == q))[0]
        jb = np.nonzero(np.isin(pr["supercell"], near) & (pr["species"] == q))[0]
        assert len(ja) == len(jb), "the particles around the disagreeing supercells differ in number"
        a = np.mod(np.stack([ps[k][ja] for k in comps], axis=1) / scale + shift, box)
        b = np.mod(np.stack([pr[k][jb] for k in comps], axis=1) / scale + shift, box)
        dist, j = cKDTree(b, boxsize=box).query(a, p=np.inf)
        assert np.all(dist < 1.0), "a particle has no counterpart within the tolerances"
        assert len(np.unique(j)) == len(ja), "the nearest-neighbour match is not one to one"
    return len(groups)


def move_counts(m):
    """Number of moves per (species, source, destination)."""
    if len(m) == 0:
        return {}
    keys, n = np.unique(m[:, [0, 1, 3]], axis=0, return_counts=True)
    return {tuple(k): int(c) for k, c in zip(keys.tolist(), n.tolist())}


def cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


@pytest.mark.parametrize("name", list(CASES))
def test_workload_at_its_own_size_matches_oracle(name):
    make, resort, steps = CASES[name]
    wl = make()
    sim = dict(wl["sim"], resort_every=resort)
    species = sim.get("species", (pg.ELECTRON,))
    args = host_plasma(wl["specs"])
    s = pg.Simulation(**sim)
    s.upload_particles(*args)
    o = po.Oracle(sim["n"], sim["supercell"], sim["h"], sim["dt"], form=sim["form"], shape=sim["shape"],
                  deposit=sim["deposit"], species=species, threads=cores(), resort_every=resort)
    o.load(*args)
    del args
    zeros = [np.zeros(sim["n"])] * 9
    s.upload_fields(zeros)
    o.set_fields(zeros)
    assert np.array_equal(s.counts(), o.counts())
    s.record_migrations(True)
    moved, ties = 0, 0
    for st in range(steps):
        s.step(1)
        o.step(1)
        cs, co = s.counts(), o.counts()
        m, mo = s.migrations(), o.migrations()
        moved += len(m)
        if ties == 0 and np.array_equal(cs, co):
            assert np.array_equal(m, mo), f"migration lists differ after step {st + 1}"
            continue
        d = (cs - co).reshape(-1)
        nd = int(np.count_nonzero(d))
        ties += nd // 2
        assert np.all(np.abs(d) <= 1) and int(d.sum()) == 0 and nd % 2 == 0, f"counts differ after step {st + 1}"
        assert ties <= TIES, f"{ties} ties by step {st + 1}"
        ma, mb = move_counts(m), move_counts(mo)
        off = sum(abs(ma.get(k, 0) - mb.get(k, 0)) for k in set(ma) | set(mb))
        assert off <= 2 * TIES, f"moves differ by {off} after step {st + 1}"
    assert moved > 0
    s.record_migrations(False)
    ps, pr = s.particles(), o.particles()
    L = [sim["n"][d] * sim["h"][d] for d in range(3)]
    nsc3 = tuple(sim["n"][d] // sim["supercell"][d] for d in range(3))
    compare_ensembles(ps, pr, L, nsc3)
    del ps, pr
    fs, fo = s.fields(), o.get_fields()
    for c in range(9):
        assert rel_err(fs[c], fo[c]) < 1e-4, c
    s.close()
