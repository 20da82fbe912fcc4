"""Shared helpers for the parity tests: comparisons, fixture loading, runners."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

C = 29979245800.0
E = -4.80320427e-10
ME = 9.10938215e-28
PI = 3.14159265358


def rel_err(a, b):
    """Norm-wise relative error max |a - b| / max |b| (the infinity-norm relative
    error of the whole array; 0 when both are zero).  This is the metric of every
    "relative" tolerance in these tests unless a test says otherwise: a field or
    momentum component has values that cross zero, where an element-wise ratio
    measures cancellation rather than the error of the step."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.max(np.abs(b)) if b.size else 0.0
    num = np.max(np.abs(a - b)) if b.size else 0.0
    return 0.0 if num == 0.0 else num / max(den, 1e-300)


def elem_err(a, b, floor=1e-3):
    """Element-wise relative error max |a - b| / max(|b|, floor max |b|): each
    element against its own magnitude, with an absolute floor at `floor` of the
    array's largest magnitude for elements near zero."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if not b.size:
        return 0.0
    den = np.maximum(np.abs(b), floor * np.max(np.abs(b)))
    num = np.abs(a - b)
    return float(np.max(np.where(num == 0.0, 0.0, num / np.maximum(den, 1e-300))))


def periodic_err(a, b, L):
    """max periodic distance / L."""
    d = np.abs(np.asarray(a) - np.asarray(b))
    d = np.minimum(d, L - d)
    return float(np.max(d) / L) if d.size else 0.0


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def species_of(g):
    return tuple(zip(g["mass"].tolist(), g["charge"].tolist()))


def thermal_inputs(n, ppc, seed, u_sigma=0.05, hscale=(1.0, 1.0, 1.0), nspecies=1, drift=None):
    """Seeded small plasma for CPU-vs-GPU parity cases."""
    rng = np.random.default_rng(seed)
    n0 = 1e18
    wp = np.sqrt(4 * PI * n0 * E * E / ME)
    h0 = 0.05 * C / wp
    hh = tuple(h0 * s for s in hscale)
    dt = 0.5 / (C * np.sqrt(sum(1.0 / v ** 2 for v in hh)))
    idx = np.indices(n).reshape(3, -1).T
    cells = np.repeat(idx, ppc, axis=0)
    pos = (cells + rng.random(cells.shape)) * np.array(hh)
    u = rng.normal(0.0, u_sigma, cells.shape)
    if drift is not None:
        u += np.asarray(drift)
    w = np.full(len(pos), n0 * np.prod(hh) / ppc) * (1.0 + 0.1 * rng.random(len(pos)))
    sp = rng.integers(0, nspecies, len(pos)).astype(np.int32)
    return dict(h=hh, dt=dt, x=pos[:, 0], y=pos[:, 1], z=pos[:, 2], ux=u[:, 0], uy=u[:, 1], uz=u[:, 2], w=w,
                species=sp)


def particle_args(d):
    return [d[k] for k in ("x", "y", "z", "ux", "uy", "uz", "w")] + [d["species"]]


def run_1d_golden(make_sim, g, sc=(4, 1, 1)):
    """Run the pica_1d_cic_direct fixture (pica's YeeGrid<One> path) on a grid one cell
    thick along y and z; make_sim(n3, sc, h3, dt) returns an object with load-style
    (upload, set_fields, step, fields, particles) callables.  Returns (fields, particles
    sorted by x, the fixture's outputs sorted by x)."""
    n, h = int(g["n"]), float(g["h"])
    np_ = len(g["in_x"])
    yz = np.full(np_, 0.5 * h)
    load, set_fields, step, fields, particles = make_sim((n, 1, 1), sc, (h, h, h), float(g["dt"]))
    load(g["in_x"], yz, yz, g["in_ux"], g["in_uy"], g["in_uz"], g["in_w"], np.zeros(np_, np.int32))
    set_fields([a.reshape(n, 1, 1) for a in g["in_fields"][:6]] + [np.zeros((n, 1, 1))] * 3)
    step(int(g["steps"]))
    f = [a.reshape(-1) for a in fields()]
    p = particles()
    order = np.argsort(p["x"])
    ref_order = np.argsort(g["out_x"])
    got = {k: p[k][order] for k in ("x", "ux", "uy", "uz")}
    ref = {k: g["out_" + k][ref_order] for k in ("x", "ux", "uy", "uz")}
    return f, got, ref


def _splitmix(z):
    """SplitMix64 output function (S. Vigna) on uint64 arrays (modular, exact)."""
    with np.errstate(over="ignore"):
        z = z + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


CONFIG1_SEED = 20261203


def config1_plasma():
    """The plain FP64 electron plasma at its own size: 32^3 cells (h = the Debye length of
    n0 = 1e18 cm^-3 at u_th = 0.05), 50 electrons per cell uniformly random in the cell,
    momenta Maxwellian with sigma 0.05 (u = p / (m c)), dt = 0.5 Courant.  Drawn with
    integer hashing and exact sums so that every machine gets the same bits: offsets
    are 53-bit uniforms, each momentum component is the Irwin-Hall sum of twelve 32-bit
    uniforms minus 6 (variance 1, support +-6) times sigma.  Returns (sim keyword
    arguments, particle arrays in cell order)."""
    n, ppc, sigma = (32, 32, 32), 50, 0.05
    n0 = 1e18
    wp = np.sqrt(4 * PI * n0 * E * E / ME)
    h = 0.05 * C / wp
    dt = 0.5 * h / (C * np.sqrt(3.0))
    cells = np.repeat(np.arange(np.prod(n), dtype=np.uint64), ppc)
    part = np.tile(np.arange(ppc, dtype=np.uint64), int(np.prod(n)))
    base = _splitmix(np.uint64(CONFIG1_SEED)) ^ (cells << np.uint64(24)) ^ (part << np.uint64(8))
    ijk = np.stack(np.unravel_index(cells.astype(np.int64), n), axis=1).astype(np.float64)
    pos = np.empty((len(cells), 3))
    for d in range(3):
        u = (_splitmix(base ^ np.uint64(d)) >> np.uint64(11)).astype(np.float64) * 2.0 ** -53
        pos[:, d] = (ijk[:, d] + u) * h
    mom = np.empty((len(cells), 3))
    for d in range(3):
        s = np.zeros(len(cells))
        for k in range(12):
            s += (_splitmix(base ^ np.uint64(16 + 12 * d + k)) >> np.uint64(32)).astype(np.float64) * 2.0 ** -32
        mom[:, d] = sigma * (s - 6.0)
    w = np.full(len(cells), n0 * h ** 3 / ppc)
    sim = dict(n=n, h=(h, h, h), dt=dt, supercell=(2, 2, 2))
    parts = dict(x=pos[:, 0], y=pos[:, 1], z=pos[:, 2], ux=mom[:, 0], uy=mom[:, 1], uz=mom[:, 2], w=w,
                 species=np.zeros(len(cells), np.int32))
    return sim, parts


def run_checksums(step, counts, migrations, steps):
    """Per-step checksums of a run: step(1) advances it, counts() and migrations() read
    it.  Returns (number of moves per step, sum over supercells of count * (s + 1) per
    step, sum over moves of src * 7 + slot * 3 + dst per step), all int64."""
    nm, cs, ms = [], [], []
    for _ in range(steps):
        step()
        c = np.asarray(counts(), np.int64).reshape(-1)
        m = np.asarray(migrations(), np.int64).reshape(-1, 4)
        nm.append(len(m))
        cs.append(int(np.sum(c * (np.arange(len(c)) + 1))))
        ms.append(int(np.sum(m[:, 1] * 7 + m[:, 2] * 3 + m[:, 3])) if len(m) else 0)
    return np.array(nm, np.int64), np.array(cs, np.int64), np.array(ms, np.int64)
