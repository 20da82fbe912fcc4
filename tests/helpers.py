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
