"""Flat particle arrays in the oracle (pica's EnsembleOrdered / EnsembleUnordered),
pinned to pica's own classes through the harness over its headers.

* orc_order_by_position against EnsembleOrdered::reorder (EnsembleOrdered.h:61-71)
  on positions without ties (std::sort's order is then unique) and against a
  stable numpy lexsort with ties (pica leaves the order of ties unspecified).
* orc_push_flat against pica's FieldInterpolatorCIC<YeeGrid<Three,double>>,
  BorisPusher and CurrentDepositorCIC<YeeGrid<Three,double>> over an
  EnsembleUnordered: positions and momenta bit for bit; J within 1e-12 of its
  largest value (pica adds the guard layers' current onto the domain afterwards,
  the restatement adds it there directly, so sums group differently).
"""
import numpy as np
import pytest

from oracle import pic_oracle as po
from tests.helpers import C, E, ME, rel_err

REF = po.reference_available()
SPECIES = ((ME, E), (100 * ME, -E))


def flat_inputs(n, m, seed, h=0.05, u_sigma=0.1, fields=1e2):
    rng = np.random.default_rng(seed)
    L = [n[d] * h for d in range(3)]
    p = {"x": rng.uniform(0, L[0], m), "y": rng.uniform(0, L[1], m), "z": rng.uniform(0, L[2], m),
         "ux": rng.normal(0, u_sigma, m), "uy": rng.normal(0, u_sigma, m), "uz": rng.normal(0, u_sigma, m),
         "w": rng.uniform(1e2, 1e3, m), "species": (rng.integers(0, 2, m)).astype(np.int32)}
    # particles on cell faces and on the domain faces
    p["x"][:8] = np.arange(8) % n[0] * h
    p["y"][8:12] = 0.0
    f6 = [rng.normal(0, fields, n) for _ in range(6)]
    return (h, h, h), 0.5 * h / (C * np.sqrt(3.0)), p, f6


@pytest.mark.skipif(not REF, reason="pica sources not mounted")
@pytest.mark.parametrize("n", [0, 1, 7, 1000])
def test_order_matches_pica_ensemble_ordered(n):
    rng = np.random.default_rng(n)
    x, y, z = (rng.uniform(-1, 1, n) for _ in range(3))
    a = po.order_by_position(x, y, z)
    assert np.array_equal(a, po.order_by_position(x, y, z, kind="reference"))
    assert np.array_equal(a, np.lexsort((z, y, x)))


@pytest.mark.parametrize("dims", [1, 2, 3])
def test_order_is_stable_lexicographic_with_ties(dims):
    rng = np.random.default_rng(dims)
    m = 5000
    k = [np.round(rng.uniform(-2, 2, m), 1) for _ in range(3)]
    k[0][:10] = -0.0
    k[0][10:20] = 0.0
    a = po.order_by_position(*k[:dims])
    assert np.array_equal(a, np.lexsort(tuple(reversed(k[:dims]))))


@pytest.mark.skipif(not REF, reason="pica sources not mounted")
@pytest.mark.parametrize("n,m,seed", [((8, 6, 10), 3000, 1), ((4, 4, 4), 500, 2), ((12, 1, 1), 200, 3)])
def test_flat_push_matches_pica_grid_level_classes(n, m, seed):
    h, dt, p, f6 = flat_inputs(n, m, seed)
    a, ja = po.push_flat(n, h, dt, p, f6, species=SPECIES)
    b, jb = po.push_flat(n, h, dt, p, f6, species=SPECIES, kind="reference")
    for k in ("x", "y", "z", "ux", "uy", "uz"):
        assert np.array_equal(a[k], b[k]), k
    for c in range(3):
        assert rel_err(ja[c], jb[c]) < 1e-12, c
    assert np.any(a["ux"] != p["ux"])


def test_flat_push_conserves_the_array_and_wraps():
    n = (8, 8, 8)
    h, dt, p, f6 = flat_inputs(n, 2000, 4, u_sigma=0.5)
    a, j = po.push_flat(n, h, dt, p, f6, species=SPECIES, shape=po.SHAPE_TSC)
    L = n[0] * h[0]
    for k in ("x", "y", "z"):
        assert np.all((a[k] >= 0) & (a[k] < L))
    # total current = sum of q w v / V over particles (both shapes' weights sum to 1)
    u = np.stack([a["ux"], a["uy"], a["uz"]])
    ig = 1.0 / np.sqrt(1.0 + (u * u).sum(0))
    q = np.array([s[1] for s in SPECIES])[a["species"]]
    want = (u * C * ig * (q * a["w"])).sum(1) / (h[0] * h[1] * h[2])
    for c in range(3):
        assert abs(j[c].sum() - want[c]) <= 1e-10 * np.abs(u[c] * C * ig * q * a["w"]).sum() / h[0] ** 3
