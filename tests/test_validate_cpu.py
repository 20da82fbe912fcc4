"""Host logic of the FP32-vs-FP64 comparison (pica_gb300.validate.match_particles):
two ensembles of the same plasma are matched one to one although a rounding tie put
one particle in neighbouring supercells in the two of them."""
import numpy as np

from pica_gb300 import validate


def ensemble(x, y, z, u, S=4.0, nsc=4):
    sc = ((np.floor(x / S) * nsc + np.floor(y / S)) * nsc + np.floor(z / S)).astype(np.int64)
    o = np.lexsort((x, sc))   # supercell order, then an in-supercell order of the ensemble's own
    return {"x": x[o], "y": y[o], "z": z[o], "ux": u[0][o], "uy": u[1][o], "uz": u[2][o], "supercell": sc[o],
            "species": np.zeros(len(x), np.int32)}


def test_match_through_a_supercell_face_tie():
    rng = np.random.default_rng(1)
    n = 20000
    x, y, z = (rng.uniform(0, 16, n) for _ in range(3))
    u = [rng.normal(0, 0.05, n) for _ in range(3)]
    x[5] = 8.0                         # on a supercell face in one ensemble ...
    a = ensemble(x, y, z, u)
    x2 = x.copy()
    x2[5] = 8.0 - 1e-12                # ... just below it in the other
    b = ensemble(x2, y, z, [v * (1 + 1e-7) for v in u])
    ia, ib, nn = validate.match_particles(a, b, [16.0] * 3, (4, 4, 4))
    assert len(ia) == n and len(np.unique(ia)) == n and len(np.unique(ib)) == n
    assert 0 < nn < n                  # only the two disagreeing supercells went through the tree
    assert np.allclose(a["x"][ia], b["x"][ib], atol=1e-9)
    err, nn2 = validate.rms_momentum_error(a, b, [16.0] * 3, (4, 4, 4))
    assert nn2 == nn and abs(err - 1e-7) < 1e-9


def test_match_rejects_different_particle_numbers():
    rng = np.random.default_rng(2)
    x, y, z = (rng.uniform(0, 16, 100) for _ in range(3))
    u = [rng.normal(0, 0.05, 100) for _ in range(3)]
    a = ensemble(x, y, z, u)
    b = ensemble(x[1:], y[1:], z[1:], [v[1:] for v in u])
    assert validate.match_particles(a, b, [16.0] * 3, (4, 4, 4)) is None
