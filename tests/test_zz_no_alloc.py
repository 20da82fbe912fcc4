"""pica_field_energy_noalloc against pica_field_energy, through the C ABI.

The no-allocation entry point reduces six caller-owned device arrays with its
scratch in a static device array; the context entry point reduces the
context's own fields with scratch allocated at context creation.  Both are FP64
sums of the same squares in different fixed orders.
"""
import ctypes as C

import numpy as np
import pytest

import pica_gb300 as pg
from pica_gb300._lib import load

from helpers import PI, rel_err

pytestmark = pytest.mark.gpu

PICA_ERR_LIMIT = -8


def _bind(lib):
    f = lib.pica_field_energy_noalloc
    f.restype = C.c_int
    f.argtypes = [C.POINTER(C.c_void_p), C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_double), C.c_void_p,
                  C.POINTER(C.c_double)]
    return f


def _call(fn, tensors, fp64, n, h, stream):
    ptrs = (C.c_void_p * 6)(*[t.data_ptr() for t in tensors])
    nn = (C.c_int32 * 3)(*n)
    hh = (C.c_double * 3)(*h)
    out = C.c_double(-1.0)
    rc = fn(ptrs, fp64, nn, hh, C.c_void_p(stream), C.byref(out))
    return rc, out.value


@pytest.mark.parametrize("form", [pg.FORM_FP64_PLAIN, pg.FORM_FP32_CELL])
def test_noalloc_field_energy_matches_context_entry_point(form):
    torch = pytest.importorskip("torch")
    fn = _bind(load())
    n, h = (16, 20, 24), (0.3, 0.25, 0.2)
    rng = np.random.default_rng(11)
    f9 = [rng.standard_normal(n) for _ in range(9)]
    sim = pg.Simulation(n, h, 0.01, supercell=(4, 4, 4), form=form)
    sim.upload_fields(f9)
    fp64 = 1 if form == pg.FORM_FP64_PLAIN else 0
    npdt = np.float64 if fp64 else np.float32
    dev = [torch.from_numpy(np.ascontiguousarray(f9[c], dtype=npdt)).cuda() for c in range(6)]
    stream = torch.cuda.current_stream().cuda_stream
    torch.cuda.synchronize()

    ref = sim.field_energy()
    rc1, e1 = _call(fn, dev, fp64, n, h, stream)
    rc2, e2 = _call(fn, dev, fp64, n, h, stream)
    assert rc1 == 0 and rc2 == 0
    assert e1 == e2                      # fixed reduction order: same bits on repeated calls
    assert rel_err(e1, ref) < 1e-13      # same FP64 squares, different summation order
    host = sum(np.sum(np.asarray(f, dtype=npdt).astype(np.float64) ** 2) for f in f9[:6])
    assert rel_err(e1, host * h[0] * h[1] * h[2] / (8.0 * PI)) < 1e-12
    assert sim.field_energy() == ref     # the context entry point is unchanged by the static scratch
    # After the first calls (which load the kernels), a call allocates nothing: the
    # device's free memory and the caching allocator's counters stay as they were.
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    stats0 = torch.cuda.memory_stats().get("allocation.all.allocated", 0)
    rc3, e3 = _call(fn, dev, fp64, n, h, stream)
    torch.cuda.synchronize()
    assert rc3 == 0 and e3 == e1
    assert torch.cuda.mem_get_info()[0] == free0
    assert torch.cuda.memory_stats().get("allocation.all.allocated", 0) == stats0
    sim.close()


def test_noalloc_field_energy_rejects_grids_above_limit():
    torch = pytest.importorskip("torch")
    fn = _bind(load())
    dev = [torch.zeros(8, dtype=torch.float32, device="cuda") for _ in range(6)]
    # 1024 x 512 x 512 nodes is above the 512^3 scratch limit: rejected before any launch.
    rc, out = _call(fn, dev, 0, (1024, 512, 512), (1.0, 1.0, 1.0), torch.cuda.current_stream().cuda_stream)
    assert rc == PICA_ERR_LIMIT and out == -1.0
