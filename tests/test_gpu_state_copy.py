"""Raw state copies (pica_state_slots / pica_state_copy) on the GPU.

A host loop that keeps the particle state in pinned host memory uploads it
before every step and downloads it after, on copy streams of its own, with
component c of step n+1 going up once component c of step n is down (as
bench.py's end-to-end loop does).  Such a run equals the same steps without
copies bit for bit (FP32 form), across resorts that change the layout."""
import numpy as np
import pytest

import pica_gb300 as pg

from helpers import particle_args, thermal_inputs

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def make(d, n):
    s = pg.Simulation(n, d["h"], d["dt"], supercell=(4, 4, 4), form=pg.FORM_FP32_CELL, shape=pg.SHAPE_TSC,
                      deposit=pg.DEPOSIT_ESIRKEPOV, resort_every=2)
    s.upload_particles(*particle_args(d))
    rng = np.random.default_rng(72)
    s.upload_fields([1e3 * rng.standard_normal(n) for _ in range(6)] + [np.zeros(n)] * 3)
    return s


def test_state_round_trip_on_copy_streams_equals_plain_steps():
    n = (16, 8, 8)
    d = thermal_inputs(n, 6, seed=71, u_sigma=0.2)
    steps, comps = 5, 8
    ref = make(d, n)
    ref.step(steps)
    a = make(d, n)
    main = torch.cuda.current_stream()
    a.set_stream(main.cuda_stream)
    up, down = torch.cuda.Stream(), torch.cuda.Stream()
    alloc = 2 * a.state_slots(0) + 1024
    host = [torch.empty(alloc * 4, dtype=torch.uint8, pin_memory=True) for _ in range(comps)]
    for c in range(comps):
        a.state_copy(0, c, host[c].data_ptr(), False)
    torch.cuda.synchronize()
    downed = [None] * comps
    for _ in range(steps):
        assert a.state_slots(0) <= alloc
        a.set_stream(up.cuda_stream)
        upped = []
        for c in range(comps):
            if downed[c] is not None:
                up.wait_event(downed[c])
            a.state_copy(0, c, host[c].data_ptr(), True)
            ev = torch.cuda.Event()
            ev.record(up)
            upped.append(ev)
        for ev in upped:
            main.wait_event(ev)
        a.set_stream(main.cuda_stream)
        a.step(1)
        stepped = torch.cuda.Event()
        stepped.record(main)
        down.wait_event(stepped)
        a.set_stream(down.cuda_stream)
        for c in range(comps):
            a.state_copy(0, c, host[c].data_ptr(), False)
            downed[c] = torch.cuda.Event()
            downed[c].record(down)
        a.set_stream(main.cuda_stream)
    torch.cuda.synchronize()
    assert a.step_count() == steps
    assert np.array_equal(a.counts(), ref.counts())
    pa, pr = a.particles(), ref.particles()
    for k in ("x", "y", "z", "ux", "uy", "uz", "w", "species", "supercell"):
        assert np.array_equal(pa[k], pr[k]), k
    fa, fr = a.fields(), ref.fields()
    for c in range(9):
        assert np.array_equal(fa[c], fr[c]), c
    a.close()
    ref.close()


def test_packed_round_trip_on_copy_streams_equals_plain_steps():
    """The same host loop with the packed image (used slots only)."""
    n = (16, 8, 8)
    d = thermal_inputs(n, 6, seed=74, u_sigma=0.2)
    steps, comps = 5, 8
    ref = make(d, n)
    ref.step(steps)
    a = make(d, n)
    main = torch.cuda.current_stream()
    a.set_stream(main.cuda_stream)
    up, down = torch.cuda.Stream(), torch.cuda.Stream()
    packed = a.state_packed_slots(0)
    assert 0 < packed <= a.state_slots(0)
    alloc = 2 * packed + 1024
    host = [torch.empty(alloc * 4, dtype=torch.uint8, pin_memory=True) for _ in range(comps)]
    for c in range(comps):
        a.state_copy_packed(0, c, host[c].data_ptr(), False)
    torch.cuda.synchronize()
    downed = [None] * comps
    for _ in range(steps):
        a.set_stream(up.cuda_stream)
        upped = []
        for c in range(comps):
            if downed[c] is not None:
                up.wait_event(downed[c])
            a.state_copy_packed(0, c, host[c].data_ptr(), True)
            ev = torch.cuda.Event()
            ev.record(up)
            upped.append(ev)
        for ev in upped:
            main.wait_event(ev)
        a.set_stream(main.cuda_stream)
        a.step(1)
        packed = a.state_packed_slots(0)
        assert packed <= alloc
        stepped = torch.cuda.Event()
        stepped.record(main)
        down.wait_event(stepped)
        a.set_stream(down.cuda_stream)
        for c in range(comps):
            a.state_copy_packed(0, c, host[c].data_ptr(), False)
            downed[c] = torch.cuda.Event()
            downed[c].record(down)
        a.set_stream(main.cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(a.counts(), ref.counts())
    pa, pr = a.particles(), ref.particles()
    for k in ("x", "y", "z", "ux", "uy", "uz", "w", "species", "supercell"):
        assert np.array_equal(pa[k], pr[k]), k
    fa, fr = a.fields(), ref.fields()
    for c in range(9):
        assert np.array_equal(fa[c], fr[c]), c
    a.close()
    ref.close()


def test_packed_image_holds_the_ensemble_and_goes_stale_after_a_step():
    n = (8, 8, 8)
    d = thermal_inputs(n, 4, seed=75, u_sigma=0.2)
    s = make(d, n)
    s.step(3)
    m = s.state_packed_slots(0)
    cell = np.empty(m, np.uint32)
    s.state_copy_packed(0, 0, cell.ctypes.data, False)
    comp = {}
    for c, k in ((4, "ux"), (5, "uy"), (6, "uz"), (7, "w")):
        comp[k] = np.empty(m, np.float32)
        s.state_copy_packed(0, c, comp[k].ctypes.data, False)
    s.synchronize()
    p = s.particles()
    live = cell != 0xFFFFFFFF   # dead slots of the used range carry the dead-cell marker
    assert live.sum() == len(p["ux"]) == s.counts().sum()
    for k, v in comp.items():
        assert np.array_equal(v[live].astype(np.float64), p[k]), k
    s.step(1)
    with pytest.raises(pg.PicaError):
        s.state_copy_packed(0, 4, comp["ux"].ctypes.data, False)
    s.close()


@pytest.mark.parametrize("nchunks,split,edge", [(3, False, 1), (8, False, 1), (8, True, 1), (16, True, 1),
                                               (6, True, 4)])
def test_chunked_push_from_host_ranges_equals_plain_steps(nchunks, split, edge):
    """The packed image uploaded supercell range by supercell range, each range's push
    launched once its upload is in (pica_push_deposit_chunked), downloaded range by
    range: equal to plain steps bit for bit.  split: the host copies on copy streams
    of their own, apart from the gather / scatter kernels (pica_state_copy_packed_range_on).
    edge > 1: the first and last ranges cut into that many pieces, the push over those
    ranges (pica_push_deposit_ranges)."""
    n = (16, 8, 8)
    d = thermal_inputs(n, 6, seed=76, u_sigma=0.2)
    steps, comps = 5, 8
    ref = make(d, n)
    ref.step(steps)
    a = make(d, n)
    main = torch.cuda.current_stream()
    a.set_stream(main.cuda_stream)
    up, down = torch.cuda.Stream(), torch.cuda.Stream()
    upc, downc = (torch.cuda.Stream(), torch.cuda.Stream()) if split else (up, down)
    cs_up = upc.cuda_stream if split else None
    cs_down = downc.cuda_stream if split else None
    ranges = a.edge_split_ranges(nchunks, edge) if edge > 1 else a.chunk_ranges(nchunks)
    assert ranges[0][0] == 0 and ranges[-1][1] == int(np.prod(a.nsc))
    assert all(r0[1] == r1[0] for r0, r1 in zip(ranges, ranges[1:]))
    packed = a.state_packed_slots(0)
    alloc = 2 * packed + 1024
    host = [torch.empty(alloc * 4, dtype=torch.uint8, pin_memory=True) for _ in range(comps)]
    for c in range(comps):
        a.state_copy_packed(0, c, host[c].data_ptr(), False)
    torch.cuda.synchronize()
    downed = [None] * len(ranges)
    for _ in range(steps):
        a.set_stream(up.cuda_stream)
        upped = []
        for r, rg in enumerate(ranges):
            if downed[r] is not None:
                upc.wait_event(downed[r])
            for c in range(comps):
                a.state_copy_packed(0, c, host[c].data_ptr(), True, sc_range=rg, copy_stream=cs_up)
            ev = torch.cuda.Event()
            ev.record(up)
            upped.append(ev)
        a.set_stream(main.cuda_stream)
        if edge > 1:
            a.push_deposit_ranges(ranges, [ev.cuda_event for ev in upped])
        else:
            a.push_deposit_chunked([ev.cuda_event for ev in upped])
        a.update_b(0.5 * a.dt)
        a.update_e(a.dt)
        a.update_b(0.5 * a.dt)
        a.migrate()
        assert a.state_packed_slots(0) <= alloc
        stepped = torch.cuda.Event()
        stepped.record(main)
        down.wait_event(stepped)
        a.set_stream(down.cuda_stream)
        for r, rg in enumerate(ranges):
            for c in range(comps):
                a.state_copy_packed(0, c, host[c].data_ptr(), False, sc_range=rg, copy_stream=cs_down)
            downed[r] = torch.cuda.Event()
            downed[r].record(downc)
        a.set_stream(main.cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(a.counts(), ref.counts())
    pa, pr = a.particles(), ref.particles()
    for k in ("x", "y", "z", "ux", "uy", "uz", "w", "species", "supercell"):
        assert np.array_equal(pa[k], pr[k]), k
    fa, fr = a.fields(), ref.fields()
    for c in range(9):
        assert np.array_equal(fa[c], fr[c]), c
    a.close()
    ref.close()


def test_push_ranges_reject_bounds_that_do_not_cover_the_supercells():
    n = (8, 8, 8)
    d = thermal_inputs(n, 2, seed=77, u_sigma=0.1)
    s = make(d, n)
    tot = int(np.prod(s.nsc))
    for bad in ([(0, tot - 1)], [(1, tot)], [(0, 5), (5, 3), (3, tot)]):
        with pytest.raises(pg.PicaError):
            s.push_deposit_ranges(bad, [None] * len(bad))
    with pytest.raises(ValueError):
        s.push_deposit_ranges([(0, 3), (4, tot)], [None, None])
    s.step(1)   # nothing was left pending
    assert s.step_count() == 1
    s.close()
