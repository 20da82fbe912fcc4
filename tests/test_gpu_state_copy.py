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
