#!/usr/bin/env python
"""Throughput of pica's particle-in-cell step on GB300.

Workload (default): the FP32 precision form of the thermal electron plasma,
128^3 cells x 100 electrons/cell (2.1e8 particles), TSC form factor,
Esirkepov deposition, supercell 4^3, seeded synthetic input generated on the
host.  One "step" = gather + Boris push + Esirkepov deposit of every particle,
the Yee update (B half step, E step, B half step) and supercell migration.

Printed (rank 0, one JSON line): particle-steps/s with device-resident state
(`value`), the same through the C ABI with the particle state copied from and
to pinned host memory every step (`e2e`), the push kernel against the HBM
roofline, the FP64 plain form of the same workload, and the oracle
restatement timed on this machine's host cores (`cpu_baseline`).

`--workload two_stream` / `--workload weibel` time the same step on the
two-stream (256x256x128, 8.4e8 electrons, CIC) and Weibel (256^3, 2.1e9
electrons and ions, TSC) plasmas instead, generated on the device; their
lines carry `value`, the push roofline and the clocks only.

`--impl reference` times the CPU implementation of the same step instead: the
oracle restatement of the headline workload at its full size on all host cores
(plasma drawn by the oracle's own generator; nothing of the pica_gb300 package
is imported), with pica's own FP64 CIC/direct arithmetic on the same plasma
beside it.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s on 1 GB300, FP32 vs FP64 form at stated error; % HBM peak"
UNIT = "particle-steps/s"
BYTES_PER_PARTICLE_FP32 = 60   # cell 4 + offsets 12 + u 12, read and written, + weight read
BYTES_PER_PARTICLE_FP64 = 104  # x 24 + u 24, read and written, + weight read
PUSH_GRID_BYTES_PER_CELL_FP32 = 36  # E/B gather 6 words + J write 3 words, FP32


def batched_measure(args, rank=0, world=1, dist=None):
    """The batching form on independent thermal plasmas of uneven size (members drawn
    as in pica_gb300.workloads.batched_members, at full size unless --batched-half),
    with the supercell edge and resort cadence tuned on a sample of them.  Timed
    with the host clock: every batch step ends with a stream synchronisation (the
    host reads each member's migration flags).  On N ranks the plasmas are binned
    over the ranks by particle count (no communication on the data path); the job's
    throughput is every rank's particles over the slowest rank's time.  Every rank
    calls this; rank 0 gets the result."""
    import torch

    import pica_gb300 as pg
    from pica_gb300 import autotune, workloads
    from pica_gb300.replicas import bin_members, job_throughput_binned
    full = not args.batched_half
    # Supercell edge and resort cadence of the whole batch, tuned on a sample (the
    # first 8 members of the draw; part of the warm-up).
    def make_sample(sc, every):
        sample = workloads.batched_members(count=min(8, args.batched), half=not full, resort_every=every,
                                           supercell=sc)
        sb = pg.Batch([m["sim"] for m in sample])
        for sim, wl in zip(sb.members, sample):
            sim.generate_plasma(wl["specs"])
            sim.upload_fields([np.zeros(wl["sim"]["n"])] * 9)
        sb.reorder()
        return sb

    cfg_tune = autotune.tune_batch_config(make_sample)
    if dist is not None:   # every rank takes rank 0's choice
        box = [cfg_tune]
        dist.broadcast_object_list(box, src=0)
        cfg_tune = box[0]
    members = workloads.batched_members(count=args.batched, half=not full, resort_every=cfg_tune["resort_every"],
                                        supercell=cfg_tune["supercell"])
    edges = [m["sim"]["n"][0] for m in members]
    nall = len(members)
    if world > 1:
        counts = [sum(pg.plasma_count(s) for s in m["specs"]) for m in members]
        mine = bin_members(counts, world)[rank]
        members = [members[i] for i in mine]
    K = args.batched_steps
    if not members:   # more ranks than plasmas: this rank only takes part in the timing
        for _ in range(2):   # the graph run and the eager run, as below
            if dist is not None:
                dist.barrier()
            job_throughput_binned(0, K, 0.0, dist, device="cuda")
        return None
    b = pg.Batch([m["sim"] for m in members])
    for sim, wl in zip(b.members, members):
        sim.generate_plasma(wl["specs"])   # drawn on the device
        sim.upload_fields([np.zeros(wl["sim"]["n"])] * 9)
    b.reorder()
    npart = b.num_particles()
    tune = autotune.tune_batch(b, steps=3)
    best = min(tune, key=tune.get)
    b.step(3)
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    s0 = b.stats()
    t = time.perf_counter()
    b.step(K)
    el = time.perf_counter() - t
    s1 = b.stats()
    value, el = job_throughput_binned(npart, K, el, dist, device="cuda")
    b.set_options(use_graph=False, variant=best)
    b.step(1)
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    t = time.perf_counter()
    b.step(K)
    el_eager = time.perf_counter() - t
    eager_value, _ = job_throughput_binned(npart, K, el_eager, dist, device="cuda")
    b.close()
    if rank != 0:
        return None
    sc = "x".join(str(v) for v in cfg_tune["supercell"])
    return {"workload": f"{nall} thermal plasmas, edges {min(edges)}-{max(edges)} cells"
                        f"{'' if full else ' (member edges halved)'}, 16-128 ppc, CIC, Esirkepov, "
                        f"supercell {sc} and resort every {cfg_tune['resort_every']} (autotuned), FP32 cell form",
            "autotune": {k: v for k, v in cfg_tune.items()},
            "ranks": world, "members_on_rank0": len(members),
            "sharding": "plasmas binned over the ranks by particle count, no communication" if world > 1 else None,
            "particles": int(round(value * el / K)), "steps": K, "value": value, "unit": UNIT,
            "ms_per_step": 1e3 * el / K,
            "timer": "host clock, each step synchronised", "graph_captures": s1["captures"] - s0["captures"],
            "kernel_launches_per_step": (s1["kernel_launches"] - s0["kernel_launches"]) / K,
            "eager_value": eager_value, "push_variant": best,
            "variant_s_per_step": {str(k): v for k, v in tune.items()}}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=12)
    ap.add_argument("--e2e-trials", type=int, default=3,
                    help="timed runs of --e2e-steps steps each; the line reports the median run (the host link's "
                         "rate varies with what else the machine does)")
    ap.add_argument("--e2e-chunks", type=int, default=16, help="supercell ranges of the e2e upload / push pipeline")
    ap.add_argument("--e2e-edge-split", type=int, default=1,
                    help="the first and last e2e ranges are cut into this many pieces (pica_push_deposit_ranges)")
    ap.add_argument("--e2e-copy-split", type=int, default=1,
                    help="each e2e push range's host copies in this many pieces (upload piece after download piece)")
    ap.add_argument("--e2e-raw", type=int, default=0,
                    help="1: e2e copies move the raw slots of each supercell range (layout slack included, one copy "
                         "per component and range, no gather / scatter kernel) instead of the packed image")
    ap.add_argument("--e2e-split", type=int, default=1,
                    help="1: e2e host copies on copy streams of their own, gather / scatter kernels on two more")
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--edge", type=int, default=None,
                    help="grid edge in cells (thermal: 128; two_stream: 256, grid edge x edge x edge/2; weibel: 256)")
    ap.add_argument("--workload", default="thermal", choices=["thermal", "two_stream", "weibel"],
                    help="thermal: 128^3 x 100 ppc (the headline); two_stream: 256x256x128, 10-190 ppc, CIC; "
                         "weibel: 256^3, electrons and ions, 2.1e9 particles (both generated on the device)")
    ap.add_argument("--resort-every", type=int, default=None,
                    help="in-supercell cell sort cadence (steps; default 2, two_stream 4)")
    ap.add_argument("--variant", type=int, default=-1, help="push-kernel launch variant (-1: autotune)")
    ap.add_argument("--batched", type=int, default=64, help="members of the batching-form run (0: skip)")
    ap.add_argument("--batched-half", action="store_true",
                    help="batching form with every member edge halved (default: the full member sizes, grids "
                         "32^3-96^3, 1.85e9 particles)")
    ap.add_argument("--batched-steps", type=int, default=10)
    ap.add_argument("--flat-steps", type=int, default=0,
                    help="pushes per order of the flat-layout leg (pica's EnsembleUnordered / EnsembleOrdered, "
                         "FP64 CIC direct) against the supercell layout (0: skip)")
    ap.add_argument("--slabs", type=int, default=0,
                    help="also step the headline plasma as this many x-slab contexts of one domain decomposition "
                         "on this GPU (halo, current fold, particle exchange; pica_gb300.domain) (0: skip)")
    ap.add_argument("--slab-steps", type=int, default=6)
    ap.add_argument("--validate-steps", type=int, default=1000,
                    help="steps of the FP32-vs-FP64 error run on a 32^3 block (0: skip)")
    return ap.parse_args()


def host_link_probe(nbytes=1 << 30, reps=3):
    """Pinned host memory <-> device bandwidth of this machine by the copy engines: one
    direction alone, and both at once on two streams (GB/s, CUDA events).  The
    ceiling of the end-to-end loop, which moves the particle state both ways."""
    import torch

    h_up = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    h_down = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    d_up = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    d_down = torch.ones(nbytes, dtype=torch.uint8, device="cuda")
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    cur = torch.cuda.current_stream()

    def timed(fn, moved):
        fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(cur)
        for _ in range(reps):
            s1.wait_stream(cur)
            s2.wait_stream(cur)
            fn()
            cur.wait_stream(s1)
            cur.wait_stream(s2)
        b.record(cur)
        torch.cuda.synchronize()
        return moved * reps / (a.elapsed_time(b) * 1e-3) / 1e9

    def up():
        with torch.cuda.stream(s1):
            d_up.copy_(h_up, non_blocking=True)

    def down():
        with torch.cuda.stream(s2):
            h_down.copy_(d_down, non_blocking=True)

    def both():
        up()
        down()

    out = {"h2d_gbs": timed(up, nbytes), "d2h_gbs": timed(down, nbytes), "both_gbs": timed(both, 2 * nbytes),
           "bytes_per_copy": nbytes, "source": "pinned host memory, copy engines, CUDA events"}
    del h_up, h_down, d_up, d_down
    return out


def measured_hbm_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        time.sleep(0.2)
        self.out = ""
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out = ""

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def make_workload(edge, form):
    import pica_gb300 as pg
    from pica_gb300 import workloads

    wl = workloads.thermal(n=(edge, edge, edge), ppc=100, supercell=(4, 4, 4), form=form, shape=pg.SHAPE_TSC,
                           deposit=pg.DEPOSIT_ESIRKEPOV, steps=1000)
    return wl


def workload_description(name, edge=None):
    """One-line description of a workload (the same for both arms of the bench)."""
    if name == "thermal":
        e = edge or 128
        return (f"thermal electron plasma {e}^3 cells x 100 ppc, FP32 cell+offset form, TSC, Esirkepov, "
                "supercell 4^3, Boris, periodic")
    e = edge or 256
    if name == "two_stream":
        return (f"two-stream {e}x{e}x{e // 2} cells, two electron beams +-0.2c along x, density "
                "1 + 0.9 cos(2 pi x / Lx) (10-190 ppc), FP32 cell+offset form, CIC, Esirkepov, supercell 4^3")
    return (f"Weibel {e}^3 cells, electrons and ions (m_i = 100 m_e), beams +-0.3c along z, 32 ppc per "
            "species per beam, FP32 cell+offset form, TSC, Esirkepov, supercell 4^3")


def bench_config(desc, npart, ncells, world):
    """The `config` object of a bench line (the same for both arms)."""
    return {"workload": f"{desc} ({npart} particles per GPU)", "particles_per_gpu": npart, "cells": ncells,
            "parallelism": f"replicas x{world}",
            "l2": "inputs larger than L2 (particle state %.1f GB)" % (npart * 32 / 1e9)}


def named_workload(name, edge=None):
    """The two-stream (256x256x128, CIC) and Weibel (256^3, TSC, two species) plasmas;
    `edge` scales the grid (a smaller case of the same plasma for profiling)."""
    from pica_gb300 import workloads

    e = edge or 256
    if name == "two_stream":
        wl = workloads.two_stream(n=(e, e, e // 2))
    else:
        wl = workloads.weibel(n=(e, e, e))
    return wl, workload_description(name, edge)


# ---------------------------------------------------------------------------
# CPU legs (the oracle only; nothing here loads the pica_gb300 library)
# ---------------------------------------------------------------------------
# pica's CGS constants (math/Constants.h:10-14) and the workloads' physical set-up,
# equal to pica_gb300.workloads (tests/test_bench_cpu.py checks that they agree):
# n0 = 1e18 cm^-3, h = 0.05 c / omega_p, dt = 0.5 h / (c sqrt 3), weight n0 h^3 / ppc.
_PI, _C, _QE, _ME, _N0 = 3.14159265358, 29979245800.0, -4.80320427e-10, 9.10938215e-28, 1e18
_SEED = 20261203


def _cell_size():
    return 0.05 * _C / math.sqrt(4.0 * _PI * _N0 * _QE ** 2 / _ME)


def oracle_workload(name, edge=None, resort_every=None):
    """The oracle's description of workload `name` ("thermal", "two_stream", "weibel";
    `edge` scales the grid): Oracle keyword arguments, the oracle generator's
    populations, the resort cadence and a short description.  FP32 cell form."""
    from oracle import pic_oracle as po

    h = _cell_size()
    hh = (h, h, h)
    dt = 0.5 * h / (_C * math.sqrt(3.0))
    beta_u = lambda b: b / math.sqrt(1.0 - b * b)   # noqa: E731
    if name == "thermal":
        e = edge or 128
        n = (e, e, e)
        specs = [po.plasma(n, hh, 100, 0.05, _N0 * h ** 3 / 100, _SEED)]
        species, shape, resort = ((_ME, _QE),), po.SHAPE_TSC, 2
        what = f"thermal {e}^3 cells x 100 ppc"
    elif name == "two_stream":
        e = edge or 256
        n = (e, e, e // 2)
        specs = [po.plasma(n, hh, 100, 0.01, _N0 * h ** 3 / 100, _SEED, density_mod=0.9, nbeams=2,
                           drift_u=beta_u(0.2), drift_axis=0)]
        species, shape, resort = ((_ME, _QE),), po.SHAPE_CIC, 4
        what = f"two-stream {e}x{e}x{e // 2} cells"
    else:
        e = edge or 256
        n = (e, e, e)
        w = _N0 * h ** 3 / 64
        u = beta_u(0.3)
        specs = [po.plasma(n, hh, 64, 0.01, w, _SEED, species=0, nbeams=2, drift_u=u, drift_axis=2),
                 po.plasma(n, hh, 64, 0.01 / math.sqrt(100.0), w, _SEED + 1, species=1, nbeams=2, drift_u=u,
                           drift_axis=2)]
        species, shape, resort = ((_ME, _QE), (_ME * 100.0, -_QE)), po.SHAPE_TSC, 1
        what = f"Weibel {e}^3 cells, electrons and ions"
    if resort_every is not None:
        resort = resort_every
    kw = dict(n=n, sc=(4, 4, 4), h=hh, dt=dt, form=po.FORM_FP32_CELL, shape=shape, deposit=po.DEPOSIT_ESIRKEPOV,
              species=species, resort_every=resort)
    return kw, specs, what


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_sample(workload="thermal", edge=None, steps=2, warmup=1, pica_path=False, resort_every=None):
    """The CPU step of a workload in the oracle, all host cores: the restatement of its
    own step (FP32 cell form, its form factor, Esirkepov), or with `pica_path` pica's own
    arithmetic on the same plasma (FP64 positions, CIC, Boris, direct deposition: the
    oracle form equal bit for bit to a harness over pica's headers).  The plasma is
    drawn by the oracle's generator.  `warmup` untimed steps, then `steps` timed ones.
    Returns (particle-steps/s, cores, sample description, timed seconds)."""
    from oracle import pic_oracle as po

    kw, specs, what = oracle_workload(workload, edge, resort_every)
    cores = host_cores()
    p = po.generate(specs, threads=cores)
    if pica_path:
        kw = dict(kw, form=po.FORM_FP64_PLAIN, shape=po.SHAPE_CIC, deposit=po.DEPOSIT_DIRECT)
    n, sc, h, dt = kw.pop("n"), kw.pop("sc"), kw.pop("h"), kw.pop("dt")
    o = po.Oracle(n, sc, h, dt, threads=cores, **kw)
    o.load(*[p[k] for k in ("x", "y", "z", "ux", "uy", "uz", "w", "species")])
    npart = len(p["x"])
    del p
    o.set_fields([np.zeros(n)] * 9)
    if warmup > 0:
        o.step(int(warmup))
    t = time.perf_counter()
    o.step(int(steps))
    el = time.perf_counter() - t
    del o
    if pica_path:
        sample = (f"{what} ({npart} particles), pica's path: FP64 positions, CIC, Boris, direct deposition, "
                  f"supercell 4^3, {steps} steps after {warmup} warm-up, oracle form equal bit for bit to pica's "
                  f"headers, OpenMP {cores} threads")
    else:
        shape = "TSC" if kw["shape"] == po.SHAPE_TSC else "CIC"
        sample = (f"{what} ({npart} particles), {shape}, Esirkepov, supercell 4^3, FP32 cell form, {steps} steps "
                  f"after {warmup} warm-up, oracle restatement (pica has no Esirkepov"
                  f"{'' if shape == 'CIC' else ' or TSC'}), OpenMP {cores} threads")
    return npart * steps / el, cores, sample, el


def slab_measure(args, parts, resort):
    """The headline plasma stepped as args.slabs x-slab contexts on this GPU
    (pica_gb300.domain.local_decomposition: per step an E/B halo, the push of every
    slab, the current fold and halo, the field update and migration of every slab,
    and the particle exchange).  Slabs run one after another on the one GPU, so the
    step time is the sum over slabs plus the exchanges; the bench times whole steps
    with the host clock (the exchange reads counts back) and, separately, the halo,
    fold and exchange phases.  Checks that no particle is lost."""
    import torch

    import pica_gb300 as pg
    from pica_gb300 import domain

    wl = make_workload(args.edge, pg.FORM_FP32_CELL)
    sim = dict(wl["sim"])
    n, sc = sim.pop("n"), sim.pop("supercell")
    h, dt = sim.pop("h"), sim.pop("dt")
    dec = domain.local_decomposition(n, h, dt, sc, args.slabs, resort_every=resort, **sim)
    keys = ("x", "y", "z", "ux", "uy", "uz", "w", "species")
    total = len(parts["x"])
    zeros = [np.zeros(n)] * 9
    for d, part, f in zip(dec.domains, domain.split_particles(dec.plan, {k: parts[k] for k in keys}, h[0]),
                          domain.split_fields(dec.plan, zeros)):
        d.sim.upload_particles(*[part[k] for k in keys])
        d.sim.upload_fields(f)
    dec.step(3)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    dec.step(args.slab_steps)
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    # the exchange phases alone, once more after the timed steps
    t1 = time.perf_counter()
    dec.t.halo(dec.plan)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    for d in dec.domains:
        d.sim.push_deposit()
    torch.cuda.synchronize()
    t3 = time.perf_counter()
    dec.t.fold(dec.plan)
    dec.t.halo(dec.plan, domain.J)
    torch.cuda.synchronize()
    t4 = time.perf_counter()
    for d in dec.domains:
        d.sim.update_b(0.5 * dt)
        d.sim.update_e(dt)
        d.sim.update_b(0.5 * dt)
        d.sim.migrate()
    torch.cuda.synchronize()
    t5 = time.perf_counter()
    dec.t.exchange(dec.plan)
    torch.cuda.synchronize()
    t6 = time.perf_counter()
    owned = 0
    for r, d in enumerate(dec.domains):
        c = d.sim.counts().reshape(d.nspecies, -1, d.sim.nsc[1], d.sim.nsc[2])
        g = dec.plan.G // sc[0]
        owned += int(c[:, g:g + dec.plan.w[r] // sc[0]].sum())
    out = {"slabs": args.slabs, "guard_cells": dec.plan.G, "steps": args.slab_steps,
           "value": total * args.slab_steps / el, "unit": UNIT, "ms_per_step": 1e3 * el / args.slab_steps,
           "timer": "host clock, whole steps (the exchange reads counts back)",
           "phase_ms": {"halo": 1e3 * (t2 - t1), "push": 1e3 * (t3 - t2), "fold_and_current_halo": 1e3 * (t4 - t3),
                        "fields_and_migration": 1e3 * (t5 - t4), "particle_exchange": 1e3 * (t6 - t5)},
           "particles_conserved": owned == total}
    for d in dec.domains:
        d.sim.close()
    del dec
    torch.cuda.synchronize()
    return out


def flat_measure(args, parts, stream):
    """pica's own operators (FP64 positions, CIC, Boris, direct deposition) on the
    headline plasma in three layouts: supercells (pica_push_deposit, shared-memory
    current tiles), and one flat array (pica_push_flat, FP64 global atomics) in the
    generator's cell order, in a random order, and after EnsembleOrdered::reorder
    (pica_order_by_position).  Milliseconds per push by CUDA events (median of
    args.flat_steps after one untimed push), and the reorder's time."""
    import torch

    import pica_gb300 as pg

    keys = ("x", "y", "z", "ux", "uy", "uz", "w")
    wl = make_workload(args.edge, pg.FORM_FP64_PLAIN)
    sim = dict(wl["sim"], shape=pg.SHAPE_CIC, deposit=pg.DEPOSIT_DIRECT)
    n = sim["n"]

    def timed(fn, after=None):
        ts = []
        for r in range(args.flat_steps + 1):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
            if after:
                after()
        return float(np.median(ts[1:]))

    out = {"workload": "the headline plasma, FP64 positions, CIC, Boris, direct deposition, E = B = 0"}
    s = pg.Simulation(**sim)
    s.set_stream(stream.cuda_stream)
    s.upload_particles(*[parts[k] for k in keys], parts["species"])
    s.upload_fields([np.zeros(n)] * 9)

    def rest():
        s.update_b(0.5 * s.dt)
        s.update_e(s.dt)
        s.update_b(0.5 * s.dt)
        s.migrate()
    out["supercell_push_ms"] = timed(s.push_deposit, rest)
    s.close()
    f = pg.Simulation(**dict(sim, supercell=(1, 1, 1)))
    f.set_stream(stream.cuda_stream)
    f.upload_fields([np.zeros(n)] * 9)
    e = pg.FlatEnsemble(f)
    e.add(*[parts[k] for k in keys], parts["species"])
    out["flat_cell_order_push_ms"] = timed(e.push)
    g = torch.Generator(device="cuda")
    g.manual_seed(1)
    perm = torch.randperm(e.size(), device="cuda", generator=g)
    for k in e.KEYS:
        e.t[k] = e.t[k][perm].contiguous()
    e.species = e.species[perm].contiguous()
    del perm
    out["flat_random_push_ms"] = timed(e.push)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    e.reorder()
    b.record(stream)
    torch.cuda.synchronize()
    out["reorder_ms"] = a.elapsed_time(b)
    out["flat_ordered_push_ms"] = timed(e.push)
    out["pushes"] = args.flat_steps
    del e
    f.close()
    torch.cuda.synchronize()
    return out


def run_reference(args):
    """The CPU implementation of the path on this machine's host cores: the thermal
    headline workload at its full size (128^3 x 100 ppc unless --edge), K timed steps
    after W warm-up steps of the oracle restatement of its own step (FP32, TSC,
    Esirkepov; pica has neither), plus pica's own FP64 CIC/direct arithmetic on the
    same plasma (a few steps).  The two-stream and Weibel plasmas (8.4e8 and 2.1e9
    particles) do not fit a CPU run of minutes: for them, a block of the plasma."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    if args.workload == "thermal":
        edge = args.edge or 128
    else:
        edge = 32
    resort = args.resort_every
    value, cores, sample, el = cpu_sample(args.workload, edge, steps=args.steps, warmup=args.warmup,
                                          resort_every=resort)
    pk = max(1, min(args.steps, 3))
    pv, _, psample, _ = cpu_sample(args.workload, edge, steps=pk, warmup=min(1, args.warmup), pica_path=True,
                                   resort_every=resort)
    if args.workload == "thermal":
        ncells = edge ** 3
        config = bench_config(workload_description("thermal", edge), 100 * ncells, ncells, 1)
    else:
        config = {"workload": workload_description(args.workload, args.edge) + " (CPU step on a block of it: "
                  + sample.split(" (")[0] + ")", "parallelism": "OpenMP over supercells"}
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / max(1, args.steps),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
        "config": config,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample,
                         "pica_path": {"value": pv, "unit": UNIT, "cores": cores, "sample": psample}},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import torch

    import pica_gb300 as pg

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    # ---------------- FP32 form, device-resident ----------------
    headline = args.workload == "thermal"
    from pica_gb300.replicas import job_throughput, replica_seed
    stream = torch.cuda.current_stream()
    if headline:
        args.edge = args.edge or 128
        wl = make_workload(args.edge, pg.FORM_FP32_CELL)
        desc = workload_description("thermal", args.edge)
        resort = 2 if args.resort_every is None else args.resort_every
    else:
        wl, desc = named_workload(args.workload, args.edge)
        resort = wl["sim"].get("resort_every", 2) if args.resort_every is None else args.resort_every
    for spec in wl["specs"]:
        spec.seed = replica_seed(spec.seed, rank)   # independent replica per rank (weak scaling)
    ncells = int(np.prod(wl["sim"]["n"]))
    sim = pg.Simulation(**dict(wl["sim"], resort_every=resort))
    sim.set_stream(stream.cuda_stream)
    if headline:
        parts = pg.generate_plasma(wl["specs"][0])
        sim.upload_particles(*[parts[k] for k in ("x", "y", "z", "ux", "uy", "uz", "w")], parts["species"])
        npart = len(parts["x"])
    else:
        sim.generate_plasma(wl["specs"])   # on the device: no host copy of 1e9 particles
        parts = None
        npart = sim.num_particles()
    sim.upload_fields([np.zeros(wl["sim"]["n"])] * 9)
    dt = wl["sim"]["dt"]

    def one_step(ev0=None, ev1=None):
        if ev0 is not None:
            ev0.record(stream)
        sim.push_deposit()
        if ev1 is not None:
            ev1.record(stream)
        sim.update_b(0.5 * dt)
        sim.update_e(dt)
        sim.update_b(0.5 * dt)
        sim.migrate()

    # Launch variant of the push kernel chosen on this workload (part of the warm-up).
    from pica_gb300 import autotune
    if args.variant < 0:
        tune = autotune.tune_variant(sim)
    else:
        sim.set_variant(args.variant)
        tune = {}
    for _ in range(args.warmup):
        one_step()
    barrier()
    K = args.steps
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    t_start, t_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = sim.launch_count()
    with ClockSampler(local) as clk:
        barrier()
        t_start.record(stream)
        for k in range(K):
            one_step(*evs[k])
        t_end.record(stream)
        barrier()
    launches = sim.launch_count() - launches0
    sim_variant = sim.variant()[0]
    elapsed = t_start.elapsed_time(t_end) / 1e3
    push_ms = [a.elapsed_time(b) for a, b in evs]
    value, elapsed = job_throughput(npart, K, elapsed, dist, device="cuda")
    push_avg = float(np.mean(push_ms)) / 1e3
    peak, peak_kind = measured_hbm_peak()
    alg_bytes = BYTES_PER_PARTICLE_FP32 * npart + PUSH_GRID_BYTES_PER_CELL_FP32 * ncells
    achieved = alg_bytes / push_avg / 1e9
    kname = "CIC" if wl["sim"]["shape"] == pg.SHAPE_CIC else "TSC"
    roofline = {"bound": "hbm", "kernel": f"k_push_cell_esirkepov<{kname}>", "achieved": achieved, "peak": peak,
                "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                "traffic": None,   # DRAM bytes come from ncu only, never from a run that is timed
                "algorithmic_bytes_per_launch": alg_bytes, "push_ms": 1e3 * push_avg,
                "step_fraction_in_push": push_avg * K / elapsed}
    step_alg = BYTES_PER_PARTICLE_FP32 * npart + 120 * ncells
    clocks = clk.summary()

    # ---------------- e2e through the C ABI with host buffers ----------------
    # Every step uploads the particle state from pinned host memory, steps, and
    # downloads it again: the packed image of the used slots, moved in supercell
    # ranges (pica_state_copy_packed_range).  Uploads run on one copy stream and
    # downloads on another; range r of step n+1 goes up as soon as range r of step
    # n is down, so the two link directions overlap, and the push of range r starts
    # as soon as its upload is in (pica_push_deposit_chunked), overlapping the rest
    # of the upload.  With --e2e-split the host copies run on two copy streams and
    # the gather / scatter kernels on two others (pica_state_copy_packed_range_on),
    # so that each direction's copies follow one another without waiting for the
    # kernels in between.
    e2e = None
    if headline and args.e2e_steps > 0:
        comps = 8
        done = h2d = d2h = 0
        # High priority: the copy streams' pack and unpack kernels get SMs ahead of the push.
        up, down = torch.cuda.Stream(priority=-1), torch.cuda.Stream(priority=-1)
        upc, downc = (torch.cuda.Stream(priority=-1), torch.cuda.Stream(priority=-1)) if args.e2e_split else (up, down)
        cs_up = upc.cuda_stream if args.e2e_split else None
        cs_down = downc.cuda_stream if args.e2e_split else None
        ranges = sim.edge_split_ranges(args.e2e_chunks, args.e2e_edge_split)
        k = max(1, args.e2e_copy_split)
        pieces = [[(b + (e - b) * i // k, b + (e - b) * (i + 1) // k) for i in range(k)] for b, e in ranges]
        flat = [p for ps in pieces for p in ps]
        # Pinned host buffers are set up once, outside the timed region, with room
        # for the layout to grow at a resort or capacity rebuild.
        torch.cuda.synchronize()
        raw = bool(args.e2e_raw)
        state_slots = (lambda: sim.state_slots(0)) if raw else (lambda: sim.state_packed_slots(0))

        def copy(c, ptr, to_device, rg, cs):
            if raw:
                sim.state_copy_range(0, c, ptr, to_device, rg, copy_stream=cs)
            else:
                sim.state_copy_packed(0, c, ptr, to_device, sc_range=rg, copy_stream=cs)
        slots = state_slots()
        alloc = int(slots * 1.25) + 1024
        host = [torch.empty(alloc * 4, dtype=torch.uint8, pin_memory=True) for _ in range(comps)]
        for c in range(comps):
            copy(c, host[c].data_ptr(), False, (0, int(np.prod(sim.nsc))), None)
        torch.cuda.synchronize()
        downed = [None] * len(flat)
        trials = []
        for _trial in range(max(1, args.e2e_trials)):
            done = h2d = d2h = 0
            te0, te1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            barrier()
            w0 = time.perf_counter()
            te0.record(stream)
            up.wait_event(te0)
            upc.wait_event(te0)
            for _ in range(args.e2e_steps):
                upped = []
                sim.set_stream(up.cuda_stream)
                for r in range(len(ranges)):
                    for q in range(r * k, (r + 1) * k):
                        if downed[q] is not None:
                            upc.wait_event(downed[q])
                        for c in range(comps):
                            copy(c, host[c].data_ptr(), True, flat[q], cs_up)
                    ev = torch.cuda.Event()
                    ev.record(up)
                    upped.append(ev)
                h2d += slots * 4 * comps
                sim.set_stream(stream.cuda_stream)
                sim.push_deposit_ranges(ranges, [ev.cuda_event for ev in upped])
                sim.update_b(0.5 * dt)
                sim.update_e(dt)
                sim.update_b(0.5 * dt)
                sim.migrate()   # returns once the step's device work is done (it reads the flags)
                slots = state_slots()   # the image of the new layout and counts
                if slots > alloc:            # no copy is in flight here
                    torch.cuda.synchronize()
                    host = [torch.empty(slots * 4, dtype=torch.uint8, pin_memory=True) for _ in range(comps)]
                    alloc = slots
                stepped = torch.cuda.Event()
                stepped.record(stream)
                down.wait_event(stepped)
                sim.set_stream(down.cuda_stream)
                for q, rg in enumerate(flat):
                    for c in range(comps):
                        copy(c, host[c].data_ptr(), False, rg, cs_down)
                    downed[q] = torch.cuda.Event()
                    downed[q].record(downc)
                sim.set_stream(stream.cuda_stream)
                d2h += slots * 4 * comps
                done += 1
            for ev in downed:
                stream.wait_event(ev)
            te1.record(stream)
            barrier()
            wall = time.perf_counter() - w0
            e_el = te0.elapsed_time(te1) / 1e3
            trials.append((npart * done / max(e_el, wall), done, h2d, d2h, max(e_el, wall)))
        # The median run (by throughput) is the line's e2e; every run is listed.
        trials.sort(key=lambda t: t[0])
        _, done, h2d, d2h, e_t = trials[len(trials) // 2]
        link = host_link_probe()   # outside the timed region
        moved = (h2d + d2h) / e_t / 1e9
        e2e = {"value": world * npart * done / e_t, "unit": UNIT,
               "h2d_bytes_per_step": h2d // max(1, done), "d2h_bytes_per_step": d2h // max(1, done),
               "link_gbs": moved, "host_link": link, "link_frac": moved / link["both_gbs"],
               "steps": done, "trials": len(trials), "trial_values": [world * t[0] for t in trials],
               "ranges": len(ranges), "edge_split": args.e2e_edge_split, "copy_pieces": k,
               "split_copy_streams": bool(args.e2e_split), "raw_slots": raw,
               "path": "pica_state_copy_range_on (pinned host, the raw slots of each supercell range, no kernel) -> "
                       "pica_push_deposit_ranges (each range after its upload) -> pica_update_b/update_e/update_b/"
                       "migrate -> pica_state_slots, pica_state_copy_range_on; uploads and downloads overlapped "
                       "across steps on copy streams" if raw else
                       "pica_state_copy_packed_range_on (pinned host, per supercell range) -> "
                       "pica_push_deposit_ranges (each range after its upload) -> pica_update_b/update_e/update_b/"
                       "migrate -> pica_state_packed_slots, pica_state_copy_packed_range_on; uploads and downloads "
                       "overlapped across steps, host copies on copy streams apart from the gather / scatter "
                       "kernels" if args.e2e_split else
                       "pica_state_copy_packed_range (pinned host, per supercell range) -> "
                       "pica_push_deposit_ranges (each range after its upload) -> pica_update_b/update_e/update_b/"
                       "migrate -> pica_state_packed_slots, pica_state_copy_packed_range; uploads and downloads "
                       "on two copy streams, overlapped across steps"}
        del host
    sim.close()
    del sim
    torch.cuda.synchronize()

    # ---------------- FP64 plain form of the same workload ----------------
    fp64 = None
    if headline and args.fp64_steps > 0:
        wl64 = make_workload(args.edge, pg.FORM_FP64_PLAIN)
        s64 = pg.Simulation(**wl64["sim"])
        s64.set_stream(stream.cuda_stream)
        s64.upload_particles(*[parts[k] for k in ("x", "y", "z", "ux", "uy", "uz", "w")], parts["species"])
        s64.upload_fields([np.zeros(wl64["sim"]["n"])] * 9)
        s64.step(1)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        s64.step(args.fp64_steps)
        b.record(stream)
        torch.cuda.synchronize()
        el64 = a.elapsed_time(b) / 1e3
        fp64 = {"value": npart * args.fp64_steps / el64, "ms_per_step": 1e3 * el64 / args.fp64_steps,
                "steps": args.fp64_steps, "dtype": "fp64", "form": "FP64 plain (absolute positions)"}
        s64.close()

    # ---------------- flat layouts (EnsembleUnordered / EnsembleOrdered) ----------------
    flat = None
    if headline and args.flat_steps > 0:
        flat = flat_measure(args, parts, stream)

    # ---------------- one plasma as x slabs (domain decomposition on this GPU) ----------------
    slabs = None
    if headline and args.slabs > 0:
        slabs = slab_measure(args, parts, resort)

    # ---------------- batching form: many plasmas, persistent push + CUDA graph ----------------
    batched = None
    if headline and args.batched > 0:
        batched = batched_measure(args, rank, world, dist)

    # ---------------- FP32 form against the FP64 plain form (error metrics) ----------------
    errors = None
    if headline and args.validate_steps > 0 and rank == 0:
        from pica_gb300 import validate
        errors = validate.compare_forms(n=(32, 32, 32), ppc=100, steps=args.validate_steps, every=20)

    if rank != 0:
        if dist is not None:
            dist.barrier()
            dist.destroy_process_group()
        return
    cpu = None
    if not args.no_cpu_baseline:
        # A bounded sample: the headline plasma at its full size for 2 steps (the
        # two-stream and Weibel plasmas on a 32-cell-edge block for 3).
        parts = None
        edge = args.edge if headline else 32
        k = 2 if headline else 3
        v, cores, sample, _ = cpu_sample(args.workload, edge, steps=k, warmup=1, resort_every=resort)
        cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample}
        v, cores, sample, _ = cpu_sample(args.workload, edge, steps=k - 1, warmup=1, pica_path=True,
                                         resort_every=resort)
        cpu["pica_path"] = {"value": v, "unit": UNIT, "cores": cores, "sample": sample}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": args.warmup,
        "ms_per_step": 1e3 * elapsed / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32", "data": "synthetic",
        "config": bench_config(desc, npart, ncells, world),
        "roofline": roofline,
        "step_hbm_frac": step_alg / (elapsed / K) / 1e9 / peak,
        "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks, "gpu_launches": launches,
        "fp64_form": fp64, "fp32_over_fp64": (value / world / fp64["value"]) if fp64 else None,
        "fp32_vs_fp64_errors": errors,
        "flat_layout": flat,
        "slabs": slabs,
        "batched": batched,
        "tuning": {"push_variant": sim_variant, "variant_s_per_step": {str(k): v for k, v in tune.items()},
                   "resort_every": resort},
    }
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
