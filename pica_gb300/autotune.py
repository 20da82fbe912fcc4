"""Autotuner for the supercell PIC step.

Three knobs change speed:

* the launch variant of the FP32 charge-conserving push kernel (CTA size and
  CTAs per SM) -- ``tune_variant`` times each on the live simulation.  Every
  variant sums the same particles in the same order, so the results are the same
  bit for bit;
* the in-supercell resort cadence (how often each supercell is compacted and
  re-sorted by cell, which keeps the warps of the push kernel on one cell);
* the supercell edge (tile size against particles per CTA).

The last two change the order of particles within a supercell and hence the
FP32 rounding of the pre-summed window currents (results agree to FP32 rounding,
not bit for bit).

``tune_config`` searches the last two on a sample of the workload (a block of
the grid with the same particles per cell) through a caller-supplied factory
and caches the answer in a JSON file keyed by grid, particles per cell, form,
shape and depositor.  ``tune_batch_config`` does the same for the batching form
(one supercell edge for every member, one cadence), on a sample of the members.
"""
import json
import os
import time

DEFAULT_CACHE = os.path.join(os.path.expanduser("~"), ".cache", "pica_gb300", "autotune.json")


def _timed_steps(sim, steps):
    sim.synchronize()
    t = time.perf_counter()
    sim.step(steps)
    sim.synchronize()
    return (time.perf_counter() - t) / steps


def tune_variant(sim, steps=None, rounds=3):
    """Time every launch variant and keep the fastest.  Returns {variant: s/step},
    the median over `rounds` rounds.  Each round times every variant for `steps`
    steps (default: the resort cadence, so that every window holds one resort, the
    push right after it and those between resorts; 3 without a cadence), in an
    order rotated from round to round: a plasma that evolves while the variants are
    timed one after another then biases none of them.  The simulation advances by
    variants x (1 + rounds x steps) steps."""
    _, count = sim.variant()
    if steps is None:
        cfg = getattr(sim, "cfg", None)
        every = int(getattr(cfg, "resort_every", 0)) if cfg is not None else 0
        steps = every if every > 0 else 3
    for v in range(count):
        sim.set_variant(v)
        sim.step(1)  # first launch of a variant sets its attributes
    samples = {v: [] for v in range(count)}
    for r in range(rounds):
        for j in range(count):
            v = (j + r) % count
            sim.set_variant(v)
            samples[v].append(_timed_steps(sim, steps))
    times = {v: sorted(t)[len(t) // 2] for v, t in samples.items()}
    best = min(times, key=times.get)
    sim.set_variant(best)
    return times


def tune_batch(batch, steps=2, variants=4):
    """tune_variant for a Batch: time each launch variant of the batched push (graph
    replay, after one capture step) and keep the fastest.  Returns {variant: s/step}."""
    times = {}
    for v in range(variants):
        batch.set_options(use_graph=True, variant=v)
        batch.step(1)
        t = time.perf_counter()
        batch.step(steps)
        times[v] = (time.perf_counter() - t) / steps
    best = min(times, key=times.get)
    batch.set_options(use_graph=True, variant=best)
    return times


def config_key(n, ppc, form, shape, deposit):
    return f"{n[0]}x{n[1]}x{n[2]}|ppc={ppc}|form={form}|shape={shape}|deposit={deposit}"


def tune_config(make_sim, key, supercells=((4, 4, 4), (2, 2, 2)), cadences=(4, 8, 16), steps=4, cache=DEFAULT_CACHE):
    """make_sim(supercell, resort_every) -> Simulation with particles and fields loaded
    (a sample of the workload).  Returns the best {"supercell", "resort_every",
    "variant", "s_per_step"} and stores it in `cache` under `key`."""
    if cache and os.path.exists(cache):
        with open(cache) as f:
            known = json.load(f)
        if key in known:
            return known[key]
    else:
        known = {}
    best = None
    for sc in supercells:
        for every in cadences:
            sim = make_sim(sc, every)
            vt = tune_variant(sim, steps=1, rounds=1)
            v = min(vt, key=vt.get)
            sim.set_variant(v)
            t = _timed_steps(sim, steps)
            sim.close()
            if best is None or t < best["s_per_step"]:
                best = {"supercell": list(sc), "resort_every": every, "variant": v, "s_per_step": t}
    if cache:
        os.makedirs(os.path.dirname(cache), exist_ok=True)
        known[key] = best
        with open(cache, "w") as f:
            json.dump(known, f, indent=1)
    return best


def tune_batch_config(make_batch, supercells=((4, 4, 4), (2, 2, 2)), cadences=(2, 4, 8), steps=3):
    """Supercell edge and resort cadence of the batching form.  make_batch(supercell,
    resort_every) -> Batch with its members' particles and fields loaded (a sample of
    the workload's members).  Each combination: the fastest push variant
    (tune_batch), then `steps` timed steps after a resort-cadence's worth of warm-up
    (so that sorted and unsorted pushes are both timed).  Returns the best
    {"supercell", "resort_every", "variant", "s_per_step"} and every combination's
    time under "tried"."""
    best, tried = None, {}
    for sc in supercells:
        for every in cadences:
            b = make_batch(sc, every)
            vt = tune_batch(b, steps=2)
            v = min(vt, key=vt.get)
            b.set_options(use_graph=True, variant=v)
            b.step(every)
            t0 = time.perf_counter()
            b.step(max(steps, every))
            t = (time.perf_counter() - t0) / max(steps, every)
            b.close()
            tried[f"{sc[0]}x{sc[1]}x{sc[2]}/every{every}"] = t
            if best is None or t < best["s_per_step"]:
                best = {"supercell": list(sc), "resort_every": every, "variant": v, "s_per_step": t}
    best["tried"] = tried
    return best
