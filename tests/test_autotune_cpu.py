"""The autotuner's search on the CPU, through fakes of a Simulation and a Batch whose
steps take a known time: every combination is timed, the fastest is chosen, and
tune_config caches its answer by key."""
import json
import time

from pica_gb300 import autotune


class FakeSim:
    """A simulation whose step takes `cost(variant)` seconds."""

    def __init__(self, cost):
        self.cost, self.v, self.closed = cost, 0, False

    def variant(self):
        return self.v, 3

    def set_variant(self, v):
        self.v = v

    def step(self, n=1):
        time.sleep(n * self.cost(self.v))

    def synchronize(self):
        pass

    def close(self):
        self.closed = True


class FakeBatch(FakeSim):
    def set_options(self, use_graph=True, variant=0):
        self.v = variant


def test_tune_variant_keeps_the_fastest():
    s = FakeSim(lambda v: {0: 0.006, 1: 0.002, 2: 0.004}[v])
    t = autotune.tune_variant(s, steps=2)
    assert set(t) == {0, 1, 2} and s.v == 1


def test_tune_config_searches_every_combination_and_caches(tmp_path):
    made = []

    def make(sc, every):
        made.append((tuple(sc), every))
        return FakeSim(lambda v: 0.001 * (sc[0] + abs(every - 8) + v))

    cache = str(tmp_path / "tune.json")
    best = autotune.tune_config(make, "k", supercells=((4, 4, 4), (2, 2, 2)), cadences=(4, 8), steps=2, cache=cache)
    assert sorted(made) == sorted([((4, 4, 4), 4), ((4, 4, 4), 8), ((2, 2, 2), 4), ((2, 2, 2), 8)])
    assert best["supercell"] == [2, 2, 2] and best["resort_every"] == 8 and best["variant"] == 0
    assert json.load(open(cache))["k"] == best
    made.clear()
    assert autotune.tune_config(make, "k", cache=cache) == best and made == []   # from the cache


def test_tune_batch_config_picks_the_fastest_combination():
    def make(sc, every):
        return FakeBatch(lambda v: 0.001 * (sc[0] / 2 + (every == 2) + 0.5 * v))

    best = autotune.tune_batch_config(make, supercells=((4, 4, 4), (2, 2, 2)), cadences=(2, 4), steps=2)
    assert set(best["tried"]) == {"4x4x4/every2", "4x4x4/every4", "2x2x2/every2", "2x2x2/every4"}
    assert best["supercell"] == [2, 2, 2] and best["resort_every"] == 4 and best["variant"] == 0
