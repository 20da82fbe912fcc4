"""bench.py's reference arm on the CPU: one JSON line with the keys of the bench
contract (the oracle's CPU step of the thermal workload, all host cores; here on
a 16^3 grid), no pica_gb300 module or library in its process, the same `config`
as the GPU arm's, and a second rank of a multi-rank launch that prints nothing.
The oracle's description of each workload equals pica_gb300.workloads."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run(args, env=None):
    e = dict(os.environ)
    e.update(env or {})
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args, capture_output=True, text=True,
                       timeout=600, env=e, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    return [ln for ln in r.stdout.splitlines() if ln.strip()]


def test_reference_arm_prints_one_contract_line():
    lines = run(["--impl", "reference", "--steps", "2", "--warmup", "1", "--edge", "16"])
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for k in ("metric", "unit", "config", "dtype", "data", "scaling"):
        assert d[k], k
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["steps"] == 2 and d["warmup"] == 1 and d["n_gpus"] == 1
    assert d["higher_is_better"] is True
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["unit"] == d["unit"] and cb["cores"] >= 1
    assert cb["kind"] in ("port", "reference") and cb["sample"]
    assert cb["pica_path"]["value"] > 0 and "pica's path" in cb["pica_path"]["sample"]
    sys.path.insert(0, ROOT)
    import bench
    assert d["config"] == bench.bench_config(bench.workload_description("thermal", 16), 100 * 16 ** 3, 16 ** 3, 1)
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_print_nothing():
    assert run(["--impl", "reference", "--steps", "1", "--warmup", "0"], env={"RANK": "1", "WORLD_SIZE": "2"}) == []


def test_reference_arm_loads_no_product_code():
    code = ("import sys, runpy; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0', "
            "'--edge', '8']; runpy.run_path('bench.py', run_name='__main__'); "
            "maps = open('/proc/self/maps').read(); "
            "print('MODULE' if any(m.startswith('pica_gb300') for m in sys.modules) else 'nomodule'); "
            "print('LIB' if 'libpica_gb300' in maps else 'nolib')")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    out = r.stdout.split()
    assert out[-2:] == ["nomodule", "nolib"], r.stdout


def test_oracle_workloads_equal_the_package_workloads():
    sys.path.insert(0, ROOT)
    import bench
    import pica_gb300 as pg
    from pica_gb300 import workloads
    cases = {"thermal": (workloads.thermal(n=(16, 16, 16), ppc=100, supercell=(4, 4, 4), form=pg.FORM_FP32_CELL,
                                           shape=pg.SHAPE_TSC, deposit=pg.DEPOSIT_ESIRKEPOV), 16, 2),
             "two_stream": (workloads.two_stream(n=(16, 16, 8)), 16, 4),
             "weibel": (workloads.weibel(n=(16, 16, 16)), 16, 1)}
    for name, (wl, edge, resort) in cases.items():
        kw, specs, _ = bench.oracle_workload(name, edge)
        sim = wl["sim"]
        assert tuple(kw["n"]) == tuple(sim["n"]) and tuple(kw["sc"]) == tuple(sim["supercell"]), name
        assert tuple(kw["h"]) == tuple(sim["h"]) and kw["dt"] == sim["dt"], name
        assert (kw["shape"], kw["deposit"], kw["form"]) == (sim["shape"], sim["deposit"], sim["form"]), name
        assert tuple(kw["species"]) == tuple(sim.get("species", (pg.ELECTRON,))), name
        assert kw["resort_every"] == resort and sim.get("resort_every", resort) == resort, name
        assert len(specs) == len(wl["specs"]), name
        for a, b in zip(specs, wl["specs"]):
            for f, _ in a._fields_:
                va, vb = getattr(a, f), getattr(b, f)
                if hasattr(va, "__len__"):
                    va, vb = list(va), list(vb)
                assert va == vb, (name, f)
