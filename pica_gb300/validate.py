"""FP32 precision form against the FP64 plain form, from the same seeded input.

Both forms run the same step (shape, depositor, supercell policy) on the GPU; the
FP64 plain form is the one pinned to pica's own FP64 arithmetic.  Error metrics,
all from FP64 reductions on the GPU:

* energy drift: W(t) = field + kinetic energy; the relative drift
  (W(t) - W(0)) / W(0) of the FP32 form minus that of the FP64 form, largest
  magnitude over the run;
* RMS momentum error after `rms_steps` steps: sqrt(mean |u32 - u64|^2) /
  sqrt(mean |u64|^2), particles matched by ensemble slot (valid while both forms
  keep every particle in the same cell, which is checked);
* charge-conservation residual of the FP32 form over one step:
  max |(rho^{n+1} - rho^n)/dt + div J^{n+1/2}| on the cell-centred lattice,
  divided by max |rho^n| / dt, and also by max |(rho^{n+1} - rho^n)/dt|.
"""
import numpy as np

from . import DEPOSIT_ESIRKEPOV, FORM_FP32_CELL, FORM_FP64_PLAIN, SHAPE_TSC, Simulation, generate_plasma
from . import workloads


def div_faces(jx, jy, jz, h):
    """Divergence at cell centres of face-centred J (pica's J staggering, periodic)."""
    return ((np.roll(jx, -1, 0) - jx) / h[0] + (np.roll(jy, -1, 1) - jy) / h[1] + (np.roll(jz, -1, 2) - jz) / h[2])


def _make(wl, form, particles):
    s = dict(wl["sim"])
    s["form"] = form
    sim = Simulation(**s)
    sim.upload_particles(particles["x"], particles["y"], particles["z"], particles["ux"], particles["uy"],
                         particles["uz"], particles["w"], particles["species"])
    n = s["n"]
    sim.upload_fields([np.zeros(n)] * 9)
    return sim


def _energy(sim, bg):
    d = sim.diagnostics(bg)
    return d["field_energy"] + d["kinetic_energy"]


def charge_residual(sim):
    """One step of `sim`; returns (residual / (max|rho|/dt), residual / max|drho/dt|)."""
    r0 = sim.charge_density()
    sim.push_deposit()
    f = sim.fields()
    sim.update_b(0.5 * sim.dt)
    sim.update_e(sim.dt)
    sim.update_b(0.5 * sim.dt)
    sim.migrate()
    r1 = sim.charge_density()
    drho = (r1 - r0) / sim.dt
    res = np.max(np.abs(drho + div_faces(f[6], f[7], f[8], sim.h)))
    return float(res / (np.max(np.abs(r0)) / sim.dt)), float(res / max(np.max(np.abs(drho)), 1e-300))


def rms_momentum_error(a, b):
    """RMS |u_a - u_b| / RMS |u_b| with particles matched by slot; None if the ensembles differ."""
    if len(a["x"]) != len(b["x"]) or not np.array_equal(a["supercell"], b["supercell"]):
        return None
    du = sum((a[k] - b[k]) ** 2 for k in ("ux", "uy", "uz"))
    u2 = sum(b[k] ** 2 for k in ("ux", "uy", "uz"))
    return float(np.sqrt(np.mean(du) / np.mean(u2)))


def compare_forms(n=(32, 32, 32), ppc=100, steps=1000, every=10, rms_steps=10, seed=20261203, shape=SHAPE_TSC,
                  deposit=DEPOSIT_ESIRKEPOV, supercell=(4, 4, 4), sigma=0.05):
    """Run the thermal plasma in both forms; returns the error metrics and the energy histories."""
    wl = workloads.thermal(n=n, ppc=ppc, sigma=sigma, supercell=supercell, shape=shape, deposit=deposit, seed=seed)
    particles = generate_plasma(wl["specs"][0])
    bg = wl["bg"]
    sims = {f: _make(wl, f, particles) for f in (FORM_FP64_PLAIN, FORM_FP32_CELL)}
    hist = {f: [_energy(s, bg)] for f, s in sims.items()}
    rms = None
    done = 0
    while done < steps:
        k = min(every, steps - done)
        if done < rms_steps < done + k:
            k = rms_steps - done
        for f, s in sims.items():
            s.step(k)
            hist[f].append(_energy(s, bg))
        done += k
        if done == rms_steps:
            rms = rms_momentum_error(sims[FORM_FP32_CELL].particles(), sims[FORM_FP64_PLAIN].particles())
    drift = {f: (np.array(h) - h[0]) / h[0] for f, h in hist.items()}
    res_rho, res_drho = charge_residual(sims[FORM_FP32_CELL])
    for s in sims.values():
        s.close()
    dd = drift[FORM_FP32_CELL] - drift[FORM_FP64_PLAIN]
    return {
        "sample": f"thermal {n[0]}x{n[1]}x{n[2]} x {ppc} ppc, sigma {sigma}, supercell {supercell[0]}, {steps} steps",
        "steps": steps,
        "energy_drift_fp64": float(drift[FORM_FP64_PLAIN][-1]),
        "energy_drift_fp32": float(drift[FORM_FP32_CELL][-1]),
        "energy_drift_diff_max": float(np.max(np.abs(dd))),
        "rms_momentum_error": rms,
        "rms_momentum_steps": rms_steps,
        "charge_residual": res_rho,
        "charge_residual_vs_drho": res_drho,
    }
