"""FP32 precision form against the FP64 plain form, from the same seeded input.

Both forms run the same step (shape, depositor, supercell policy) on the GPU; the
FP64 plain form is the one pinned to pica's own FP64 arithmetic.  Error metrics,
all from FP64 reductions on the GPU:

* energy drift: W(t) = field + kinetic energy; the relative drift
  (W(t) - W(0)) / W(0) of the FP32 form minus that of the FP64 form, largest
  magnitude over the run;
* RMS momentum error after `rms_steps` steps: sqrt(mean |u32 - u64|^2) /
  sqrt(mean |u64|^2) over matched particles.  Particles are matched by ensemble
  slot within each (species, supercell) whose counts and slot-wise positions
  agree; a rounding difference at a cell face can put a particle in the next
  cell in one form, which changes the counts or, after a resort, the slot order
  of the supercells around it, and those supercells are matched by nearest
  neighbour in (position, momentum) instead (`match_particles`);
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


def match_particles(a, b, L, nsc3, pos_tol=1e-3):
    """One-to-one match of two ensembles of the same plasma (particles() dicts).

    Slot by slot within every (species, supercell) whose counts agree and whose
    slot-wise positions lie within pos_tol of the box edge per axis; the particles of
    the other supercells (a particle that sits in neighbouring supercells in the two
    ensembles makes both of them disagree) are matched by nearest neighbour in
    (position, momentum), positions periodic, across all of them at once.  Returns
    index arrays (ia, ib) and the number of particles matched by nearest neighbour;
    None when the ensembles differ in size per species or the match is not one to
    one."""
    nsc = int(np.prod(nsc3))
    nsp = int(max(a["species"].max(initial=0), b["species"].max(initial=0))) + 1
    ka = a["species"].astype(np.int64) * nsc + a["supercell"]
    kb = b["species"].astype(np.int64) * nsc + b["supercell"]
    ca, cb = np.bincount(ka, minlength=nsp * nsc), np.bincount(kb, minlength=nsp * nsc)
    if not np.array_equal(ca.reshape(nsp, nsc).sum(1), cb.reshape(nsp, nsc).sum(1)):
        return None
    sa, sb = np.cumsum(ca) - ca, np.cumsum(cb) - cb
    ib = np.nonzero(ca[kb] == cb[kb])[0]
    ia = sa[kb[ib]] + (ib - sb[kb[ib]])
    bad = np.zeros(len(ib), bool)
    for d, k in enumerate(("x", "y", "z")):
        dd = np.abs(a[k][ia] - b[k][ib])
        bad |= np.minimum(dd, L[d] - dd) >= pos_tol * L[d]
    groups = np.union1d(np.nonzero(ca != cb)[0], kb[ib[bad]])
    if len(groups) == 0:
        return ia, ib, 0
    near = np.unique(groups % nsc)
    keep = ~np.isin(b["supercell"][ib], near)
    ia, ib = [ia[keep]], [ib[keep]]
    from scipy.spatial import cKDTree
    umax = [max(np.max(np.abs(b[k])), 1e-300) for k in ("ux", "uy", "uz")]
    scale = np.array([pos_tol * L[0], pos_tol * L[1], pos_tol * L[2]] + umax)
    box = np.array([1.0 / pos_tol] * 3 + [1e12] * 3)
    shift = np.array([0.0] * 3 + [0.5e12] * 3)
    nn = 0
    for q in range(nsp):
        ja = np.nonzero(np.isin(a["supercell"], near) & (a["species"] == q))[0]
        jb = np.nonzero(np.isin(b["supercell"], near) & (b["species"] == q))[0]
        if len(ja) != len(jb):
            return None
        comps = ("x", "y", "z", "ux", "uy", "uz")
        pa = np.mod(np.stack([a[k][ja] for k in comps], axis=1) / scale + shift, box)
        pb = np.mod(np.stack([b[k][jb] for k in comps], axis=1) / scale + shift, box)
        _, j = cKDTree(pb, boxsize=box).query(pa)
        if len(np.unique(j)) != len(ja):
            return None
        ia.append(ja)
        ib.append(jb[j])
        nn += len(ja)
    return np.concatenate(ia), np.concatenate(ib), nn


def rms_momentum_error(a, b, L, nsc3):
    """RMS |u_a - u_b| / RMS |u_b| over matched particles (`match_particles`).
    Returns (error, particles matched by nearest neighbour); (None, 0) when the
    ensembles cannot be matched one to one."""
    m = match_particles(a, b, L, nsc3)
    if m is None:
        return None, 0
    ia, ib, nn = m
    du = sum((a[k][ia] - b[k][ib]) ** 2 for k in ("ux", "uy", "uz"))
    u2 = sum(b[k][ib] ** 2 for k in ("ux", "uy", "uz"))
    return float(np.sqrt(np.mean(du) / np.mean(u2))), nn


def compare_forms(n=(32, 32, 32), ppc=100, steps=1000, every=10, rms_steps=10, seed=20261203, shape=SHAPE_TSC,
                  deposit=DEPOSIT_ESIRKEPOV, supercell=(4, 4, 4), sigma=0.05):
    """Run the thermal plasma in both forms; returns the error metrics and the energy histories."""
    wl = workloads.thermal(n=n, ppc=ppc, sigma=sigma, supercell=supercell, shape=shape, deposit=deposit, seed=seed)
    particles = generate_plasma(wl["specs"][0])
    bg = wl["bg"]
    sims = {f: _make(wl, f, particles) for f in (FORM_FP64_PLAIN, FORM_FP32_CELL)}
    hist = {f: [_energy(s, bg)] for f, s in sims.items()}
    rms, rms_nn = None, 0
    L = [n[d] * wl["sim"]["h"][d] for d in range(3)]
    nsc3 = tuple(n[d] // supercell[d] for d in range(3))
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
            rms, rms_nn = rms_momentum_error(sims[FORM_FP32_CELL].particles(), sims[FORM_FP64_PLAIN].particles(), L,
                                             nsc3)
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
        "rms_momentum_nn_matched": rms_nn,
        "charge_residual": res_rho,
        "charge_residual_vs_drho": res_drho,
    }
