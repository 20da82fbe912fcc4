"""Synthetic plasma workloads (seeded; generated on the host by generate_plasma or on
the device by Simulation.generate_plasma, from the same specs).

Each workload gives the Simulation arguments, the plasma specs and a step
count.  Physical set-up shared by all of them: electron density n0 =
1e18 cm^-3, cell size h = 0.05 c / omega_p (the Debye length of a plasma with
thermal spread u = 0.05), time step dt = 0.5 h / (c sqrt 3) (half the 3D
Courant limit), macro-particle weight n0 h^3 / (particles per cell).
"""
import math

from . import (DEPOSIT_DIRECT, DEPOSIT_ESIRKEPOV, ELECTRON_CHARGE, ELECTRON_MASS, FORM_FP32_CELL, FORM_FP64_PLAIN,
               LIGHT_VELOCITY, PI, SHAPE_CIC, SHAPE_TSC, plasma_spec)

N0 = 1e18


def plasma_frequency(n0=N0, mass=ELECTRON_MASS):
    return math.sqrt(4.0 * PI * n0 * ELECTRON_CHARGE ** 2 / mass)


def cell_size(n0=N0):
    return 0.05 * LIGHT_VELOCITY / plasma_frequency(n0)


def time_step(h):
    return 0.5 * h / (LIGHT_VELOCITY * math.sqrt(3.0))


def background_density(n0=N0):
    """Charge density of immobile neutralising ions (statC/cm^3)."""
    return -ELECTRON_CHARGE * n0


def _u_of_beta(beta):
    return beta / math.sqrt(1.0 - beta * beta)


def thermal(n=(32, 32, 32), ppc=50, sigma=0.05, supercell=(2, 2, 2), form=FORM_FP64_PLAIN, shape=SHAPE_CIC,
            deposit=DEPOSIT_DIRECT, steps=100, seed=20261203):
    """Electron plasma with immobile ions, E = B = 0, Maxwellian u ~ N(0, sigma)."""
    h = cell_size()
    hh = (h, h, h)
    sim = dict(n=n, h=hh, dt=time_step(h), supercell=supercell, form=form, shape=shape, deposit=deposit)
    spec = plasma_spec(n, hh, ppc, sigma, N0 * h ** 3 / ppc, seed)
    return dict(name=f"thermal {n[0]}x{n[1]}x{n[2]} ppc={ppc}", sim=sim, specs=[spec], steps=steps,
                bg=background_density())


def config1():
    """Plain FP64 3D electron plasma: 32^3, 50 ppc, CIC, Boris, direct, supercell 2^3, 100 steps."""
    return thermal()


def config2(form=FORM_FP32_CELL):
    """128^3, 100 ppc (2.1e8 electrons), TSC, Esirkepov, supercell 4^3, 1000 steps."""
    return thermal(n=(128, 128, 128), ppc=100, supercell=(4, 4, 4), form=form, shape=SHAPE_TSC,
                   deposit=DEPOSIT_ESIRKEPOV, steps=1000)


def two_stream(n=(256, 256, 128), ppc=100, beta=0.2, sigma=0.01, modulation=0.9, supercell=(4, 4, 4),
               form=FORM_FP32_CELL, shape=SHAPE_CIC, deposit=DEPOSIT_ESIRKEPOV, steps=500, seed=20261203):
    """Two electron beams at +-beta c along x, density 1 + a cos(2 pi x / Lx) (per-cell counts
    round(ppc (1 + a cos)), split evenly between the beams)."""
    h = cell_size()
    hh = (h, h, h)
    sim = dict(n=n, h=hh, dt=time_step(h), supercell=supercell, form=form, shape=shape, deposit=deposit,
               resort_every=4)
    spec = plasma_spec(n, hh, ppc, sigma, N0 * h ** 3 / ppc, seed, density_mod=modulation, nbeams=2,
                       drift_u=_u_of_beta(beta), drift_axis=0)
    return dict(name=f"two-stream {n[0]}x{n[1]}x{n[2]}", sim=sim, specs=[spec], steps=steps, bg=background_density())


def config3():
    return two_stream()


def weibel(n=(256, 256, 256), ppc_per_beam=32, beta=0.3, sigma=0.01, mass_ratio=100.0, supercell=(4, 4, 4),
           form=FORM_FP32_CELL, steps=300, seed=20261203):
    """Counter-streaming electrons and mobile ions (m_i = 100 m_e), beams +-beta c along z."""
    h = cell_size()
    hh = (h, h, h)
    ion = (ELECTRON_MASS * mass_ratio, -ELECTRON_CHARGE)
    sim = dict(n=n, h=hh, dt=time_step(h), supercell=supercell, form=form, shape=SHAPE_TSC,
               deposit=DEPOSIT_ESIRKEPOV, species=((ELECTRON_MASS, ELECTRON_CHARGE), ion), resort_every=1)
    w = N0 * h ** 3 / (2 * ppc_per_beam)
    u = _u_of_beta(beta)
    specs = [plasma_spec(n, hh, 2 * ppc_per_beam, sigma, w, seed, species=0, nbeams=2, drift_u=u, drift_axis=2),
             plasma_spec(n, hh, 2 * ppc_per_beam, sigma / math.sqrt(mass_ratio), w, seed + 1, species=1, nbeams=2,
                         drift_u=u, drift_axis=2)]
    return dict(name=f"weibel {n[0]}^3", sim=sim, specs=specs, steps=steps, bg=0.0)


def config5():
    return weibel()


def batched_members(count=64, seed_base=0, half=False, resort_every=4, supercell=(4, 4, 4)):
    """64 independent thermal plasmas: plasma k seeded by k; edge in {32, 36, ..., 96}, ppc in
    16..128, sigma in [0.02, 0.1].  Uses a SplitMix64 stream so the draws are reproducible.
    half=True halves every edge (rounded to a multiple of 4): the same members at 1/8 of
    the cells.  `supercell` and `resort_every` apply to every member (the batching form
    takes one supercell edge for all)."""
    def mix(z):
        z = (z + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
        return z ^ (z >> 31)

    out = []
    for k in range(count):
        r = [mix((seed_base + k) * 16 + i) for i in range(3)]
        edge = 32 + 4 * (r[0] % 17)
        if half:
            edge = 4 * round(edge / 8)
        ppc = 16 + r[1] % 113
        sigma = 0.02 + 0.08 * (r[2] >> 11) / float(1 << 53)
        wl = thermal(n=(edge, edge, edge), ppc=ppc, sigma=sigma, supercell=tuple(supercell), form=FORM_FP32_CELL,
                     shape=SHAPE_CIC, deposit=DEPOSIT_ESIRKEPOV, steps=200, seed=1000 + k)
        wl["sim"]["resort_every"] = resort_every
        out.append(wl)
    return out
