"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loads oracle/build/libpic_oracle.so (the restatement, ``Oracle(kind="port")``)
or oracle/_ref/libpica_ref.so (the harness over pica's own headers,
``Oracle(kind="reference")``).  Only tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py import this module; the pica_gb300 package never
does.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "build", "libpic_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libpica_ref.so")

FORM_FP64_PLAIN, FORM_FP32_CELL = 0, 1
SHAPE_CIC, SHAPE_TSC = 1, 2
DEPOSIT_DIRECT, DEPOSIT_ESIRKEPOV = 0, 1


class OrcConfig(C.Structure):
    _fields_ = [
        ("n", C.c_int32 * 3), ("sc", C.c_int32 * 3), ("h", C.c_double * 3), ("dt", C.c_double),
        ("form", C.c_int32), ("shape", C.c_int32), ("deposit", C.c_int32), ("nspecies", C.c_int32),
        ("mass", C.c_double * 4), ("charge", C.c_double * 4), ("threads", C.c_int32), ("resort_every", C.c_int32),
    ]


class OrcDiag(C.Structure):
    _fields_ = [("field_energy", C.c_double), ("kinetic_energy", C.c_double), ("total_charge", C.c_double),
                ("gauss_max", C.c_double), ("rho_max", C.c_double), ("pad_", C.c_double * 3)]


class OrcPlasma(C.Structure):
    """orc_plasma (oracle/pic_oracle.h): one synthetic population."""
    _fields_ = [
        ("n", C.c_int32 * 3), ("species", C.c_int32), ("h", C.c_double * 3), ("ppc", C.c_double),
        ("density_mod", C.c_double), ("drift_u", C.c_double), ("sigma_u", C.c_double), ("weight", C.c_double),
        ("seed", C.c_uint64), ("nbeams", C.c_int32), ("drift_axis", C.c_int32),
    ]


def plasma(n, h, ppc, sigma, weight, seed, species=0, density_mod=0.0, drift_u=0.0, drift_axis=0, nbeams=1):
    s = OrcPlasma()
    for d in range(3):
        s.n[d], s.h[d] = int(n[d]), float(h[d])
    s.species, s.ppc, s.density_mod, s.drift_u, s.sigma_u = int(species), float(ppc), float(density_mod), \
        float(drift_u), float(sigma)
    s.weight, s.seed, s.nbeams, s.drift_axis = float(weight), int(seed), int(nbeams), int(drift_axis)
    return s


def generate(specs, threads=0):
    """The populations `specs` (OrcPlasma) drawn on the host by the oracle's generator,
    concatenated in order: a dict of x y z ux uy uz w (FP64) and species (int32)."""
    lib, _ = _lib("port")
    counts = [int(lib.orc_plasma_count(C.byref(s))) for s in specs]
    if min(counts, default=0) < 0:
        raise ValueError("bad plasma description")
    n = sum(counts)
    out = {k: np.empty(n) for k in ("x", "y", "z", "ux", "uy", "uz", "w")}
    out["species"] = np.empty(n, np.int32)
    o = 0
    for s, c in zip(specs, counts):
        ptr = [out[k][o:].ctypes.data_as(C.POINTER(C.c_double)) for k in ("x", "y", "z", "ux", "uy", "uz", "w")]
        if lib.orc_plasma_generate(C.byref(s), int(threads), *ptr, out["species"][o:].ctypes.data_as(C.POINTER(C.c_int32))):
            raise RuntimeError("plasma generation failed")
        o += c
    return out


def pica_include_dir():
    """pica's include directory when the pica sources are mounted (the recipe in
    oracle/Makefile knows where: PICA_REF), else None."""
    r = subprocess.run(["make", "-s", "-C", HERE, "include-dir"], capture_output=True, text=True)
    d = r.stdout.strip()
    return d if r.returncode == 0 and d and os.path.isdir(os.path.join(d, "pica")) else None


def reference_available():
    """True when the harness over pica's headers is built or can be built here."""
    return os.path.exists(REF_SO) or pica_include_dir() is not None


def build(reference=True):
    """Compile the restatement (and, where the pica sources exist, the harness)."""
    targets = ["oracle"] + (["ref"] if reference else [])
    subprocess.run(["make", "-s", "-C", HERE] + targets, check=True)


_libs = {}


def _lib(kind):
    if kind not in _libs:
        path = PORT_SO if kind == "port" else REF_SO
        if not os.path.exists(path):
            build(reference=(kind == "reference"))
        lib = C.CDLL(path)
        p = "orc_" if kind == "port" else "ref_"
        vp, dp, ip, i64 = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int32), C.c_int64
        sig = {
            "create": (vp, [C.POINTER(OrcConfig)]), "destroy": (None, [vp]),
            "load": (C.c_int, [vp, i64] + [dp] * 7 + [ip]),
            "set_fields": (C.c_int, [vp, C.POINTER(dp)]), "get_fields": (C.c_int, [vp, C.POINTER(dp)]),
            "step": (C.c_int, [vp, C.c_int32]), "num_particles": (i64, [vp]),
            "get_particles": (C.c_int, [vp] + [dp] * 7 + [ip, ip]),
            "get_counts": (C.c_int, [vp, ip]), "num_migrations": (i64, [vp]),
            "get_migrations": (C.c_int, [vp, ip, ip, ip, ip]),
            "order_by_position": (C.c_int, [i64, C.c_int32, dp, dp, dp, C.POINTER(C.c_int64)]),
            "push_flat": (C.c_int, [C.POINTER(OrcConfig), C.c_int32, i64] + [dp] * 7 + [ip, C.POINTER(dp),
                                                                                   C.POINTER(dp)]),
        }
        if kind == "port":
            fp = C.POINTER(C.c_float)
            sig.update({
                "plasma_count": (i64, [C.POINTER(OrcPlasma)]),
                "plasma_generate": (C.c_int, [C.POINTER(OrcPlasma), C.c_int32] + [dp] * 7 + [ip]),
                "get_particles_cell": (C.c_int, [vp, ip] + [fp] * 7),
                "charge_density": (C.c_int, [vp, dp]),
                "diagnostics": (C.c_int, [vp, C.c_double, C.POINTER(OrcDiag)]),
            })
        for name, (res, args) in sig.items():
            fn = getattr(lib, p + name)
            fn.restype, fn.argtypes = res, args
        _libs[kind] = (lib, p)
    return _libs[kind]


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def order_by_position(x, y=None, z=None, kind="port"):
    """Indexes of the particles in lexicographic (x, y, z) order, over as many
    coordinates as are given (EnsembleOrdered::reorder, EnsembleOrdered.h:61-71).
    "port": stable (ties in input order); "reference": pica's own std::sort."""
    lib, p = _lib(kind)
    keys = [np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z) if a is not None]
    n = len(keys[0])
    while len(keys) < 3:
        keys.append(keys[0])
    order = np.zeros(n, np.int64)
    dims = sum(a is not None for a in (x, y, z))
    rc = getattr(lib, p + "order_by_position")(n, dims, _dp(keys[0]), _dp(keys[1]), _dp(keys[2]),
                                              order.ctypes.data_as(C.POINTER(C.c_int64)))
    if rc != 0:
        raise RuntimeError(f"order_by_position failed: {rc}")
    return order


def push_flat(n, h, dt, particles, f6, shape=SHAPE_CIC, species=((9.10938215e-28, -4.80320427e-10),), guard=2,
              kind="port"):
    """One push of a flat particle array (pica's EnsembleUnordered with the grid-level
    CIC interpolator and depositor).  particles: dict with x y z ux uy uz w species
    (updated copies are returned); f6: ex ey ez bx by bz.  Returns (particles, j3)."""
    lib, p = _lib(kind)
    cfg = OrcConfig()
    for d in range(3):
        cfg.n[d], cfg.sc[d], cfg.h[d] = int(n[d]), 1, float(h[d])
    cfg.dt, cfg.form, cfg.shape, cfg.deposit = float(dt), FORM_FP64_PLAIN, shape, DEPOSIT_DIRECT
    cfg.nspecies = len(species)
    for i, (m, q) in enumerate(species):
        cfg.mass[i], cfg.charge[i] = m, q
    out = {k: np.array(particles[k], dtype=np.float64) for k in ("x", "y", "z", "ux", "uy", "uz")}
    w = np.ascontiguousarray(particles["w"], dtype=np.float64)
    sp = np.ascontiguousarray(particles.get("species", np.zeros(len(w), np.int32)), dtype=np.int32)
    fs = [np.ascontiguousarray(f, dtype=np.float64).reshape(-1) for f in f6]
    j3 = [np.zeros(int(np.prod(n))) for _ in range(3)]
    fa = (C.POINTER(C.c_double) * 6)(*[_dp(f) for f in fs])
    ja = (C.POINTER(C.c_double) * 3)(*[_dp(j) for j in j3])
    rc = getattr(lib, p + "push_flat")(C.byref(cfg), int(guard), len(w), *[_dp(out[k]) for k in
                                       ("x", "y", "z", "ux", "uy", "uz")], _dp(w), _ip(sp), fa, ja)
    if rc != 0:
        raise RuntimeError(f"push_flat failed: {rc}")
    out["w"], out["species"] = w, sp
    return out, [j.reshape(n) for j in j3]


class Oracle:
    """One CPU simulation.  kind = "port" (restatement) or "reference" (pica headers)."""

    def __init__(self, n, sc, h, dt, form=FORM_FP64_PLAIN, shape=SHAPE_CIC, deposit=DEPOSIT_DIRECT,
                 species=((9.10938215e-28, -4.80320427e-10),), threads=0, kind="port", resort_every=0):
        self.lib, self.p = _lib(kind)
        cfg = OrcConfig()
        for d in range(3):
            cfg.n[d], cfg.sc[d], cfg.h[d] = int(n[d]), int(sc[d]), float(h[d])
        cfg.dt, cfg.form, cfg.shape, cfg.deposit = float(dt), form, shape, deposit
        cfg.nspecies = len(species)
        for i, (m, q) in enumerate(species):
            cfg.mass[i], cfg.charge[i] = m, q
        cfg.threads = threads
        cfg.resort_every = int(resort_every)
        self.cfg = cfg
        self.n = tuple(int(v) for v in n)
        self.nsc = tuple(int(n[d]) // int(sc[d]) for d in range(3))
        self.nspecies = len(species)
        self.h_ = self._f("create")(C.byref(cfg))
        if not self.h_:
            raise ValueError("oracle rejected the configuration")

    def _f(self, name):
        return getattr(self.lib, self.p + name)

    def __del__(self):
        if getattr(self, "h_", None):
            self._f("destroy")(self.h_)
            self.h_ = None

    def load(self, x, y, z, ux, uy, uz, w, species=None):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z, ux, uy, uz, w)]
        sp = None if species is None else np.ascontiguousarray(species, dtype=np.int32)
        rc = self._f("load")(self.h_, len(arrs[0]), *[_dp(a) for a in arrs], None if sp is None else _ip(sp))
        if rc:
            raise RuntimeError(f"load failed: {rc}")

    def set_fields(self, f9):
        arrs = [np.ascontiguousarray(a, dtype=np.float64).reshape(-1) for a in f9]
        ptrs = (C.POINTER(C.c_double) * 9)(*[_dp(a) for a in arrs])
        self._keep = arrs
        if self._f("set_fields")(self.h_, ptrs):
            raise RuntimeError("set_fields failed")

    def get_fields(self):
        out = [np.zeros(self.n, dtype=np.float64) for _ in range(9)]
        ptrs = (C.POINTER(C.c_double) * 9)(*[_dp(a) for a in out])
        if self._f("get_fields")(self.h_, ptrs):
            raise RuntimeError("get_fields failed")
        return out

    def step(self, nsteps=1):
        rc = self._f("step")(self.h_, int(nsteps))
        if rc:
            raise RuntimeError(f"oracle step failed: {rc}")

    def num_particles(self):
        return int(self._f("num_particles")(self.h_))

    def particles(self):
        n = self.num_particles()
        a = [np.zeros(n) for _ in range(7)]
        sp, sc = np.zeros(n, np.int32), np.zeros(n, np.int32)
        if self._f("get_particles")(self.h_, *[_dp(v) for v in a], _ip(sp), _ip(sc)):
            raise RuntimeError("get_particles failed")
        return dict(zip(("x", "y", "z", "ux", "uy", "uz", "w"), a), species=sp, supercell=sc)

    def particles_cell(self):
        n = self.num_particles()
        cell = np.zeros(n, np.int32)
        f = [np.zeros(n, np.float32) for _ in range(7)]
        if self._f("get_particles_cell")(self.h_, _ip(cell), *[_fp(v) for v in f]):
            raise RuntimeError("get_particles_cell failed")
        return dict(zip(("ox", "oy", "oz", "ux", "uy", "uz", "w"), f), cell=cell)

    def counts(self):
        c = np.zeros(self.nspecies * int(np.prod(self.nsc)), np.int32)
        self._f("get_counts")(self.h_, _ip(c))
        return c.reshape(self.nspecies, -1)

    def migrations(self):
        n = int(self._f("num_migrations")(self.h_))
        a = [np.zeros(n, np.int32) for _ in range(4)]
        self._f("get_migrations")(self.h_, *[_ip(v) for v in a])
        return np.stack(a, axis=1)

    def charge_density(self):
        rho = np.zeros(self.n)
        self._f("charge_density")(self.h_, _dp(rho))
        return rho

    def diagnostics(self, bg_density=0.0):
        d = OrcDiag()
        self._f("diagnostics")(self.h_, float(bg_density), C.byref(d))
        return {k: getattr(d, k) for k in ("field_energy", "kinetic_energy", "total_charge", "gauss_max", "rho_max")}
