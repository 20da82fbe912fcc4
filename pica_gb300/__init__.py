"""pica_gb300: pica's particle-in-cell step on one GB300 (sm_103a).

Host-side mirror of pica's operator API for the hot path.  pica drives
per-particle objects (YeeGrid, YeeSolver, FieldInterpolatorCIC[Supercell],
BorisPusher, CurrentDepositorCIC[Supercell], EnsembleSupercells); here one
``Simulation`` owns the device-resident grid and supercell ensemble and each
operator call advances every particle at once through the C ABI
(include/pica_gb300.h).  The compute runs only in the CUDA library; there is
no CPU fallback.
"""
import ctypes as C

import numpy as np

from ._lib import PicaConfig, PicaDiag, PicaPlasmaSpec, load

FORM_FP64_PLAIN, FORM_FP32_CELL = 0, 1
SHAPE_CIC, SHAPE_TSC = 1, 2
DEPOSIT_DIRECT, DEPOSIT_ESIRKEPOV = 0, 1

# pica math/Constants.h:10-14 (CGS; pi truncated as in the reference)
PI = 3.14159265358
LIGHT_VELOCITY = 29979245800.0
ELECTRON_CHARGE = -4.80320427e-10
ELECTRON_MASS = 9.10938215e-28

ELECTRON = (ELECTRON_MASS, ELECTRON_CHARGE)


class PicaError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"pica_gb300 error {status}: {message}")
        self.status = status


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


class Simulation:
    """A periodic Yee grid plus a supercell ensemble of particles on the GPU.

    Arguments mirror pica: ``n`` = YeeGrid size in cells, ``h`` = step,
    ``supercell`` = EnsembleSupercells numCellsPerSupercell, ``species`` =
    the ParticleTypes table as (mass, charge) pairs, ``dt`` = BorisPusher dt.
    """

    def __init__(self, n, h, dt, supercell=(2, 2, 2), form=FORM_FP64_PLAIN, shape=SHAPE_CIC,
                 deposit=DEPOSIT_DIRECT, species=(ELECTRON,), slack=0.15, resort_every=0, threads=0):
        self.lib = load()
        self._describe(make_config(n, h, dt, supercell, form, shape, deposit, species, slack, resort_every, threads))
        handle = C.c_void_p()
        rc = self.lib.pica_ctx_create(C.byref(self.cfg), C.byref(handle))
        if rc:
            raise PicaError(rc, self.lib.pica_status_string(rc).decode())
        self.ctx = handle
        self._owned = True

    def _describe(self, cfg):
        self.cfg = cfg
        self.n = tuple(int(cfg.n[d]) for d in range(3))
        self.h = tuple(float(cfg.h[d]) for d in range(3))
        self.dt = float(cfg.dt)
        self.form = int(cfg.form)
        self.nsc = tuple(self.n[d] // int(cfg.sc[d]) for d in range(3))
        self.nspecies = int(cfg.nspecies)
        self.species = tuple((cfg.mass[i], cfg.charge[i]) for i in range(self.nspecies))

    @classmethod
    def _member(cls, lib, handle, cfg):
        """A context owned by a Batch (not destroyed by close())."""
        self = cls.__new__(cls)
        self.lib = lib
        self._describe(cfg)
        self.ctx = C.c_void_p(handle)
        self._owned = False
        return self

    # -- lifetime ------------------------------------------------------------
    def close(self):
        if getattr(self, "ctx", None):
            if getattr(self, "_owned", True):
                self.lib.pica_ctx_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc:
            raise PicaError(rc, self.lib.pica_last_error(self.ctx).decode() or self.lib.pica_status_string(rc).decode())

    def set_stream(self, stream_ptr):
        """Enqueue all work on this cudaStream_t (an int, e.g. torch.cuda.current_stream().cuda_stream)."""
        self._check(self.lib.pica_set_stream(self.ctx, C.c_void_p(int(stream_ptr))))

    def synchronize(self):
        self._check(self.lib.pica_synchronize(self.ctx))

    def launch_count(self):
        return int(self.lib.pica_launch_count(self.ctx))

    def set_variant(self, variant):
        """Launch shape of the FP32 charge-conserving push kernel (see pica_gb300.autotune)."""
        self._check(self.lib.pica_set_variant(self.ctx, int(variant)))

    def variant(self):
        v, n = C.c_int32(), C.c_int32()
        self._check(self.lib.pica_get_variant(self.ctx, C.byref(v), C.byref(n)))
        return v.value, n.value

    # -- data ----------------------------------------------------------------
    def upload_particles(self, x, y, z, ux, uy, uz, w, species=None):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z, ux, uy, uz, w)]
        sp = None if species is None else np.ascontiguousarray(species, dtype=np.int32)
        self._check(self.lib.pica_upload_particles(self.ctx, len(arrs[0]), *[_dp(a) for a in arrs],
                                                   None if sp is None else _ip(sp)))

    def generate_plasma(self, specs):
        """Synthetic plasma drawn on the device (FP32 cell form) in place of an upload:
        ``specs`` are ``plasma_spec`` populations on this grid (see pica_generate_plasma)."""
        if isinstance(specs, PicaPlasmaSpec):
            specs = [specs]
        arr = (PicaPlasmaSpec * len(specs))(*specs)
        self._check(self.lib.pica_generate_plasma(self.ctx, arr, len(specs)))

    def num_particles(self):
        n = int(self.lib.pica_num_particles(self.ctx))
        if n < 0:
            self._check(n)
        return n

    def particles(self):
        """Particles in ensemble order (species, supercell, slot) as a dict of arrays."""
        n = self.num_particles()
        a = [np.empty(n) for _ in range(7)]
        sp, sc = np.empty(n, np.int32), np.empty(n, np.int32)
        self._check(self.lib.pica_download_particles(self.ctx, *[_dp(v) for v in a], _ip(sp), _ip(sc)))
        return dict(zip(("x", "y", "z", "ux", "uy", "uz", "w"), a), species=sp, supercell=sc)

    def counts(self):
        c = np.empty(self.nspecies * int(np.prod(self.nsc)), np.int32)
        self._check(self.lib.pica_get_counts(self.ctx, _ip(c)))
        return c.reshape(self.nspecies, -1)

    def record_migrations(self, enable=True):
        """Keep each step's migration list (pica_record_migrations)."""
        self._check(self.lib.pica_record_migrations(self.ctx, int(bool(enable))))

    def migrations(self):
        """The last recorded step's moves as an (m, 4) int32 array of (species, source
        supercell, source slot, destination supercell), ordered by species, source, slot."""
        m = int(self.lib.pica_num_migrations(self.ctx))
        if m < 0:
            self._check(m)
        cols = [np.empty(m, np.int32) for _ in range(4)]
        self._check(self.lib.pica_get_migrations(self.ctx, *[_ip(c) for c in cols]))
        return np.stack(cols, axis=1) if m else np.zeros((0, 4), np.int32)

    def upload_fields(self, f9):
        arrs = [np.ascontiguousarray(a, dtype=np.float64).reshape(-1) for a in f9]
        ptrs = (C.POINTER(C.c_double) * 9)(*[_dp(a) for a in arrs])
        self._check(self.lib.pica_upload_fields(self.ctx, ptrs))

    def fields(self):
        """[ex, ey, ez, bx, by, bz, jx, jy, jz] as (nx, ny, nz) float64 arrays."""
        out = [np.empty(self.n) for _ in range(9)]
        ptrs = (C.POINTER(C.c_double) * 9)(*[_dp(a) for a in out])
        self._check(self.lib.pica_download_fields(self.ctx, ptrs))
        return out

    # -- operators -------------------------------------------------------------
    def push_deposit(self):
        """FieldInterpolator::get + BorisPusher::push + CurrentDepositor::deposit for every particle."""
        self._check(self.lib.pica_push_deposit(self.ctx))

    def update_b(self, dt):
        """YeeSolver::updateB(grid, dt) on the periodic grid."""
        self._check(self.lib.pica_update_b(self.ctx, float(dt)))

    def update_e(self, dt):
        """YeeSolver::updateE(grid, dt) on the periodic grid."""
        self._check(self.lib.pica_update_e(self.ctx, float(dt)))

    def migrate(self):
        """Periodic wrap and supercell re-binning after push_deposit."""
        self._check(self.lib.pica_migrate(self.ctx))

    def step(self, nsteps=1):
        self._check(self.lib.pica_step(self.ctx, int(nsteps)))

    # -- diagnostics -----------------------------------------------------------
    def diagnostics(self, bg_density=0.0):
        d = PicaDiag()
        self._check(self.lib.pica_diagnostics(self.ctx, float(bg_density), C.byref(d)))
        return {k: getattr(d, k) for k in ("field_energy", "kinetic_energy", "total_charge", "gauss_max", "rho_max")}

    def charge_density(self):
        rho = np.empty(self.n)
        self._check(self.lib.pica_charge_density(self.ctx, _dp(rho)))
        return rho

    def field_energy(self):
        v = C.c_double()
        self._check(self.lib.pica_field_energy(self.ctx, C.byref(v)))
        return v.value

    # -- checkpoints ---------------------------------------------------------------
    def step_count(self):
        return int(self.lib.pica_step_count(self.ctx))

    def save_checkpoint(self, path):
        """Complete state between steps; a Simulation of the same configuration loaded
        from it continues like this one (FP32 form: bit for bit; FP64 form: to the
        rounding of the FP64 atomic current sums)."""
        self._check(self.lib.pica_checkpoint_save(self.ctx, str(path).encode()))

    def load_checkpoint(self, path):
        self._check(self.lib.pica_checkpoint_load(self.ctx, str(path).encode()))

    # -- raw device state (host loops that keep the state in host memory) ------
    def state_slots(self, species=0):
        return int(self.lib.pica_state_slots(self.ctx, int(species)))

    def state_copy(self, species, comp, host_ptr, to_device):
        self._check(self.lib.pica_state_copy(self.ctx, int(species), int(comp), C.c_void_p(int(host_ptr)),
                                             1 if to_device else 0))

    def state_packed_slots(self, species=0):
        """Lay out the packed state image (used slots only) and return its size in slots."""
        n = int(self.lib.pica_state_packed_slots(self.ctx, int(species)))
        if n < 0:
            self._check(n)
        return n

    def state_copy_range(self, species, comp, host_ptr, to_device, sc_range, copy_stream=None):
        """Raw slots of the supercells ``sc_range=(begin, end)`` (slack included, one
        contiguous copy at the same offset of host_ptr as on the device; no kernel),
        on ``copy_stream`` ordered against the context stream (pica_state_copy_range_on)."""
        self._check(self.lib.pica_state_copy_range_on(self.ctx, int(species), int(comp), C.c_void_p(int(host_ptr)),
                                                      1 if to_device else 0, int(sc_range[0]), int(sc_range[1]),
                                                      C.c_void_p(int(copy_stream)) if copy_stream else None))

    def state_copy_packed(self, species, comp, host_ptr, to_device, sc_range=None, copy_stream=None):
        """One component of the packed image; ``sc_range=(begin, end)``: only the part of
        those supercells (host_ptr is still the start of the whole image).  ``copy_stream``
        (a cudaStream_t as an int): the host copy goes on that stream, the gather / scatter
        kernel stays on the context stream (pica_state_copy_packed_range_on)."""
        if copy_stream is not None:
            b, e = sc_range if sc_range is not None else (0, int(np.prod(self.nsc)))
            self._check(self.lib.pica_state_copy_packed_range_on(self.ctx, int(species), int(comp),
                                                                 C.c_void_p(int(host_ptr)), 1 if to_device else 0,
                                                                 int(b), int(e), C.c_void_p(int(copy_stream))))
        elif sc_range is None:
            self._check(self.lib.pica_state_copy_packed(self.ctx, int(species), int(comp), C.c_void_p(int(host_ptr)),
                                                        1 if to_device else 0))
        else:
            self._check(self.lib.pica_state_copy_packed_range(self.ctx, int(species), int(comp),
                                                              C.c_void_p(int(host_ptr)), 1 if to_device else 0,
                                                              int(sc_range[0]), int(sc_range[1])))

    def reorder(self):
        """Sort every supercell by cell now (EnsembleOrdered::reorder's role)."""
        self._check(self.lib.pica_reorder(self.ctx))

    def push_flat(self, x, y, z, ux, uy, uz, w, species=None, guard=2):
        """One push of a flat particle array on this context's fields (pica_push_flat):
        float64 CUDA tensors of one length (positions and momenta updated in place),
        species an int32 CUDA tensor or None; J is replaced by the array's current.
        FP64 plain form with direct deposition only."""
        ts = (x, y, z, ux, uy, uz, w)
        n = int(x.numel())
        for t in ts:
            if not (t.is_cuda and t.dtype.itemsize == 8 and t.is_contiguous() and t.numel() == n):
                raise ValueError("flat arrays: contiguous float64 CUDA tensors of one length")
        if species is not None and not (species.is_cuda and species.dtype.itemsize == 4 and species.numel() == n):
            raise ValueError("species: an int32 CUDA tensor of the same length")
        ptrs = [C.c_void_p(t.data_ptr()) for t in ts]
        sp = C.c_void_p(species.data_ptr()) if species is not None else None
        self._check(self.lib.pica_push_flat(self.ctx, n, *ptrs, sp, int(guard)))

    def chunk_ranges(self, nchunks):
        """Supercell ranges of pica_push_deposit_chunked: [n r / nchunks, n (r+1) / nchunks)."""
        return supercell_ranges(int(np.prod(self.nsc)), nchunks)

    def push_deposit_chunked(self, wait_events):
        """pica_push_deposit in len(wait_events) supercell ranges, range r launched after
        a wait for wait_events[r] (cudaEvent_t handles as ints, or None)."""
        arr = (C.c_void_p * len(wait_events))(*[C.c_void_p(int(e)) if e else None for e in wait_events])
        self._check(self.lib.pica_push_deposit_chunked(self.ctx, len(wait_events), arr))

    def edge_split_ranges(self, nchunks, split):
        """chunk_ranges(nchunks) with the first and the last range each cut into `split`
        equal pieces: the ranges of a host loop that keeps the link busy at the ends of
        a step (the first download and the last upload and push are short)."""
        return supercell_ranges(int(np.prod(self.nsc)), nchunks, split)

    def push_deposit_ranges(self, ranges, wait_events):
        """pica_push_deposit over the consecutive supercell ranges ``[(begin, end), ...]``
        (covering every supercell once, in order), range r launched after a wait for
        wait_events[r] (pica_push_deposit_ranges)."""
        if len(ranges) != len(wait_events):
            raise ValueError("one wait event (or None) per range")
        bounds = (C.c_int32 * (len(ranges) + 1))(*([int(r[0]) for r in ranges] + [int(ranges[-1][1])]))
        for (b0, e0), (b1, _) in zip(ranges, ranges[1:]):
            if e0 != b1:
                raise ValueError("ranges must be consecutive")
        arr = (C.c_void_p * len(wait_events))(*[C.c_void_p(int(e)) if e else None for e in wait_events])
        self._check(self.lib.pica_push_deposit_ranges(self.ctx, len(ranges), bounds, arr))


def order_by_position(x, y=None, z=None, stream=0):
    """EnsembleOrdered::reorder's order on the device (pica_order_by_position): an
    int64 CUDA tensor of indexes that sorts the particles lexicographically by the
    given coordinates (float64 CUDA tensors), ties in input order."""
    import torch

    keys = [t for t in (x, y, z) if t is not None]
    n = int(keys[0].numel())
    for t in keys:
        if not (t.is_cuda and t.dtype == torch.float64 and t.is_contiguous() and t.numel() == n):
            raise ValueError("positions: contiguous float64 CUDA tensors of one length")
    order = torch.empty(n, dtype=torch.int64, device=keys[0].device)
    p = [C.c_void_p(t.data_ptr()) for t in keys] + [None] * (3 - len(keys))
    rc = load().pica_order_by_position(n, len(keys), p[0], p[1], p[2], C.c_void_p(order.data_ptr()),
                                       C.c_void_p(int(stream)) if stream else None)
    if rc:
        raise PicaError(rc, load().pica_status_string(rc).decode())
    return order


class FlatEnsemble:
    """pica's EnsembleUnordered (particles/EnsembleUnordered.h:14-40) on the device:
    one flat SoA array of FP64 particles in insertion order, pushed by one thread per
    particle on a Simulation's fields (FP64 plain form, direct deposition), with
    ``reorder()`` as EnsembleOrdered::reorder (EnsembleOrdered.h:61-71).

    The grid-level gather and deposit see the Simulation's periodic grid as a pica
    YeeGrid whose origin is ``-guard`` cells (``guard`` = 2 as in pica's supercell
    helpers).  Tensors are float64 (x y z ux uy uz w) and int32 (species)."""

    KEYS = ("x", "y", "z", "ux", "uy", "uz", "w")

    def __init__(self, sim, guard=2):
        import torch

        if sim.form != FORM_FP64_PLAIN:
            raise ValueError("flat ensembles hold FP64 positions: an FP64 plain-form Simulation")
        self.sim, self.guard = sim, int(guard)
        dev = torch.device("cuda", torch.cuda.current_device())
        self.t = {k: torch.empty(0, dtype=torch.float64, device=dev) for k in self.KEYS}
        self.species = torch.empty(0, dtype=torch.int32, device=dev)
        L = [sim.n[d] * sim.h[d] for d in range(3)]
        self.min_position, self.max_position = (0.0, 0.0, 0.0), tuple(L)

    def size(self):
        return int(self.t["x"].numel())

    def add(self, x, y, z, ux, uy, uz, w, species=None):
        """Append particles (EnsembleUnordered::add): host arrays or tensors."""
        import torch

        dev = self.t["x"].device
        new = [torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64)).to(dev) for a in (x, y, z, ux, uy, uz, w)]
        sp = np.zeros(len(x), np.int32) if species is None else np.ascontiguousarray(species, dtype=np.int32)
        for k, a in zip(self.KEYS, new):
            self.t[k] = torch.cat([self.t[k], a])
        self.species = torch.cat([self.species, torch.as_tensor(sp).to(dev)])

    def particles(self):
        """The array in its current order (EnsembleUnordered::getParticles)."""
        out = {k: v.cpu().numpy() for k, v in self.t.items()}
        out["species"] = self.species.cpu().numpy()
        return out

    def reorder(self):
        """EnsembleOrdered::reorder: sort by position (x, then y, then z), stably."""
        order = order_by_position(self.t["x"], self.t["y"], self.t["z"])
        for k in self.KEYS:
            self.t[k] = self.t[k][order].contiguous()
        self.species = self.species[order].contiguous()
        return order

    def push(self):
        """Gather, Boris push and direct deposit of every particle (J replaced)."""
        self.sim.push_flat(*[self.t[k] for k in self.KEYS], self.species, guard=self.guard)

    def step(self, nsteps=1):
        """push; update_b(dt/2); update_e(dt); update_b(dt/2) -- pica's step order."""
        for _ in range(int(nsteps)):
            self.push()
            self.sim.update_b(0.5 * self.sim.dt)
            self.sim.update_e(self.sim.dt)
            self.sim.update_b(0.5 * self.sim.dt)


class Driver:
    """A host loop over a Simulation, in the role of the PICADOR driver around pica's
    kernels: steps in chunks, takes the FP64 diagnostics every ``diag_every`` steps
    and writes a checkpoint every ``checkpoint_every`` steps (``checkpoint_path`` may
    hold ``{step}``).  Boundaries are periodic (the only kind the step supports).
    ``run`` returns the diagnostics records [(step, dict), ...]; ``on_diag(step, d)``
    is called for each as well."""

    def __init__(self, sim, diag_every=0, checkpoint_every=0, checkpoint_path=None, bg_density=0.0, on_diag=None):
        if checkpoint_every and not checkpoint_path:
            raise ValueError("checkpoint_every needs checkpoint_path")
        self.sim = sim
        self.diag_every = int(diag_every)
        self.checkpoint_every = int(checkpoint_every)
        self.checkpoint_path = checkpoint_path
        self.bg = float(bg_density)
        self.on_diag = on_diag
        self.checkpoints = []

    @property
    def step(self):
        return self.sim.step_count()

    def _next_event(self, step):
        nxt = []
        for every in (self.diag_every, self.checkpoint_every):
            if every > 0:
                nxt.append((step // every + 1) * every)
        return min(nxt) if nxt else None

    def run(self, nsteps):
        records = []
        end = self.step + int(nsteps)
        if self.diag_every > 0 and self.step % self.diag_every == 0:
            records.append((self.step, self.sim.diagnostics(self.bg)))
        while self.step < end:
            nxt = self._next_event(self.step)
            target = end if nxt is None else min(nxt, end)
            self.sim.step(target - self.step)
            s = self.step
            if self.diag_every > 0 and s % self.diag_every == 0:
                d = self.sim.diagnostics(self.bg)
                records.append((s, d))
                if self.on_diag:
                    self.on_diag(s, d)
            if self.checkpoint_every > 0 and s % self.checkpoint_every == 0:
                path = str(self.checkpoint_path).format(step=s)
                self.sim.save_checkpoint(path)
                self.checkpoints.append(path)
        return records


def make_config(n, h, dt, supercell=(2, 2, 2), form=FORM_FP64_PLAIN, shape=SHAPE_CIC, deposit=DEPOSIT_DIRECT,
                species=(ELECTRON,), slack=0.15, resort_every=0, threads=0):
    """pica_config for the given grid (cells n, step h), time step and supercell edges."""
    cfg = PicaConfig()
    for d in range(3):
        cfg.n[d], cfg.sc[d], cfg.h[d] = int(n[d]), int(supercell[d]), float(h[d])
    cfg.dt, cfg.form, cfg.shape, cfg.deposit = float(dt), int(form), int(shape), int(deposit)
    cfg.nspecies = len(species)
    for i, (m, q) in enumerate(species):
        cfg.mass[i], cfg.charge[i] = float(m), float(q)
    cfg.slack, cfg.resort_every, cfg.threads = float(slack), int(resort_every), int(threads)
    return cfg


class Batch:
    """Many independent plasmas advanced together (the batching form, FP32 cell form
    with Esirkepov deposition): one persistent push launch over every member's
    supercells and the device part of the step replayed as a CUDA graph.
    ``members`` is a list of Simulation keyword dicts (n, h, dt, supercell, shape,
    species, resort_every, ...); ``batch.members[k]`` is a Simulation view of member k
    for uploads, downloads and diagnostics."""

    def __init__(self, members):
        self.lib = load()
        cfgs = (PicaConfig * len(members))()
        for k, m in enumerate(members):
            kw = dict(m)
            kw.setdefault("form", FORM_FP32_CELL)
            kw.setdefault("deposit", DEPOSIT_ESIRKEPOV)
            cfgs[k] = make_config(**kw)
        handle = C.c_void_p()
        rc = self.lib.pica_batch_create(cfgs, len(members), C.byref(handle))
        if rc:
            raise PicaError(rc, self.lib.pica_status_string(rc).decode())
        self.batch = handle
        self.members = [Simulation._member(self.lib, self.lib.pica_batch_member(handle, k), cfgs[k])
                        for k in range(len(members))]

    def _check(self, rc):
        if rc:
            raise PicaError(rc, self.lib.pica_batch_last_error(self.batch).decode() or
                            self.lib.pica_status_string(rc).decode())

    def set_options(self, use_graph=True, variant=0):
        self._check(self.lib.pica_batch_set_options(self.batch, 1 if use_graph else 0, int(variant)))

    def step(self, nsteps=1):
        self._check(self.lib.pica_batch_step(self.batch, int(nsteps)))

    def stats(self):
        out = (C.c_int64 * 4)()
        self._check(self.lib.pica_batch_stats(self.batch, out))
        return dict(captures=out[0], graph_launches=out[1], kernel_launches=out[2], steps=out[3])

    def reorder(self):
        """Recompute the work order from the members' particle counts at the next step
        (after uploads through ``members``)."""
        for k in range(len(self.members)):
            self.lib.pica_batch_member(self.batch, k)

    def num_particles(self):
        return sum(m.num_particles() for m in self.members)

    def close(self):
        if getattr(self, "batch", None):
            for m in self.members:
                m.ctx = None
            self.lib.pica_batch_destroy(self.batch)
            self.batch = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def plasma_spec(n, h, ppc, sigma_u, weight, seed, species=0, density_mod=0.0, nbeams=1, drift_u=0.0, drift_axis=0):
    s = PicaPlasmaSpec()
    for d in range(3):
        s.n[d], s.h[d] = int(n[d]), float(h[d])
    s.species, s.ppc, s.density_mod = int(species), float(ppc), float(density_mod)
    s.drift_u, s.sigma_u, s.weight, s.seed = float(drift_u), float(sigma_u), float(weight), int(seed)
    s.nbeams, s.drift_axis = int(nbeams), int(drift_axis)
    return s


def supercell_ranges(total, nchunks, edge_split=1):
    """Consecutive supercell ranges [(begin, end), ...] covering 0..total: the nchunks
    ranges [total r / nchunks, total (r+1) / nchunks) of pica_push_deposit_chunked, with
    the first and the last cut into edge_split equal pieces when edge_split > 1."""
    if nchunks < 1 or total < 0:
        raise ValueError("nchunks >= 1 and total >= 0")
    out = []
    for r in range(nchunks):
        b, e = total * r // nchunks, total * (r + 1) // nchunks
        k = edge_split if (r == 0 or r == nchunks - 1) and edge_split > 1 else 1
        out += [(b + (e - b) * i // k, b + (e - b) * (i + 1) // k) for i in range(k)]
    return out


def plasma_count(spec):
    """Particles that `spec` (a plasma_spec) draws, computed on the host."""
    n = int(load().pica_plasma_count(C.byref(spec)))
    if n < 0:
        raise PicaError(n, "bad plasma spec")
    return n


def generate_plasma(spec, threads=0):
    """Synthetic plasma on the host (counter-based RNG; independent of thread count)."""
    lib = load()
    n = int(lib.pica_plasma_count(C.byref(spec)))
    if n < 0:
        raise PicaError(n, "bad plasma spec")
    a = [np.empty(n) for _ in range(7)]
    sp = np.empty(n, np.int32)
    rc = lib.pica_plasma_generate(C.byref(spec), int(threads), *[_dp(v) for v in a], _ip(sp))
    if rc:
        raise PicaError(rc, "plasma generation failed")
    return dict(zip(("x", "y", "z", "ux", "uy", "uz", "w"), a), species=sp)
