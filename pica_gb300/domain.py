"""One periodic plasma split into slabs along x (domain decomposition).

pica reserves the fields of a domain decomposition (Parameters.h:16-27) and lists
one as planned (README.md:21); it has none.  Here a plasma of N = (nx, ny, nz)
cells is cut along x into D slabs of whole supercells.  Slab r owns the global
cells [x0[r], x1[r]) and runs as one pica context whose grid also holds G guard
cells on both x faces: local cell l is global cell x0[r] - G + l (mod nx), the
owned cells are local [G, G + w[r]).  G is the smallest multiple of the supercell
edge that is at least 3, so that

* the gather of an owned supercell (nodes m-1 .. m+S+1) and its current deposit
  (nodes m-2 .. m+S+2) stay inside the slab's grid;
* the Yee update (B dt/2, E dt, B dt/2) leaves the owned fields exact: the local
  grid is periodic, so each of the three stencil passes spoils at most one more
  layer from the far guard inwards (two layers per face in all), never an owned one.

A step of every slab:

1. halo: each slab's E and B guard layers are filled from the owned layers of the
   neighbour that owns those cells (its top G owned layers below, its bottom G
   above);
2. push and deposit (pica_push_deposit);
3. current fold: the current a slab deposited into its guard layers is added to
   the owned layers of the neighbour that owns them; then the current halo copies
   the completed owned current back into the neighbours' guard layers.  The guard
   current is needed within the step: the E update of a guard layer feeds the
   second B half step of the owned layer next to it;
4. B dt/2, E dt, B dt/2 and the migration, each slab on its own;
5. particle exchange: the particles that migrated into a slab's guard supercells
   are taken out (pica_take_supercells) and appended to the neighbour's supercells
   at the same global place (pica_append_to_supercells, cell x shifted into the
   neighbour's frame).  Guard supercells line up one to one with the neighbour's
   owned supercells, so the particles of a guard supercell go to exactly one
   supercell, in slot order: the exchange is deterministic.

The exchange of steps 1, 3 and 5 goes through a transport: Local (every slab a
context in this process, e.g. on one GPU: device-to-device copies) or Dist (one
slab per rank, torch.distributed point-to-point messages between neighbours;
NCCL for device buffers, gloo for host buffers).  No collective is needed on the
data path; diagnostics sums are the only all-reduce.
"""
import ctypes as C

import numpy as np

E_B = (0, 1, 2, 3, 4, 5)
J = (6, 7, 8)


def guard_cells(S):
    """Smallest multiple of the supercell edge S that is at least 3."""
    return S * ((3 + S - 1) // S)


class SlabPlan:
    """Index arithmetic of the decomposition of nx cells (supercell edge S) into D slabs."""

    def __init__(self, n, S, domains, guard=None):
        nx = int(n[0])
        if nx % S:
            raise ValueError("the x extent must be a multiple of the supercell edge")
        nsx = nx // S
        if domains < 1 or domains > nsx:
            raise ValueError("1 <= domains <= supercell columns")
        self.n, self.S, self.D = tuple(int(v) for v in n), int(S), int(domains)
        self.G = int(guard) if guard is not None else guard_cells(S)
        if self.G % S or self.G < 3:
            raise ValueError("the guard must be a multiple of the supercell edge and at least 3 cells")
        self.x0 = [S * (nsx * r // domains) for r in range(domains)]
        self.x1 = self.x0[1:] + [nx]
        self.w = [b - a for a, b in zip(self.x0, self.x1)]
        if min(self.w) < self.G:
            raise ValueError(f"every slab needs at least {self.G} cells (the guard width)")
        self.layer_sc = (self.n[1] // S) * (self.n[2] // S)   # supercells per x-supercell column

    def local_n(self, r):
        return (self.w[r] + 2 * self.G, self.n[1], self.n[2])

    def low(self, r):
        return (r - 1) % self.D

    def high(self, r):
        return (r + 1) % self.D

    # --- fields: runs of x-layers in local indices ---
    def halo_low(self, r):
        """(layers of the low neighbour that fill slab r's low guard, r's low guard start)."""
        return self.w[self.low(r)], 0

    def halo_high(self, r):
        """(layers of the high neighbour that fill slab r's high guard, r's high guard start)."""
        return self.G, self.G + self.w[r]

    # --- particles: supercell ranges (linear index, x-supercell slowest) ---
    def guard_low_sc(self, r):
        return 0, (self.G // self.S) * self.layer_sc

    def guard_high_sc(self, r):
        a = (self.G + self.w[r]) // self.S * self.layer_sc
        return a, a + (self.G // self.S) * self.layer_sc

    def to_low(self, r):
        """Slab r's low guard supercells go to the low neighbour: (its first supercell, dx cells)."""
        q = self.low(r)
        return self.w[q] // self.S * self.layer_sc, self.w[q]

    def to_high(self, r):
        """Slab r's high guard supercells go to the high neighbour: (its first supercell, dx cells)."""
        return (self.G // self.S) * self.layer_sc, -self.w[r]

    def owner_of(self, gx):
        """Slab that owns global cell gx."""
        gx %= self.n[0]
        for r in range(self.D):
            if self.x0[r] <= gx < self.x1[r]:
                return r
        raise ValueError(gx)

    def to_local(self, r, gx):
        """Local cell index in slab r of global cell gx (owned or guard)."""
        return (gx - self.x0[r] + self.G) % self.n[0] if self.D > 1 else gx + self.G


class GPUDomain:
    """Slab r as a pica context on this process's GPU (device buffers are torch tensors)."""

    def __init__(self, plan, r, sim_kwargs):
        import torch

        from . import Simulation
        self.torch = torch
        self.plan, self.r = plan, r
        kw = dict(sim_kwargs)
        kw["n"] = plan.local_n(r)
        self.sim = Simulation(**kw)
        self.lib = self.sim.lib
        self.fp64 = self.sim.form == 0
        self.dtype = torch.float64 if self.fp64 else torch.float32
        self.ncomp = 7 if self.fp64 else 8
        self.comp_dtype = [torch.float64] * 7 if self.fp64 else [torch.int32] + [torch.float32] * 7
        self.nspecies = self.sim.nspecies
        self.layer = plan.n[1] * plan.n[2]

    def _check(self, rc):
        self.sim._check(rc)

    def slab(self, comp, x0, nx):
        t = self.torch.empty(nx * self.layer, dtype=self.dtype, device="cuda")
        self._check(self.lib.pica_field_slab(self.sim.ctx, comp, x0, nx, C.c_void_p(t.data_ptr()), 0))
        return t

    def put_slab(self, comp, x0, t, add=False):
        nx = t.numel() // self.layer
        self._check(self.lib.pica_field_slab(self.sim.ctx, comp, x0, nx, C.c_void_p(t.data_ptr()), 2 if add else 1))

    def take(self, species, b, e):
        m = e - b
        counts = np.zeros(m, np.int32)
        cp = counts.ctypes.data_as(C.POINTER(C.c_int32))
        tot = int(self.lib.pica_take_supercells(self.sim.ctx, species, b, e, None, 0, cp))
        if tot < 0:
            self._check(tot)
        bufs = [self.torch.empty(max(tot, 1), dtype=dt, device="cuda") for dt in self.comp_dtype]
        ptrs = (C.c_void_p * self.ncomp)(*[t.data_ptr() for t in bufs])
        got = int(self.lib.pica_take_supercells(self.sim.ctx, species, b, e, ptrs, tot, cp))
        if got < 0:
            self._check(got)
        return counts, [t[:tot] for t in bufs]

    def append(self, species, b, e, counts, bufs, dx):
        counts = np.ascontiguousarray(counts, np.int32)
        if int(counts.sum()) == 0:
            return
        ptrs = (C.c_void_p * self.ncomp)(*[t.data_ptr() for t in bufs])
        rc = self.lib.pica_append_to_supercells(self.sim.ctx, species, b, e,
                                                counts.ctypes.data_as(C.POINTER(C.c_int32)), ptrs, dx)
        if rc == -4:   # PICA_ERR_OVERFLOW: re-upload the ensemble with the arrivals, from the host
            self._reupload_with(species, bufs, dx)
        else:
            self._check(rc)

    def _reupload_with(self, species, bufs, dx):
        p = self.sim.particles()
        h = self.sim.h
        comps = [t.cpu().numpy() for t in bufs]
        if self.fp64:
            xs = [comps[0] + dx * h[0], comps[1], comps[2]]
            us, w = comps[3:6], comps[6]
        else:
            cell = comps[0].view(np.uint32).astype(np.int64)
            cx, cy, cz = (cell >> 21) + dx, (cell >> 10) & 0x7FF, cell & 0x3FF
            xs = [(cx + comps[1]) * h[0], (cy + comps[2]) * h[1], (cz + comps[3]) * h[2]]
            us, w = comps[4:7], comps[7]
        n = len(w)
        keys = ("x", "y", "z", "ux", "uy", "uz", "w")
        merged = {k: np.concatenate([p[k], np.asarray(v, np.float64)]) for k, v in zip(keys, xs + list(us) + [w])}
        sp = np.concatenate([p["species"], np.full(n, species, np.int32)])
        self.sim.upload_particles(*[merged[k] for k in keys], sp)

    def synchronize(self):
        self.sim.synchronize()


class LocalTransport:
    """Every slab in this process: neighbours' buffers are reached directly."""

    def __init__(self, domains):
        self.domains = domains

    def halo(self, plan, comps=E_B):
        for r, d in enumerate(self.domains):
            lo, hi = self.domains[plan.low(r)], self.domains[plan.high(r)]
            src_lo, dst_lo = plan.halo_low(r)
            src_hi, dst_hi = plan.halo_high(r)
            for c in comps:
                d.put_slab(c, dst_lo, lo.slab(c, src_lo, plan.G))
                d.put_slab(c, dst_hi, hi.slab(c, src_hi, plan.G))

    def fold(self, plan):
        guards = []
        for r, d in enumerate(self.domains):   # read every guard before any owned layer changes
            guards.append([(d.slab(c, 0, plan.G), d.slab(c, plan.G + plan.w[r], plan.G)) for c in J])
        for r in range(len(self.domains)):
            lo, hi = self.domains[plan.low(r)], self.domains[plan.high(r)]
            for c, (gl, gh) in zip(J, guards[r]):
                lo.put_slab(c, plan.w[plan.low(r)], gl, add=True)
                hi.put_slab(c, plan.G, gh, add=True)

    def exchange(self, plan):
        moves = []
        for r, d in enumerate(self.domains):   # take everything first: a guard range may feed a slab we append to
            for q in range(d.nspecies):
                b, e = plan.guard_low_sc(r)
                moves.append((plan.low(r), q, plan.to_low(r), e - b, d.take(q, b, e)))
                b, e = plan.guard_high_sc(r)
                moves.append((plan.high(r), q, plan.to_high(r), e - b, d.take(q, b, e)))
        for dst, q, (first, dx), m, (counts, bufs) in moves:
            self.domains[dst].append(q, first, first + m, counts, bufs, dx)


class DistTransport:
    """One slab per rank: point-to-point messages with the two neighbours
    (torch.distributed; NCCL for device buffers, gloo for host buffers)."""

    def __init__(self, domain, rank, world, dist):
        self.d, self.r, self.world, self.dist = domain, rank, world, dist

    def _sendrecv(self, plan, send_lo, send_hi, recv_lo, recv_hi):
        """Send send_lo to the low neighbour and send_hi to the high one; receive into
        recv_lo (what the low neighbour sends to its high neighbour) and recv_hi (what
        the high neighbour sends to its low one).  Messages between two ranks match in
        the order they are posted: every rank posts its sends low then high, and its
        receives high then low, so that with two slabs (one rank is both neighbours)
        the first message from the peer, meant for its low neighbour, lands in recv_hi."""
        dist, lo, hi = self.dist, plan.low(self.r), plan.high(self.r)
        ops = []
        for t in send_lo:
            ops.append(dist.P2POp(dist.isend, t, lo))
        for t in send_hi:
            ops.append(dist.P2POp(dist.isend, t, hi))
        for t in recv_hi:
            ops.append(dist.P2POp(dist.irecv, t, hi))
        for t in recv_lo:
            ops.append(dist.P2POp(dist.irecv, t, lo))
        if ops:
            for w in dist.batch_isend_irecv(ops):
                w.wait()

    def halo(self, plan, comps=E_B):
        d, r, G = self.d, self.r, plan.G
        send_lo = [d.slab(c, G, G) for c in comps]                  # my bottom owned layers -> low neighbour's high guard
        send_hi = [d.slab(c, plan.w[r], G) for c in comps]          # my top owned layers -> high neighbour's low guard
        recv_lo = [d.slab(c, 0, G) for c in comps]                  # buffers of the right size
        recv_hi = [d.slab(c, G + plan.w[r], G) for c in comps]
        self._sendrecv(plan, send_lo, send_hi, recv_lo, recv_hi)
        for c, t in zip(comps, recv_lo):
            d.put_slab(c, 0, t)
        for c, t in zip(comps, recv_hi):
            d.put_slab(c, G + plan.w[r], t)

    def fold(self, plan):
        d, r, G = self.d, self.r, plan.G
        send_lo = [d.slab(c, 0, G) for c in J]                    # my low guard current -> low neighbour's top layers
        send_hi = [d.slab(c, G + plan.w[r], G) for c in J]        # my high guard current -> high neighbour's bottom
        recv_lo = [d.slab(c, G, G) for c in J]                    # from the low neighbour's high guard
        recv_hi = [d.slab(c, plan.w[r], G) for c in J]            # from the high neighbour's low guard
        self._sendrecv(plan, send_lo, send_hi, recv_lo, recv_hi)
        for c, t in zip(J, recv_lo):
            d.put_slab(c, G, t, add=True)
        for c, t in zip(J, recv_hi):
            d.put_slab(c, plan.w[r], t, add=True)

    def exchange(self, plan):
        import torch
        d, r = self.d, self.r
        for q in range(d.nspecies):
            bl, el = plan.guard_low_sc(r)
            bh, eh = plan.guard_high_sc(r)
            cl, tl = d.take(q, bl, el)
            ch, th = d.take(q, bh, eh)
            m = el - bl
            dev = tl[0].device
            # counts first (the receiver sizes its buffers), then the packed components
            rcl, rch = torch.zeros(m, dtype=torch.int32, device=dev), torch.zeros(m, dtype=torch.int32, device=dev)
            self._sendrecv(plan, [torch.as_tensor(cl, device=dev)], [torch.as_tensor(ch, device=dev)], [rcl], [rch])
            nl, nh = int(rcl.sum()), int(rch.sum())
            bufs_l = [torch.empty(nl, dtype=t.dtype, device=dev) for t in tl]
            bufs_h = [torch.empty(nh, dtype=t.dtype, device=dev) for t in th]
            self._sendrecv(plan, [t for t in tl if t.numel()] if int(cl.sum()) else [],
                           [t for t in th if t.numel()] if int(ch.sum()) else [],
                           bufs_l if nl else [], bufs_h if nh else [])
            # from the low neighbour: its high guard -> my bottom owned supercells
            first, _ = plan.to_high(plan.low(r))
            d.append(q, first, first + m, rcl.cpu().numpy(), bufs_l, -plan.w[plan.low(r)])
            # from the high neighbour: its low guard -> my top owned supercells
            first, _ = plan.to_low(plan.high(r))
            d.append(q, first, first + m, rch.cpu().numpy(), bufs_h, plan.w[r])


class SlabDecomposition:
    """A periodic plasma of n cells stepped as D slabs (contexts) with guard layers.
    `transport` is LocalTransport (all slabs here) or DistTransport (one per rank)."""

    def __init__(self, plan, domains, transport, dt):
        self.plan, self.domains, self.t, self.dt = plan, domains, transport, float(dt)

    def step(self, n=1):
        for _ in range(n):
            self.t.halo(self.plan)
            for d in self.domains:
                d.sim.push_deposit()
            self.t.fold(self.plan)
            self.t.halo(self.plan, J)   # the completed current back into the guard layers
            for d in self.domains:
                d.sim.update_b(0.5 * self.dt)
                d.sim.update_e(self.dt)
                d.sim.update_b(0.5 * self.dt)
                d.sim.migrate()
            self.t.exchange(self.plan)


def local_decomposition(n, h, dt, supercell, domains, **sim_kwargs):
    """D slab contexts of one plasma in this process (one GPU)."""
    plan = SlabPlan(n, supercell[0], domains)
    kw = dict(sim_kwargs, h=h, dt=dt, supercell=supercell)
    doms = [GPUDomain(plan, r, kw) for r in range(domains)]
    return SlabDecomposition(plan, doms, LocalTransport(doms), dt)


def split_particles(plan, p, h0):
    """Route global particles (dict of x y z ux uy uz w species, positions in [0, L),
    cell size h0 along x) to the slabs: per slab the particles it owns, x moved into
    its local frame."""
    cx = np.floor(p["x"] / h0).astype(np.int64) % plan.n[0]
    out = []
    for r in range(plan.D):
        sel = (cx >= plan.x0[r]) & (cx < plan.x1[r])
        q = {k: v[sel] for k, v in p.items()}
        q["x"] = q["x"] + (plan.G - plan.x0[r]) * h0
        out.append(q)
    return out


def split_fields(plan, f9):
    """Global N^3 field arrays to each slab's local arrays (guards included, filled
    with the neighbours' values)."""
    out = []
    for r in range(plan.D):
        idx = [(plan.x0[r] - plan.G + l) % plan.n[0] for l in range(plan.local_n(r)[0])]
        out.append([np.ascontiguousarray(np.asarray(a)[idx]) for a in f9])
    return out


def gather_fields(plan, per_slab):
    """Each slab's owned layers back into global N^3 arrays."""
    out = [np.empty(plan.n) for _ in range(9)]
    for r, f in enumerate(per_slab):
        for c in range(9):
            out[c][plan.x0[r]:plan.x1[r]] = np.asarray(f[c])[plan.G:plan.G + plan.w[r]]
    return out
