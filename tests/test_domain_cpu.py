"""The domain decomposition's exchange protocol on the CPU (pica_gb300.domain).

FakeDomain is a host-memory test double of a slab's device context: the same
field-slab, take and append operations (pica_field_slab, pica_take_supercells,
pica_append_to_supercells) on torch CPU tensors.  Every slab starts with owned
fields that are a known function of the global cell, NaN guards, a known current
in its guard layers, and particles in its guard supercells tagged with their
global cell.  One halo, fold and particle exchange must then leave:

* every guard layer equal to the function at the global cell it stands for;
* the owned current next to each face raised by the neighbour's guard current,
  and, after the current halo, every guard current equal to the completed
  current of the cell it stands for;
* every particle in the owned supercell of the slab that owns its global cell, at
  the local cell that stands for it.

The same checks run in one process (LocalTransport, 1 to 3 slabs) and as gloo
ranks (DistTransport, world sizes 2 and 3: with two slabs one rank is both
neighbours, which is where message order matters).
"""
import os
import socket

import numpy as np
import pytest
import torch

from pica_gb300 import domain

S = 4


def pack(x, y, z):
    return (x << 21) | (y << 10) | z


def unpack(c):
    c = c.astype(np.int64) & 0xFFFFFFFF
    return c >> 21, (c >> 10) & 0x7FF, c & 0x3FF


class FakeDomain:
    """Slab r on host tensors (one species, the FP32 cell form's 8 components)."""

    def __init__(self, plan, r):
        self.plan, self.r, self.nspecies = plan, r, 1
        n = plan.local_n(r)
        self.n, self.layer = n, n[1] * n[2]
        self.f = [torch.zeros(n[0] * self.layer, dtype=torch.float64) for _ in range(9)]
        self.nsc3 = (n[0] // S, n[1] // S, n[2] // S)
        self.parts = [[] for _ in range(int(np.prod(self.nsc3)))]   # per supercell: rows of 8 floats

    def slab(self, comp, x0, nx):
        return self.f[comp][x0 * self.layer:(x0 + nx) * self.layer].clone()

    def put_slab(self, comp, x0, t, add=False):
        seg = self.f[comp][x0 * self.layer:x0 * self.layer + t.numel()]
        if add:
            seg += t
        else:
            seg.copy_(t)

    def take(self, q, b, e):
        rows = [row for s in range(b, e) for row in self.parts[s]]
        counts = np.array([len(self.parts[s]) for s in range(b, e)], np.int32)
        for s in range(b, e):
            self.parts[s] = []
        a = np.array(rows, np.float64).reshape(-1, 8)
        bufs = [torch.tensor(a[:, 0].astype(np.int64).astype(np.int32))] + \
               [torch.tensor(a[:, k].astype(np.float32)) for k in range(1, 8)]
        return counts, bufs

    def append(self, q, b, e, counts, bufs, dx):
        cells = bufs[0].numpy().astype(np.int64)
        cx, cy, cz = unpack(cells)
        cells = pack((cx + dx) % self.n[0], cy, cz)
        cols = [cells.astype(np.float64)] + [t.numpy().astype(np.float64) for t in bufs[1:]]
        o = 0
        for i, c in enumerate(counts):
            for k in range(o, o + int(c)):
                self.parts[b + i].append([col[k] for col in cols])
            o += int(c)


def value(c, gx, rest):
    return 1000.0 * c + gx + 1e-3 * rest


def setup(plan, r):
    d = FakeDomain(plan, r)
    G = plan.G
    for c in range(9):
        a = d.f[c].view(d.n[0], d.layer)
        for l in range(d.n[0]):
            gx = (plan.x0[r] - G + l) % plan.n[0]
            if G <= l < G + plan.w[r]:
                a[l] = torch.tensor(value(c, gx, np.arange(d.layer)))
            elif c >= 6:
                a[l] = 7.0          # current deposited into the guard layers
            else:
                a[l] = float("nan")
    # particles in the guard supercells: two per guard cell column x, tagged with the global cell
    rng = np.random.default_rng(r)
    for l in list(range(G)) + list(range(G + plan.w[r], 2 * G + plan.w[r])):
        gx = (plan.x0[r] - G + l) % plan.n[0]
        for _ in range(2):
            y, z = int(rng.integers(0, d.n[1])), int(rng.integers(0, d.n[2]))
            s = ((l // S) * d.nsc3[1] + y // S) * d.nsc3[2] + z // S
            d.parts[s].append([pack(l, y, z), 0.5, 0.25, 0.75, 0.1, 0.2, 0.3, float(gx)])
    return d


def check(plan, r, d):
    G = plan.G
    for c in range(9):
        a = d.f[c].view(d.n[0], d.layer).numpy()
        for l in range(d.n[0]):
            gx = (plan.x0[r] - G + l) % plan.n[0]
            want = value(c, gx, np.arange(d.layer))
            if c < 6 and (l < G or l >= G + plan.w[r]):
                assert np.array_equal(a[l], want), (r, c, l)          # halo
            if c >= 6 and G <= l < G + plan.w[r]:
                near = l < 2 * G or l >= plan.w[r]
                assert np.array_equal(a[l], want + (7.0 if near else 0.0)), (r, c, l)   # fold
            if c >= 6 and (l < G or l >= G + plan.w[r]):
                assert np.array_equal(a[l], want + 7.0), (r, c, l)    # current halo: the owner's completed value
    got = 0
    for s, rows in enumerate(d.parts):
        sx = s // (d.nsc3[1] * d.nsc3[2])
        for row in rows:
            lx, _, _ = unpack(np.array([int(row[0])]))
            lx = int(lx[0])
            assert G <= lx < G + plan.w[r], (r, lx)                   # an owned cell
            assert lx // S == sx                                      # of this supercell
            assert (plan.x0[r] - G + lx) % plan.n[0] == int(row[7])   # the cell it stood for
            got += 1
    return got


def nx_for(world):
    return 12 * world


def test_plan_index_arithmetic():
    p = domain.SlabPlan((36, 8, 8), S, 3)
    assert p.G == 4 and p.x0 == [0, 12, 24] and p.w == [12, 12, 12]
    assert p.guard_low_sc(1) == (0, 4) and p.guard_high_sc(1) == (16, 20)
    for r in range(3):
        for l in range(p.local_n(r)[0]):
            gx = (p.x0[r] - p.G + l) % 36
            assert p.to_local(p.owner_of(gx), gx) in range(p.G, p.G + p.w[p.owner_of(gx)])
    assert domain.guard_cells(2) == 4 and domain.guard_cells(4) == 4 and domain.guard_cells(8) == 8
    with pytest.raises(ValueError):
        domain.SlabPlan((8, 8, 8), 2, 3)    # slabs of 2 cells, narrower than the 4-cell guard


@pytest.mark.parametrize("slabs", [1, 2, 3])
def test_local_transport_moves_layers_current_and_particles(slabs):
    plan = domain.SlabPlan((nx_for(slabs), 8, 8), S, slabs)
    doms = [setup(plan, r) for r in range(slabs)]
    sent = sum(len(rows) for d in doms for rows in d.parts)
    t = domain.LocalTransport(doms)
    t.halo(plan)
    t.fold(plan)
    t.halo(plan, domain.J)
    t.exchange(plan)
    assert sum(check(plan, r, d) for r, d in enumerate(doms)) == sent


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        plan = domain.SlabPlan((nx_for(world), 8, 8), S, world)
        d = setup(plan, rank)
        sent = sum(len(rows) for rows in d.parts)
        t = domain.DistTransport(d, rank, world, dist)
        t.halo(plan)
        t.fold(plan)
        t.halo(plan, domain.J)
        t.exchange(plan)
        q.put((rank, sent, check(plan, rank, d), None))
    except Exception as e:   # report to the parent
        q.put((rank, 0, 0, repr(e)))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_dist_transport_over_gloo(world):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in ps:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in ps:
        p.join(timeout=60)
    errs = [e for _, _, _, e in res if e]
    assert not errs, errs
    assert sum(s for _, s, _, _ in res) == sum(g for _, _, g, _ in res)
