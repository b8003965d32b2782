"""Slab domain decomposition of one periodic system over ranks, one GPU per rank.

The reference decomposes a system into a regular grid of subdomains and, every step, exchanges halo particles
dimension by dimension with the neighbouring ranks, then migrates particles that left their subdomain
(examples/md-flexible/src/domainDecomposition/RegularGridDecomposition.cpp:159-300).  Here the grid is a row of
slabs along one axis: in that axis a rank's neighbours are the ranks before and after it (periodically); in the
other two axes a rank is its own neighbour, so the exchange there forms the periodic images locally.  The
exchange follows the reference's rules:

* for the neighbour below, the particles within [local_min, local_min + rc + skin) of the axis, and, from the
  halo particles received in earlier dimensions, those within [local_min - skin, local_min + rc + skin); above
  likewise with [local_max - rc - skin, local_max) and [local_max - rc - skin, local_max + skin);
* a particle sent across the global boundary takes the image position x + len (below) or x + (-len) (above),
  one rounding, as md-flexible writes it; between ranks positions travel unchanged;
* migrants (owned particles outside the local box after a step) go to the neighbour in the direction they left,
  wrapped across the global boundary, and the receiver keeps those inside its box.

Transport: `Comm` exchanges host arrays with the two neighbours of the slab axis (torch.distributed point to
point: gloo on CPU ranks, NCCL between GPUs, each rank receiving into its own buffers).  A rank's forces come
from any force function over its owned + halo particles; on a GPU that is the engine with an explicit-halo system
(`engine_forces`), in the tests the CPU oracle.  The decomposition adds no collective on the force path: the only
collective is the sum of the per-rank globals.
"""
from __future__ import annotations

import numpy as np

SELF = -1


def wrap(x, lo, hi):
    """Periodic wrap into [lo, hi) with md-flexible's rule (RegularGridDecomposition.cpp:555-590): x + len below,
    x - len above, and a coordinate that would round onto hi stays just below it."""
    length = hi - lo
    y = np.where(x < lo, x + length, np.where(x >= hi, x - length, x))
    y = np.where(y >= hi, np.nextafter(hi, lo), y)
    return np.where(y < lo, lo, y)


class Comm:
    """Neighbour exchange over torch.distributed (world > 1) or none (world 1)."""

    def __init__(self, dist=None):
        self.dist = dist

    def exchange(self, to_left, to_right, left, right):
        """Sends the float64 arrays to_left / to_right ([k, m] rows) to ranks left / right and returns the rows
        received from them, concatenated (from the left first).  A neighbour equal to SELF gets the rows back."""
        if left == SELF and right == SELF:
            return np.concatenate([to_right, to_left])  # my left neighbour's "to right" is my own "to right"
        import torch
        d = self.dist
        m = to_left.shape[1]
        # tags tell the two directions apart when both neighbours are the same rank (two ranks): what I send to
        # the left is what my left neighbour receives from its right
        T_LEFT, T_RIGHT = 1, 2
        sizes_out = [torch.tensor([len(to_left)], dtype=torch.int64), torch.tensor([len(to_right)], dtype=torch.int64)]
        sizes_in = [torch.zeros(1, dtype=torch.int64), torch.zeros(1, dtype=torch.int64)]
        reqs = [d.isend(sizes_out[0], left, tag=T_LEFT), d.isend(sizes_out[1], right, tag=T_RIGHT),
                d.irecv(sizes_in[0], left, tag=T_RIGHT), d.irecv(sizes_in[1], right, tag=T_LEFT)]
        for r in reqs:
            r.wait()
        n_from_left, n_from_right = int(sizes_in[0].item()), int(sizes_in[1].item())
        buf_left = torch.empty((n_from_left, m), dtype=torch.float64)
        buf_right = torch.empty((n_from_right, m), dtype=torch.float64)
        reqs = []
        if len(to_left):
            reqs.append(d.isend(torch.from_numpy(np.ascontiguousarray(to_left)), left, tag=T_LEFT + 2))
        if len(to_right):
            reqs.append(d.isend(torch.from_numpy(np.ascontiguousarray(to_right)), right, tag=T_RIGHT + 2))
        if n_from_left:
            reqs.append(d.irecv(buf_left, left, tag=T_RIGHT + 2))
        if n_from_right:
            reqs.append(d.irecv(buf_right, right, tag=T_LEFT + 2))
        for r in reqs:
            r.wait()
        return np.concatenate([buf_left.numpy(), buf_right.numpy()])


class SlabDecomposition:
    """The subdomain of `rank` among `world` slabs of the periodic box [gmin, gmax) along `axis`."""

    def __init__(self, rank, world, gmin, gmax, cutoff, skin, axis=0):
        self.rank, self.world, self.axis = rank, world, axis
        self.gmin = np.asarray(gmin, np.float64)
        self.gmax = np.asarray(gmax, np.float64)
        self.len = self.gmax - self.gmin
        self.cutoff, self.skin = float(cutoff), float(skin)
        self.lmin = self.gmin.copy()
        self.lmax = self.gmax.copy()
        w = self.len[axis] / world
        self.lmin[axis] = self.gmin[axis] + rank * w
        self.lmax[axis] = self.gmax[axis] if rank == world - 1 else self.gmin[axis] + (rank + 1) * w
        if world > 1 and w < cutoff + skin:
            raise ValueError(f"slab width {w} is below the interaction length {cutoff + skin}")

    def neighbours(self, dim):
        if dim != self.axis or self.world == 1:
            return SELF, SELF
        return (self.rank - 1) % self.world, (self.rank + 1) % self.world

    def inside(self, pos):
        return np.all((pos >= self.lmin) & (pos < self.lmax), axis=1)

    def exchange_halos(self, comm, owned):
        """Halo rows for the owned rows [k, m] (columns 0..2 the position, the rest carried along, e.g. the
        global id and the type).  Returns the halo rows, dimension by dimension as the reference collects them."""
        L = self.cutoff + self.skin
        halos = np.zeros((0, owned.shape[1]))
        for d in range(3):
            lo, hi = self.lmin[d], self.lmax[d]
            at_gmin, at_gmax = lo == self.gmin[d], hi == self.gmax[d]
            x_own, x_halo = owned[:, d], halos[:, d]
            to_l = np.concatenate([owned[(x_own >= lo) & (x_own < lo + L)],
                                   halos[(x_halo >= lo - self.skin) & (x_halo < lo + L)]])
            to_r = np.concatenate([owned[(x_own >= hi - L) & (x_own < hi)],
                                   halos[~((x_halo >= lo - self.skin) & (x_halo < lo + L)) &
                                         (x_halo >= hi - L) & (x_halo < hi + self.skin)]])
            # the boundary condition at the global faces: x + len (below), x + (-len) (above), one rounding
            if at_gmin and len(to_l):
                to_l = to_l.copy()
                to_l[:, d] = to_l[:, d] + self.len[d]
            if at_gmax and len(to_r):
                to_r = to_r.copy()
                to_r[:, d] = to_r[:, d] + (-self.len[d])
            left, right = self.neighbours(d)
            halos = np.concatenate([halos, comm.exchange(to_l, to_r, left, right)])
        return halos

    def migrate(self, comm, owned):
        """Owned rows after a step: the rows outside the local box go to the neighbour they moved towards, wrapped
        at the global faces (RegularGridDecomposition.cpp:238-300; the wrap of ...:555-590).  Returns the rows
        this rank owns afterwards."""
        keep = owned
        for d in range(3):
            x = keep[:, d]
            lo, hi = self.lmin[d], self.lmax[d]
            below, above = x < lo, x >= hi
            to_l, to_r = keep[below].copy(), keep[above].copy()
            keep = keep[~(below | above)]
            for rows in (to_l, to_r):
                if len(rows):
                    rows[:, d] = wrap(rows[:, d], self.gmin[d], self.gmax[d])
            left, right = self.neighbours(d)
            got = comm.exchange(to_l, to_r, left, right)
            keep = np.concatenate([keep, got])
        if len(keep) and not np.all(self.inside(keep[:, :3])):
            raise RuntimeError(f"rank {self.rank}: particles moved further than one subdomain in one step")
        return keep


def engine_forces(engine_module, cutoff, skin, lmin, lmax, precision=1, **kw):
    """A force function on the GPU engine: one explicit-halo system over the local box [lmin, lmax), owned + halo
    particles uploaded as AutoPas containers receive them.  Returns f(owned_pos, halo_pos) -> (F_owned, globals)
    with globals = (Upot, virial, interacting pairs as the container counts them: owned-owned pairs plus every
    owned-halo pair once; a pair across a rank boundary is thus counted on both ranks)."""
    def f(owned_pos, halo_pos):
        e = engine_module.PairEngine(cutoff, skin, (lmin, lmax), periodic=False, precision=precision, **kw)
        allpos = np.concatenate([owned_pos, halo_pos])
        own = np.concatenate([np.ones(len(owned_pos), np.int8), np.full(len(halo_pos), 2, np.int8)])
        e.set_particles(allpos, ownership=own)
        g = e.compute_forces()[0]
        F = e.forces()[: len(owned_pos)]
        e.close()
        return F, np.array([g["upot"], g["virial"], float(g["num_pairs"])])
    return f


def oracle_forces(orc, cutoff):
    """The same interface on the CPU oracle (FP64, explicit halos): for tests.  Its pair count is the rank's share of
    the unique pairs (owned-owned plus half the owned-halo pairs), which sums over the ranks to the system's count."""
    lj = orc.LJ(cutoff)

    def f(owned_pos, halo_pos):
        allpos = np.concatenate([owned_pos, halo_pos])
        own = np.concatenate([np.ones(len(owned_pos), np.int8), np.full(len(halo_pos), 2, np.int8)])
        R, glob, _ = orc.lj_forces(allpos, lj, own=own)
        oo, oh, _ = orc.count_interacting(allpos, cutoff, own=own)
        return R[: len(owned_pos)], np.array([glob[0], glob[1], oo + oh / 2.0])
    return f


def step_velocity_verlet(rows, forces_fn, dec, comm, dt, mass=1.0):
    """One velocity-Verlet step of a rank's owned rows [k, 3 pos | 3 vel | 3 force | id] with md-flexible's order
    (TimeDiscretization.cpp:17-66, 152-164): positions, migration, halo exchange, forces, velocities."""
    pos, vel, F = rows[:, 0:3], rows[:, 3:6], rows[:, 6:9]
    pos = pos + vel * dt + F * (dt * dt / (2 * mass))
    rows = np.concatenate([pos, vel, F, rows[:, 9:]], axis=1)
    rows = dec.migrate(comm, rows)
    halos = dec.exchange_halos(comm, rows[:, [0, 1, 2, 9]])
    Fn, glob = forces_fn(rows[:, 0:3], halos[:, 0:3])
    vel = rows[:, 3:6] + (Fn + rows[:, 6:9]) * (dt / (2 * mass))
    return np.concatenate([rows[:, 0:3], vel, Fn, rows[:, 9:]], axis=1), glob
