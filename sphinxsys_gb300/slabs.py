"""Slab decomposition of one dam break over several ranks, one GPU per rank.

The fluid is split along one axis into slabs whose boundaries lie on cell boundaries and
balance the fluid particle count at set-up.  A rank owns the fluid particles inside its
slab, holds copies ("ghosts") of its neighbours' particles within one cut-off radius of
the slab, and the wall particles within one cut-off radius of the slab.  One advection
step follows Dambreak.cpp:166-220:

* Dt: every rank takes AdvectionTimeStep over its particles (owned and ghost copies of
  owned particles elsewhere, so the global maximum is the maximum over ranks) and the
  ranks agree on the smallest Dt (all-reduce min; the formula falls as the maximum rises);
* DensitySummationComplexFreeSurface, then the ghosts' densities from their owners;
* acoustic sub-steps: dt the same way; Integration1stHalf, then the ghosts' force,
  density rate and velocity from their owners; Integration2ndHalf, then the ghosts'
  force, density rate and density;
* particles that left their slab move to the neighbour, new ghost sets are drawn, cell
  lists and relations are rebuilt.

Ghosts are exact copies wherever a neighbour reads them: the pointwise parts of both
halves (density and pressure initialisation, position half-steps) recompute them bit for
bit from exchanged inputs, the neighbour sums come from their owners.  Owned particles
therefore see the same neighbours and values as in a single-rank run; only the order of
each neighbour sum differs (local particle order), i.e. rounding.

The exchange is host-staged: rows of the device state are read into host buffers, sent
point to point with torch.distributed (CPU tensors: a gloo group), and written into the
receivers' ghost rows.  Nothing on a device waits for another rank.  Particles may move at
most one slab per advection step (checked), the Morton re-sort of the single-rank loop is
not applied (it only permutes particles).

The per-rank arithmetic is a backend with the interface of ``CudaSlabBackend`` (the FP64
drop-in on this rank's GPU); tests also drive the decomposition with the CPU oracle.
"""
from __future__ import annotations

import math
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import sph as S
from .cases import DamBreakCase

# fluid variables a rank sends with a migrating or ghost particle, and their widths
# (d = vector of the dimension)
STATE = ("Position", "Velocity", "Force", "ForcePrior", "Density", "Pressure", "DensityChangeRate", "Mass",
         "VolumetricMeasure")
VECTORS = ("Position", "Velocity", "Force", "ForcePrior")
AFTER_DENSITY = ("Density",)
AFTER_FIRST_HALF = ("Force", "DensityChangeRate", "Velocity")
AFTER_SECOND_HALF = ("Force", "DensityChangeRate", "Density")


def balanced_splits(x: np.ndarray, world: int, lower: float, upper: float, grid_spacing: float) -> np.ndarray:
    """Slab boundaries (world + 1 values, the outer ones at the domain bounds) at cell
    boundaries of the mesh, each inner one at the cell boundary nearest to the particle
    count quantile; every slab is at least two cells wide."""
    b = np.empty(world + 1)
    b[0], b[-1] = lower, upper
    xs = np.sort(np.asarray(x, dtype=np.float64))
    for r in range(1, world):
        q = xs[min(len(xs) - 1, (len(xs) * r) // world)] if len(xs) else lower + (upper - lower) * r / world
        k = round((q - lower) / grid_spacing)
        b[r] = lower + k * grid_spacing
    for r in range(1, world + 1):
        if b[r] - b[r - 1] < 2.0 * grid_spacing - 1e-12:
            raise ValueError("slabs narrower than two cells: fewer ranks or a finer case")
    return b


def owner_of(x: np.ndarray, bounds: np.ndarray) -> np.ndarray:
    """Rank owning each coordinate: slab r holds bounds[r] <= x < bounds[r + 1] (the outer
    slabs extend to infinity, like the clamped cell hash)."""
    return np.clip(np.searchsorted(bounds[1:-1], x, side="right"), 0, len(bounds) - 2)


def pack(state: Dict[str, np.ndarray], names: Sequence[str], rows=None) -> np.ndarray:
    cols = []
    for nm in names:
        a = state[nm] if rows is None else state[nm][rows]
        cols.append(a.reshape(a.shape[0], int(np.prod(a.shape[1:], dtype=np.int64))))
    return np.ascontiguousarray(np.concatenate(cols, axis=1)) if cols else np.zeros((0, 0))


def unpack(block: np.ndarray, names: Sequence[str], dim: int) -> Dict[str, np.ndarray]:
    out, c = {}, 0
    for nm in names:
        w = dim if nm in VECTORS else 1
        a = block[:, c:c + w]
        out[nm] = np.ascontiguousarray(a if w > 1 else a[:, 0])
        c += w
    return out


def width(names: Sequence[str], dim: int) -> int:
    return sum(dim if nm in VECTORS else 1 for nm in names)


class Comm:
    """Point-to-point and all-reduce on CPU tensors (a gloo process group)."""

    def __init__(self, group=None):
        import torch
        import torch.distributed as dist
        self.torch, self.dist, self.group = torch, dist, group
        self.rank = dist.get_rank(group)
        self.world = dist.get_world_size(group)

    def global_rank(self, r: int) -> int:
        return r if self.group is None else self.dist.get_global_rank(self.group, r)

    def min(self, v: float) -> float:
        t = self.torch.tensor([v], dtype=self.torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MIN, group=self.group)
        return float(t[0])

    def sendrecv(self, sends: Dict[int, np.ndarray], recv_shapes: Dict[int, tuple]) -> Dict[int, np.ndarray]:
        """Sends arrays to peers and receives arrays of known shapes (float64); empty
        transfers are skipped on both sides."""
        torch, dist = self.torch, self.dist
        reqs, outs = [], {}
        for peer, shape in recv_shapes.items():
            buf = torch.empty(shape, dtype=torch.float64)
            outs[peer] = buf
            if buf.numel():
                reqs.append(dist.irecv(buf, src=self.global_rank(peer), group=self.group))
        keep = []
        for peer, arr in sends.items():
            t = torch.from_numpy(np.ascontiguousarray(arr, dtype=np.float64))
            keep.append(t)
            if t.numel():
                reqs.append(dist.isend(t, dst=self.global_rank(peer), group=self.group))
        for q in reqs:
            q.wait()
        return {p: b.numpy() for p, b in outs.items()}

    def counts(self, sends: Dict[int, int]) -> Dict[int, int]:
        """Exchanges one integer with each peer."""
        got = self.sendrecv({p: np.array([float(v)]) for p, v in sends.items()}, {p: (1,) for p in sends})
        return {p: int(v[0]) for p, v in got.items()}

    def gather_objects(self, obj) -> List:
        out = [None] * self.world
        self.dist.all_gather_object(out, obj, group=self.group)
        return out


class CudaSlabBackend:
    """One rank's particles on its GPU through the FP64 drop-in (sph.py objects)."""

    def __init__(self, case: DamBreakCase, device: int = 0):
        d = case.dim
        self.case, self.dim = case, d
        self.system = S.SPHSystem(case.sys_lower[:d], case.sys_upper[:d], case.dp, device=device,
                                  h_spacing_ratio=case.h_ratio)
        self.wall = None
        self.fluid = None

    def set_wall(self, pos: np.ndarray, normal: np.ndarray) -> None:
        w = S.SolidBody(self.system, None, name="WallBoundary")
        w.defineMatterMaterial(S.Solid())
        w.generateParticles(positions=pos)
        if w.n:
            w.upload("NormalDirection", normal)
        w.updateCellLinkedList()
        self.wall = w

    def load(self, state: Dict[str, np.ndarray]) -> None:
        """Replaces the fluid body by these particles (owned rows first, then ghosts) and
        builds its cell list and relations."""
        c = self.case
        if self.fluid is not None:
            self.system.bodies.remove(self.fluid)
        f = S.FluidBody(self.system, None, name="WaterBody")
        f.defineMatterMaterial(S.WeaklyCompressibleFluid(c.rho0, c.c0))
        f.generateParticles(positions=state["Position"])
        self.fluid = f
        self.inner = S.InnerRelation(f)
        self.contact = S.ContactRelation(f, [self.wall])
        self.first = S.Dynamics1Level(S.Integration1stHalfWithWallRiemann, self.inner, self.contact)
        self.second = S.Dynamics1Level(S.Integration2ndHalfWithWallRiemann, self.inner, self.contact)
        self.density = S.InteractionWithUpdate(S.DensitySummationComplexFreeSurface, self.inner, self.contact)
        self.acoustic = S.ReduceDynamics(S.AcousticTimeStep, f)
        self.advection = S.ReduceDynamics(S.AdvectionTimeStep, f, c.U_ref)
        for nm in STATE:
            if nm != "Position" and f.n:
                f.upload(nm, state[nm])
        f.updateCellLinkedList()
        self.inner.updateConfiguration()
        self.contact.updateConfiguration()

    @property
    def n(self) -> int:
        return self.fluid.n

    def get(self, name: str, first: int, count: int) -> np.ndarray:
        return self.fluid.download_rows(name, first, count)

    def set(self, name: str, values: np.ndarray, first: int) -> None:
        self.fluid.upload_rows(name, values, first)

    def density_summation(self) -> None:
        self.density.exec()

    def first_half(self, dt: float) -> None:
        self.first.exec(dt)

    def second_half(self, dt: float) -> None:
        self.second.exec(dt)

    def acoustic_dt(self) -> float:
        return self.acoustic.exec() if self.fluid.n else math.inf

    def advection_dt(self) -> float:
        return self.advection.exec() if self.fluid.n else math.inf


class SlabDamBreak:
    """The dam break of ``case`` split over the ranks of ``comm`` along ``axis``."""

    def __init__(self, case: DamBreakCase, backend, comm: Comm, axis: int = 0):
        from .batch import instance_arrays
        self.case, self.backend, self.comm, self.axis = case, backend, comm, axis
        d = case.dim
        self.dim = d
        self.rc = 2.0 * case.h_ratio * case.dp
        fpos, wpos, wnrm = instance_arrays(case)  # same arrays on every rank
        md = self._mesh()
        lower = md[0][axis]
        upper = lower + md[1] * md[2][axis]
        self.bounds = balanced_splits(fpos[:, axis], comm.world, lower, upper, md[1])
        r = comm.rank
        self.lo, self.hi = self.bounds[r], self.bounds[r + 1]
        # walls within one cut-off of the slab (static)
        wx = wpos[:, axis]
        wsel = self._near(wx, self.rc)
        backend.set_wall(wpos[wsel], wnrm[wsel])
        # owned fluid at rest (Dambreak.cpp set-up: rho0, gravity as the prior force)
        own = owner_of(fpos[:, axis], self.bounds) == r
        n = int(own.sum())
        vol = case.dp * case.dp * case.dp if d == 3 else case.dp * case.dp
        g = np.array(case.gravity[:d], dtype=np.float64)
        m = case.rho0 * vol
        self.state = {
            "Position": fpos[own].copy(), "Velocity": np.zeros((n, d)), "Force": np.zeros((n, d)),
            "ForcePrior": np.tile(m * g, (n, 1)), "Density": np.full(n, case.rho0), "Pressure": np.zeros(n),
            "DensityChangeRate": np.zeros(n), "Mass": np.full(n, m), "VolumetricMeasure": np.full(n, vol)}
        self.gid = np.nonzero(own)[0].astype(np.int64)
        self.physical_time = 0.0
        self.number_of_iterations = 0
        self.migrated = 0  # particles this rank handed to a neighbour so far
        self._configure()

    def _mesh(self):
        import ctypes as C
        from . import native as N
        c, d = self.case, self.dim
        lo, up = np.zeros(3), np.zeros(3)
        lo[:d], up[:d] = c.sys_lower[:d], c.sys_upper[:d]
        md = N.MeshDesc()
        N.call("sphx_mesh_from_bounds", d, S._dptr(lo), S._dptr(up), self.rc, 2, C.byref(md))
        return list(md.lower), md.grid_spacing, list(md.all_cells)

    def _near(self, x: np.ndarray, w: float) -> np.ndarray:
        lo = -np.inf if self.comm.rank == 0 else self.lo - w
        hi = np.inf if self.comm.rank == self.comm.world - 1 else self.hi + w
        return (x >= lo) & (x < hi)

    def _peers(self) -> List[int]:
        r, w = self.comm.rank, self.comm.world
        return [p for p in (r - 1, r + 1) if 0 <= p < w]

    # -------------------------------------------------------------- configuration update
    def _configure(self) -> None:
        """Ghost sets from the owned state, then the local body.  Owned rows are ordered
        [sent to the lower neighbour | interior | sent to the upper neighbour] (each part by
        global id) so that every exchange reads two contiguous row ranges; the ghosts follow,
        those of the lower neighbour first, each in their owner's order."""
        d, ax, rc = self.dim, self.axis, self.rc
        r = self.comm.rank
        x = self.state["Position"][:, ax]
        lower = (x < self.lo + rc) if r > 0 else np.zeros(len(x), dtype=bool)
        upper = (x >= self.hi - rc) if r < self.comm.world - 1 else np.zeros(len(x), dtype=bool)
        cat = np.where(lower, 0, np.where(upper, 2, 1))
        order = np.lexsort((self.gid, cat))
        self.gid = self.gid[order]
        self.state = {nm: v[order] for nm, v in self.state.items()}
        self.n_owned = n = len(self.gid)
        n_lo, n_up = int(lower.sum()), int(upper.sum())
        self.ghost_send = {}
        if r > 0:
            self.ghost_send[r - 1] = (0, n_lo)
        if r < self.comm.world - 1:
            self.ghost_send[r + 1] = (n - n_up, n_up)
        counts = self.comm.counts({p: cnt for p, (_, cnt) in self.ghost_send.items()})
        wd = width(STATE, d) + 1
        sends = {p: np.concatenate([pack(self.state, STATE, slice(f, f + c)),
                                    self.gid[f:f + c, None].astype(np.float64)], axis=1)
                 for p, (f, c) in self.ghost_send.items()}
        got = self.comm.sendrecv(sends, {p: (counts[p], wd) for p in counts})
        local = {nm: [self.state[nm]] for nm in STATE}
        self.ghost_rows, self.ghost_gid = {}, []
        start = n
        for p in sorted(got):
            blk = got[p]
            for nm, v in unpack(blk[:, :-1], STATE, d).items():
                local[nm].append(v)
            self.ghost_rows[p] = (start, len(blk))
            self.ghost_gid.append(blk[:, -1].astype(np.int64))
            start += len(blk)
        self.backend.load({nm: np.concatenate(v) for nm, v in local.items()})

    def _exchange(self, names: Sequence[str]) -> None:
        """Refreshes the ghost rows of these variables from their owners."""
        d = self.dim
        sends = {}
        for p, (first, cnt) in self.ghost_send.items():
            own = {nm: self.backend.get(nm, first, cnt) for nm in names}
            sends[p] = pack(own, names)
        got = self.comm.sendrecv(sends, {p: (cnt, width(names, d)) for p, (_, cnt) in self.ghost_rows.items()})
        for p, blk in got.items():
            first, cnt = self.ghost_rows[p]
            if cnt:
                for nm, vals in unpack(blk, names, d).items():
                    self.backend.set(nm, vals, first)

    def _migrate(self) -> None:
        """Owned particles that left the slab go to the neighbour that owns them now."""
        d, ax = self.dim, self.axis
        st = {nm: self.backend.get(nm, 0, self.n_owned) for nm in STATE}
        x = st["Position"][:, ax]
        dest = owner_of(x, self.bounds)
        r = self.comm.rank
        if np.any(np.abs(dest - r) > 1):
            raise RuntimeError("a particle moved more than one slab in one advection step")
        leave = {p: np.nonzero(dest == p)[0] for p in self._peers()}
        self.migrated += sum(len(v) for v in leave.values())
        counts = self.comm.counts({p: len(v) for p, v in leave.items()})
        wd = width(STATE, d) + 1
        sends = {p: np.concatenate([pack(st, STATE, rows), self.gid[rows, None].astype(np.float64)], axis=1)
                 for p, rows in leave.items()}
        got = self.comm.sendrecv(sends, {p: (counts[p], wd) for p in counts})
        stay = dest == r
        parts = {nm: [st[nm][stay]] for nm in STATE}
        gids = [self.gid[stay]]
        for p in sorted(got):
            blk = got[p]
            for nm, v in unpack(blk[:, :-1], STATE, d).items():
                parts[nm].append(v)
            gids.append(blk[:, -1].astype(np.int64))
        gid = np.concatenate(gids)
        order = np.argsort(gid, kind="stable")
        self.gid = gid[order]
        self.state = {nm: np.concatenate(v)[order] for nm, v in parts.items()}

    # -------------------------------------------------------------- the loop
    def advection_step(self) -> int:
        """One pass of the Dambreak.cpp loop on every rank; returns the acoustic sub-steps."""
        b, comm = self.backend, self.comm
        Dt = comm.min(b.advection_dt())
        b.density_summation()
        self._exchange(AFTER_DENSITY)
        relaxation, sub = 0.0, 0
        while relaxation < Dt:
            dt = comm.min(b.acoustic_dt())
            b.first_half(dt)
            self._exchange(AFTER_FIRST_HALF)
            b.second_half(dt)
            self._exchange(AFTER_SECOND_HALF)
            relaxation += dt
            self.physical_time += dt
            sub += 1
        self.number_of_iterations += 1
        self._migrate()
        self._configure()
        return sub

    def gather(self, names: Sequence[str] = ("Position", "Velocity", "Density", "Pressure")):
        """All ranks' owned particles, ordered by global id (every rank gets the result)."""
        mine = (self.gid, {nm: self.backend.get(nm, 0, self.n_owned) for nm in names})
        parts = self.comm.gather_objects(mine)
        gid = np.concatenate([p[0] for p in parts])
        order = np.argsort(gid)
        return gid[order], {nm: np.concatenate([p[1][nm] for p in parts])[order] for nm in names}
