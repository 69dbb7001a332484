"""Many independent dam breaks advanced together (sphx_batch_*).

``BatchDamBreak(cases)`` sets up every case the way ``DamBreak`` does
(tests/2d_examples/test_2d_dambreak/Dambreak.cpp:56-127: lattice particles of the water
and wall shapes over the system bounds, wall normals from the wall shape, h = 1.3 dp,
the lattice number density, masses rho0 dp^d) and hands the instances to one batched
mixed-precision solver.  ``advection_step`` runs one pass of the Dambreak.cpp:166-220
loop for every instance at once; each instance keeps its own advection dt, acoustic dt,
sub-step count and physical time.  All cases must have the same dimension and the
Dambreak.cpp loop order (acoustic dt before each relaxation).
"""
from __future__ import annotations

import ctypes as C
from typing import List, Sequence

import numpy as np

from . import native as N
from . import sph as S
from .cases import DamBreakCase


class BatchInstance(C.Structure):
    _fields_ = [("mesh", N.MeshDesc), ("n_fluid", C.c_size_t), ("n_wall", C.c_size_t),
                ("fluid_pos", C.c_void_p), ("wall_pos", C.c_void_p), ("wall_normal", C.c_void_p),
                ("h", C.c_double), ("sigma0", C.c_double), ("rho0", C.c_double), ("c0", C.c_double),
                ("U_ref", C.c_double), ("fluid_mass", C.c_double), ("fluid_vol", C.c_double),
                ("wall_rho0", C.c_double), ("wall_mass", C.c_double), ("wall_vol", C.c_double),
                ("gravity", C.c_double * 3)]


def instance_arrays(case: DamBreakCase):
    """Fluid positions, wall positions and wall normals of one case (host arrays)."""
    d = case.dim
    water = S.ComplexShape("WaterBody").add(S.GeometricShapeBox(case.water_center[:d], case.water_halfsize[:d]))
    wall = S.ComplexShape("WallBoundary")
    wall.add(S.GeometricShapeBox(case.outer_center[:d], case.outer_halfsize[:d]))
    wall.subtract(S.GeometricShapeBox(case.inner_center[:d], case.inner_halfsize[:d]))
    fpos = S.lattice_positions(d, case.sys_lower, case.sys_upper, case.dp, water)
    wpos = S.lattice_positions(d, case.sys_lower, case.sys_upper, case.dp, wall)
    wnrm = wall.normal_direction(wpos) if len(wpos) else np.zeros((0, d))
    return (np.ascontiguousarray(fpos, dtype=np.float64), np.ascontiguousarray(wpos, dtype=np.float64),
            np.ascontiguousarray(wnrm, dtype=np.float64))


class BatchDamBreak:
    def __init__(self, cases: Sequence[DamBreakCase], device: int = 0, block: int = 128, use_graph: bool = True):
        cases = list(cases)
        if not cases:
            raise ValueError("empty batch")
        dims = {c.dim for c in cases}
        if len(dims) != 1:
            raise ValueError("all instances of one batch have the same dimension")
        if any(c.loop_style != 0 for c in cases):
            raise ValueError("the batched solver runs the Dambreak.cpp loop order (loop_style 0)")
        self.cases = cases
        self.dim = dims.pop()
        self.ctx = S.default_context(device)
        self.use_graph = bool(use_graph)
        d = self.dim
        keep = []  # host arrays must live until sphx_batch_create returns
        descs = (BatchInstance * len(cases))()
        self.n_fluid: List[int] = []
        for q, case in enumerate(cases):
            fpos, wpos, wnrm = instance_arrays(case)
            keep += [fpos, wpos, wnrm]
            h = case.h_ratio * case.dp
            md = N.MeshDesc()
            lo = np.zeros(3)
            up = np.zeros(3)
            lo[:d] = case.sys_lower[:d]
            up[:d] = case.sys_upper[:d]
            N.call("sphx_mesh_from_bounds", d, S._dptr(lo), S._dptr(up), 2.0 * h, 2, C.byref(md))
            s0 = C.c_double()
            N.call("sphx_lattice_number_density", d, h, case.dp, C.byref(s0))
            vol = case.dp * case.dp * case.dp if d == 3 else case.dp * case.dp
            x = descs[q]
            x.mesh = md
            x.n_fluid, x.n_wall = len(fpos), len(wpos)
            x.fluid_pos, x.wall_pos, x.wall_normal = fpos.ctypes.data, wpos.ctypes.data, wnrm.ctypes.data
            x.h, x.sigma0 = h, s0.value
            x.rho0, x.c0, x.U_ref = case.rho0, case.c0, case.U_ref
            x.fluid_mass, x.fluid_vol = case.rho0 * vol, vol
            x.wall_rho0, x.wall_mass, x.wall_vol = 1.0, 1.0 * vol, vol
            for a in range(3):
                x.gravity[a] = case.gravity[a] if a < d else 0.0
            self.n_fluid.append(len(fpos))
        hb = C.c_void_p()
        N.call("sphx_batch_create", self.ctx.h, d, len(cases), descs, C.byref(hb))
        self.handle = hb
        del keep
        self.set_tuning(block)
        self.count = len(cases)
        self.physical_time = np.zeros(self.count)
        self.substeps = np.zeros(self.count, dtype=np.int64)
        self.number_of_iterations = 0

    def set_tuning(self, block: int) -> None:
        N.call("sphx_batch_set_tuning", self.handle, int(block))

    def set_substep_cap(self, max_substeps: int) -> None:
        """Acoustic sub-steps an instance may take in one advection step before the step
        ends with SPHX_ERR_TIMEOUT (sphx_batch_set_substep_cap)."""
        N.call("sphx_batch_set_substep_cap", self.handle, int(max_substeps))

    def size(self):
        nf, nw = C.c_size_t(), C.c_size_t()
        N.call("sphx_batch_size", self.handle, C.byref(nf), C.byref(nw))
        return nf.value, nw.value

    def graph_launches(self) -> int:
        v = C.c_uint64()
        N.call("sphx_batch_graph_launches", self.handle, C.byref(v))
        return int(v.value)

    def advection_step(self, use_graph: bool = None):
        """One advection step of every instance; returns the sub-steps each took."""
        g = self.use_graph if use_graph is None else bool(use_graph)
        sub = np.zeros(self.count, dtype=np.int32)
        t = np.zeros(self.count)
        N.call("sphx_batch_advection_step", self.handle, int(g), sub.ctypes.data_as(C.POINTER(C.c_int)),
               t.ctypes.data_as(C.POINTER(C.c_double)))
        self.physical_time = t
        self.substeps += sub
        self.number_of_iterations += 1
        return sub

    def download(self, instance: int):
        """(position, velocity, density, pressure) of one instance in its input order."""
        n, d = self.n_fluid[instance], self.dim
        pos, vel = np.zeros((n, d)), np.zeros((n, d))
        rho, p = np.zeros(n), np.zeros(n)
        N.call("sphx_batch_download", self.handle, int(instance), S._dptr(pos), S._dptr(vel), S._dptr(rho),
               S._dptr(p))
        return pos, vel, rho, p

    def __del__(self):
        if getattr(self, "handle", None) is not None and N._lib is not None:
            N._lib.sphx_batch_destroy(self.handle)
            self.handle = None
