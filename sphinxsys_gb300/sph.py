"""Host-side mirror of SPHinXsys' call-site API on the CUDA execution policy.

The names and argument meanings follow the reference so a driver reads like
tests/2d_examples/test_2d_dambreak/Dambreak.cpp: ``SPHSystem``, ``FluidBody`` /
``SolidBody`` / ``ObserverBody``, ``GeometricShapeBox`` / ``ComplexShape``,
``InnerRelation`` / ``ContactRelation`` / ``ComplexRelation`` and the dynamics wrappers
``Dynamics1Level``, ``InteractionWithUpdate``, ``ReduceDynamics``, ``SimpleDynamics``,
``ParticleSorting``.  Every ``exec`` calls the C ABI of libsphx_cuda.so on the device
arrays of the bodies (``execution::CudaDevicePolicy``); errors raise ``SphxError``
instead of the reference's ``exit(1)``.

Particle generation (the lattice generator and the box shapes) runs on the host, in
numpy, before the particles are handed to the device, as the reference generates its
particles on the host before any device copy.
"""
from __future__ import annotations

import ctypes as C
import math
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import native as N


class CudaDevicePolicy:
    """Execution-policy tag of this library (stands beside ParallelDevicePolicy)."""


par_cuda = CudaDevicePolicy()

_contexts: Dict[int, "Context"] = {}


class Context:
    """A device and the stream every call of this library is enqueued on."""

    def __init__(self, device: int = 0, stream: int = 0):
        h = C.c_void_p()
        N.call("sphx_ctx_create", int(device), C.c_void_p(stream), C.byref(h))
        self.h = h
        self.device = device

    def synchronize(self) -> None:
        N.call("sphx_ctx_synchronize", self.h)

    def launch_count(self) -> int:
        v = C.c_uint64()
        N.call("sphx_ctx_launch_count", self.h, C.byref(v))
        return int(v.value)

    def stream(self) -> int:
        s = C.c_void_p()
        N.call("sphx_ctx_stream", self.h, C.byref(s))
        return int(s.value or 0)

    def __del__(self):
        if getattr(self, "h", None) is not None and N._lib is not None:
            N._lib.sphx_ctx_destroy(self.h)
            self.h = None


def default_context(device: int = 0) -> Context:
    if device not in _contexts:
        _contexts[device] = Context(device)
    return _contexts[device]


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


# ------------------------------------------------------------------ shapes
class GeometricShapeBox:
    """Box given by its centre (the Transform translation) and half size
    (src/shared/geometries/geometric_shape.cpp:6-18, geometric_element.cpp:19-55)."""

    def __init__(self, translation: Sequence[float], halfsize: Sequence[float], name: str = "Box"):
        self.c = np.asarray(translation, dtype=np.float64)
        self.hs = np.asarray(halfsize, dtype=np.float64)
        self.name = name

    def contain(self, x: np.ndarray) -> np.ndarray:
        return np.all(np.abs(x - self.c) <= self.hs, axis=1)

    def closest_point(self, x: np.ndarray) -> np.ndarray:
        p = x - self.c
        below, above = p < -self.hs, p > self.hs
        p = np.where(below, -self.hs, np.where(above, self.hs, p))
        inside = ~np.any(below | above, axis=1)
        if np.any(inside):
            pi = p[inside]
            which = np.argmin(self.hs - np.abs(pi), axis=1)
            rows = np.arange(len(pi))
            pi[rows, which] = np.where(pi[rows, which] < 0, -self.hs[which], self.hs[which])
            p[inside] = pi
        return p + self.c


class ComplexShape:
    """Union/difference of boxes (BinaryShapes, base_geometry.cpp:84-137)."""

    def __init__(self, name: str = "ComplexShape"):
        self.name = name
        self.parts: List[tuple] = []

    def add(self, shape: GeometricShapeBox) -> "ComplexShape":
        self.parts.append((shape, True))
        return self

    def subtract(self, shape: GeometricShapeBox) -> "ComplexShape":
        self.parts.append((shape, False))
        return self

    def contain(self, x: np.ndarray) -> np.ndarray:
        exist = np.zeros(len(x), dtype=bool)
        for shape, add in self.parts:
            inside = shape.contain(x)
            exist = (exist | inside) if add else (exist & ~inside)
        return exist

    def closest_point(self, x: np.ndarray) -> np.ndarray:
        best = np.zeros_like(x)
        dmin = np.full(len(x), np.finfo(np.float64).max)
        for shape, _ in self.parts:
            p = shape.closest_point(x)
            d = x - p
            dist = np.sqrt(_sqnorm(d))
            take = dist <= dmin
            best[take] = p[take]
            dmin = np.where(take, dist, dmin)
        return best

    def normal_direction(self, x: np.ndarray) -> np.ndarray:
        """Shape::findNormalDirection (base_geometry.cpp:45-58) for points off the surface."""
        inside = self.contain(x)
        d = self.closest_point(x) - x
        n = np.sqrt(_sqnorm(d))
        sign = np.where(inside, 1.0, -1.0)
        return sign[:, None] * (d / n[:, None])


def _sqnorm(d: np.ndarray) -> np.ndarray:
    s = d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]
    if d.shape[1] == 3:
        s = s + d[:, 2] * d[:, 2]
    return s


def lattice_positions(dim: int, lower, upper, dp: float, shape) -> np.ndarray:
    """ParticleGenerator<BaseParticles, Lattice> (particle_generator_lattice_{2d,3d}.cpp:12-23):
    cell centres of a dp mesh over the system bounds that the shape contains, in
    (i, j[, k]) loop order."""
    lo = np.asarray(lower[:dim], dtype=np.float64)
    up = np.asarray(upper[:dim], dtype=np.float64)
    n = [int(math.ceil((up[a] + 0.0 - lo[a]) / dp)) for a in range(dim)]
    axes = [(lo[a] + np.arange(n[a], dtype=np.float64) * dp) + 0.5 * dp for a in range(dim)]
    parts = getattr(shape, "parts", None)
    if parts and all(isinstance(p, GeometricShapeBox) for p, _ in parts):
        return _box_lattice(dim, axes, parts)
    out = []
    for x0 in axes[0]:  # slab by slab to bound memory
        if dim == 2:
            pts = np.stack([np.full(n[1], x0), axes[1]], axis=1)
        else:
            g1, g2 = np.meshgrid(axes[1], axes[2], indexing="ij")
            pts = np.stack([np.full(g1.size, x0), g1.ravel(), g2.ravel()], axis=1)
        keep = shape.contain(pts)
        if np.any(keep):
            out.append(pts[keep])
    return np.concatenate(out) if out else np.zeros((0, dim))


def _box_lattice(dim: int, axes, parts) -> np.ndarray:
    """lattice_positions for unions / differences of boxes: a box holds a lattice point
    exactly when every axis passes |x_a - c_a| <= hs_a, so the per-axis tests are taken
    once and combined slab by slab (same points, same order, without testing the points
    outside every box)."""
    masks = [[np.abs(axes[a] - box.c[a]) <= box.hs[a] for a in range(dim)] for box, _ in parts]
    rest = (len(axes[1]),) if dim == 2 else (len(axes[1]), len(axes[2]))
    planes = [m[1] if dim == 2 else (m[1][:, None] & m[2][None, :]) for m in masks]
    out = []
    for ix, x0 in enumerate(axes[0]):
        exist = np.zeros(rest, dtype=bool)
        for (box, add), m, plane in zip(parts, masks, planes):
            inside = plane if m[0][ix] else np.zeros(rest, dtype=bool)
            exist = (exist | inside) if add else (exist & ~inside)
        if not exist.any():
            continue
        if dim == 2:
            y = axes[1][exist]
            out.append(np.stack([np.full(len(y), x0), y], axis=1))
        else:
            j, k = np.nonzero(exist)
            out.append(np.stack([np.full(len(j), x0), axes[1][j], axes[2][k]], axis=1))
    return np.concatenate(out) if out else np.zeros((0, dim))


# ------------------------------------------------------------------ materials
class WeaklyCompressibleFluid:
    def __init__(self, rho0: float, c0: float):
        self.rho0, self.c0 = float(rho0), float(c0)
        self.p0 = self.rho0 * self.c0 * self.c0

    def ReferenceDensity(self) -> float:
        return self.rho0


class Solid:
    def __init__(self, rho0: float = 1.0):
        self.rho0 = float(rho0)

    def ReferenceDensity(self) -> float:
        return self.rho0


class Lattice:
    """Particle generator tag."""


class Gravity:
    def __init__(self, g: Sequence[float], reference_position: Optional[Sequence[float]] = None):
        self.g = np.zeros(3)
        self.g[: len(g)] = g
        self.reference = np.zeros(3) if reference_position is None else np.asarray(reference_position)


# ------------------------------------------------------------------ system and bodies
class SPHSystem:
    """SPHSystem(system_domain_bounds, global_resolution) (sph_system.cpp)."""

    def __init__(self, lower: Sequence[float], upper: Sequence[float], global_resolution: float,
                 device: int = 0, h_spacing_ratio: float = 1.3):
        self.dim = len(lower)
        self.lower = np.asarray(lower, dtype=np.float64)
        self.upper = np.asarray(upper, dtype=np.float64)
        self.dp = float(global_resolution)
        self.h_ratio = h_spacing_ratio
        self.ctx = default_context(device)
        self.bodies: List["SPHBody"] = []
        self.physical_time = 0.0

    def initializeSystemCellLinkedLists(self) -> None:
        for b in self.bodies:
            if isinstance(b, RealBody):
                b.updateCellLinkedList()

    def initializeSystemConfigurations(self) -> None:
        for b in self.bodies:
            for rel in b.relations:
                rel.updateConfiguration()


class SPHBody:
    def __init__(self, system: SPHSystem, shape=None, name: str = "Body"):
        self.system = system
        self.shape = shape
        self.name = getattr(shape, "name", name) if shape is not None else name
        self.material = None
        self.dim = system.dim
        self.h = system.h_ratio * system.dp  # SPHAdaptation h_ref = 1.3 dp (adaptation.h:71)
        self.handle: Optional[C.c_void_p] = None
        self.n = 0
        self.relations: List = []
        system.bodies.append(self)

    # SPHAdaptation::getKernel()->CutOffRadius()
    @property
    def cutoff_radius(self) -> float:
        return 2.0 * self.h

    def defineMatterMaterial(self, material) -> None:
        self.material = material

    def _create(self, n: int) -> None:
        h = C.c_void_p()
        N.call("sphx_body_create", self.system.ctx.h, self.dim, n, C.byref(h))
        self.handle = h
        self.n = n
        ids = np.arange(n, dtype=np.uint32)
        self.upload("OriginalID", ids, N.U32)
        self.upload("SortedID", ids, N.U32)

    def upload(self, name: str, values: np.ndarray, dtype: int = N.F64) -> None:
        a = np.ascontiguousarray(values, dtype=np.float64 if dtype == N.F64 else np.uint32)
        ncomp = 1 if a.ndim == 1 else a.shape[1]
        N.call("sphx_body_upload", self.handle, name.encode(), dtype, ncomp, a.ctypes.data_as(C.c_void_p), self.n)

    def download(self, name: str, out: Optional[np.ndarray] = None) -> np.ndarray:
        """Copies a variable to the host (AoS, n x ncomp; n for scalars).  `out`, when given,
        is a C-contiguous array of that size and type to fill (e.g. pinned host memory)."""
        ptr, dt, nc = C.c_void_p(), C.c_int(), C.c_int()
        N.call("sphx_body_device_ptr", self.handle, name.encode(), C.byref(ptr), C.byref(dt), C.byref(nc))
        dtype = np.float64 if dt.value == N.F64 else np.uint32
        if out is not None:
            if out.dtype != dtype or out.size != self.n * nc.value or not out.flags["C_CONTIGUOUS"]:
                raise ValueError(f"download of {name}: out must be C-contiguous {dtype.__name__} of "
                                 f"{self.n * nc.value} values")
            N.call("sphx_body_download", self.handle, name.encode(), out.ctypes.data_as(C.c_void_p), self.n)
            return out
        res = np.zeros((self.n, nc.value), dtype=dtype)
        N.call("sphx_body_download", self.handle, name.encode(), res.ctypes.data_as(C.c_void_p), self.n)
        return res[:, 0].copy() if nc.value == 1 else res

    def count_non_finite(self, name: str) -> int:
        """Particles of a floating-point variable with a NaN or infinite component
        (sphx_body_check_finite; 0 when the variable is finite)."""
        out = C.c_uint64()
        st = N.load().sphx_body_check_finite(self.handle, name.encode(), C.byref(out))
        if st not in (N.SPHX_OK, 7):  # 7: SPHX_ERR_NUMERIC, reported through the count
            N.check(st)
        return int(out.value)

    def upload_rows(self, name: str, values: np.ndarray, first: int) -> None:
        """Writes rows [first, first + len(values)) of a registered variable."""
        a = np.ascontiguousarray(values)
        count = a.shape[0] if a.ndim else 0
        N.call("sphx_body_upload_rows", self.handle, name.encode(), a.ctypes.data_as(C.c_void_p), int(first), count)

    def download_rows(self, name: str, first: int, count: int) -> np.ndarray:
        """Rows [first, first + count) of a registered variable (count x ncomp; count for
        scalars)."""
        ptr, dt, nc = C.c_void_p(), C.c_int(), C.c_int()
        N.call("sphx_body_device_ptr", self.handle, name.encode(), C.byref(ptr), C.byref(dt), C.byref(nc))
        res = np.zeros((count, nc.value), dtype=np.float64 if dt.value == N.F64 else np.uint32)
        N.call("sphx_body_download_rows", self.handle, name.encode(), res.ctypes.data_as(C.c_void_p), int(first),
               int(count))
        return res[:, 0].copy() if nc.value == 1 else res

    def device_ptr(self, name: str) -> int:
        ptr = C.c_void_p()
        N.call("sphx_body_device_ptr", self.handle, name.encode(), C.byref(ptr), None, None)
        return int(ptr.value)

    def generateParticles(self, generator=Lattice, positions: Optional[np.ndarray] = None) -> None:
        """generateParticles<BaseParticles, Lattice>() or explicit positions (observers)."""
        if positions is None:
            positions = lattice_positions(self.dim, self.system.lower, self.system.upper, self.system.dp,
                                          self.shape)
        positions = np.asarray(positions, dtype=np.float64).reshape(-1, self.dim)
        self._create(len(positions))
        self.upload("Position", positions)
        dp = self.system.dp
        vol = dp * dp * dp if self.dim == 3 else dp * dp
        Vol = np.full(self.n, vol)
        self.upload("VolumetricMeasure", Vol)
        rho0 = self.material.ReferenceDensity() if self.material is not None else 1.0
        self.upload("Density", np.full(self.n, rho0))
        self.upload("Mass", rho0 * Vol)  # MatterMaterial::initializeMatterVariables

    def __del__(self):
        if getattr(self, "handle", None) is not None and N._lib is not None:
            N._lib.sphx_body_destroy(self.handle)
            self.handle = None


class RealBody(SPHBody):
    def __init__(self, system: SPHSystem, shape=None, name: str = "Body"):
        super().__init__(system, shape, name)
        md = N.MeshDesc()
        lo = np.zeros(3)
        up = np.zeros(3)
        lo[: self.dim] = system.lower
        up[: self.dim] = system.upper
        # SPHAdaptation::createCellLinkedList: grid spacing = cut-off radius, buffer width 2
        N.call("sphx_mesh_from_bounds", self.dim, _dptr(lo), _dptr(up), self.cutoff_radius, 2, C.byref(md))
        self.mesh = md
        self.cell_list: Optional[C.c_void_p] = None

    def updateCellLinkedList(self) -> None:
        """SPHBody::updateCellLinkedList (base_body.cpp:103-113)."""
        if self.cell_list is None:
            h = C.c_void_p()
            N.call("sphx_cell_list_create", self.system.ctx.h, C.byref(self.mesh), self.n, C.byref(h))
            self.cell_list = h
        N.call("sphx_cell_list_update", self.cell_list, self.handle)

    def cell_list_entries(self) -> int:
        """Entries of the cell list: the particles plus their periodic images."""
        n = C.c_size_t()
        N.call("sphx_cell_list_num_entries", self.cell_list, C.byref(n))
        return n.value

    def cell_list_arrays(self):
        nc = C.c_size_t()
        N.call("sphx_cell_list_num_cells", self.cell_list, C.byref(nc))
        off = np.zeros(nc.value + 1, dtype=np.uint32)
        idx = np.zeros(self.n, dtype=np.uint32)
        N.call("sphx_cell_list_download", self.cell_list, off.ctypes.data_as(C.POINTER(C.c_uint32)),
               idx.ctypes.data_as(C.POINTER(C.c_uint32)), self.n)
        return off, idx

    def __del__(self):
        if getattr(self, "cell_list", None) is not None and N._lib is not None:
            N._lib.sphx_cell_list_destroy(self.cell_list)
            self.cell_list = None
        super().__del__()


class FluidBody(RealBody):
    pass


class SolidBody(RealBody):
    def defineMatterMaterial(self, material=None) -> None:
        self.material = material if material is not None else Solid()


class ObserverBody(SPHBody):
    def generateParticles(self, generator=None, positions=None) -> None:
        pts = np.asarray(positions, dtype=np.float64).reshape(-1, self.dim)
        self._create(len(pts))
        self.upload("Position", pts)


# ------------------------------------------------------------------ relations
class InnerRelation:
    def __init__(self, body: RealBody):
        self.body = body
        h = C.c_void_p()
        N.call("sphx_inner_relation_create", body.handle, body._cl_handle(), body.h, C.byref(h))
        self.handle = h
        body.relations.append(self)

    def updateConfiguration(self) -> None:
        N.call("sphx_relation_update", self.handle)

    def neighbors(self):
        return _download_relation(self.handle, self.body.n, self.body.dim)

    def __del__(self):
        if getattr(self, "handle", None) is not None and N._lib is not None:
            N._lib.sphx_relation_destroy(self.handle)
            self.handle = None


class ContactRelation:
    """ContactRelation(body, {&target}) with NeighborBuilderContact and SearchDepthContact."""

    def __init__(self, body: SPHBody, targets: Sequence[RealBody]):
        if len(targets) != 1:
            raise ValueError("one contact body per relation")
        self.body, self.target = body, targets[0]
        # chooseKernel: the larger smoothing length (neighborhood.cpp:72-77)
        h_k = max(body.h, self.target.h)
        gs = self.target.mesh.grid_spacing
        depth = 1 + int(math.floor((2.0 * body.h) * (1.0 / gs)))  # base_body_relation.cpp:10-16
        rho0 = self.target.material.ReferenceDensity() if self.target.material is not None else 1.0
        h = C.c_void_p()
        N.call("sphx_contact_relation_create", body.handle, self.target.handle, self.target._cl_handle(), h_k,
               depth, rho0, C.byref(h))
        self.handle = h
        self.search_depth = depth
        body.relations.append(self)

    def updateConfiguration(self) -> None:
        N.call("sphx_relation_update", self.handle)

    def neighbors(self):
        return _download_relation(self.handle, self.body.n, self.body.dim)

    def __del__(self):
        if getattr(self, "handle", None) is not None and N._lib is not None:
            N._lib.sphx_relation_destroy(self.handle)
            self.handle = None


def _cl_handle(self: RealBody):
    if self.cell_list is None:
        h = C.c_void_p()
        N.call("sphx_cell_list_create", self.system.ctx.h, C.byref(self.mesh), max(self.n, 1), C.byref(h))
        self.cell_list = h
    return self.cell_list


RealBody._cl_handle = _cl_handle


class ComplexRelation:
    def __init__(self, inner: InnerRelation, contact: ContactRelation):
        self.inner, self.contact = inner, contact

    def updateConfiguration(self) -> None:
        self.inner.updateConfiguration()
        self.contact.updateConfiguration()


def _download_relation(handle, n: int, dim: int):
    counts = np.zeros(n, dtype=np.uint32)
    total = C.c_size_t()
    u32 = C.POINTER(C.c_uint32)
    N.call("sphx_relation_download", handle, counts.ctypes.data_as(u32), None, None, None, None, None,
           C.byref(total))
    t = int(counts.sum())
    j = np.zeros(t, dtype=np.uint32)
    W, dW, r = np.zeros(t), np.zeros(t), np.zeros(t)
    e = np.zeros(t * dim)
    N.call("sphx_relation_download", handle, counts.ctypes.data_as(u32), j.ctypes.data_as(u32), _dptr(W),
           _dptr(dW), _dptr(r), _dptr(e), C.byref(total))
    return dict(counts=counts, j=j, W=W, dW=dW, r=r, e=e.reshape(t, dim))


# ------------------------------------------------------------------ dynamics
class Integration1stHalfWithWallRiemann:
    """fluid_dynamics::Integration1stHalfWithWallRiemann (tag)."""


class Integration2ndHalfWithWallRiemann:
    """fluid_dynamics::Integration2ndHalfWithWallRiemann (tag)."""


class DensitySummationComplexFreeSurface:
    """fluid_dynamics::DensitySummationComplexFreeSurface (tag)."""


class AcousticTimeStep:
    """fluid_dynamics::AcousticTimeStep (tag, acousticCFL = 0.6)."""


class AdvectionTimeStep:
    """fluid_dynamics::AdvectionTimeStep (tag, advectionCFL = 0.25)."""


class GravityForce:
    """GravityForce<Gravity> (tag)."""


class NormalDirectionFromBodyShape:
    """NormalDirectionFromBodyShape (tag)."""


def fluid_params(body: SPHBody, U_ref: float = 0.0, acoustic_cfl: float = 0.6,
                 advection_cfl: float = 0.25) -> N.FluidParams:
    # registerStateVariable of the fluid-step variables (fluid_integration.hpp:10-22)
    for v in ("Velocity", "Force", "ForcePrior"):
        N.call("sphx_body_register", body.handle, v.encode(), N.F64, body.dim)
    for v in ("Pressure", "DensityChangeRate", "DensitySummation"):
        N.call("sphx_body_register", body.handle, v.encode(), N.F64, 1)
    p = N.FluidParams()
    p.rho0, p.c0 = body.material.rho0, body.material.c0
    p.h = body.h
    s = C.c_double()
    N.call("sphx_lattice_number_density", body.dim, body.h, body.system.dp, C.byref(s))
    p.sigma0 = s.value
    p.limiter_slope = 3.0
    p.acoustic_cfl, p.advection_cfl, p.U_ref = acoustic_cfl, advection_cfl, U_ref
    return p


class Dynamics1Level:
    def __init__(self, kind, inner: InnerRelation, contact: ContactRelation):
        self.kind, self.inner, self.contact = kind, inner, contact
        self.params = fluid_params(inner.body)
        self._fn = {Integration1stHalfWithWallRiemann: "sphx_integration_1st_half_with_wall_riemann",
                    Integration2ndHalfWithWallRiemann: "sphx_integration_2nd_half_with_wall_riemann"}[kind]

    def exec(self, dt: float = 0.0) -> None:
        N.call(self._fn, self.inner.handle, self.contact.handle if self.contact else None,
               C.byref(self.params), float(dt))


class InteractionWithUpdate:
    def __init__(self, kind, inner: InnerRelation, contact: ContactRelation):
        if kind is not DensitySummationComplexFreeSurface:
            raise ValueError("unsupported interaction")
        self.inner, self.contact = inner, contact
        self.params = fluid_params(inner.body)

    def exec(self, dt: float = 0.0) -> None:
        N.call("sphx_density_summation_complex_free_surface", self.inner.handle,
               self.contact.handle if self.contact else None, C.byref(self.params))


class ReduceDynamics:
    def __init__(self, kind, body: SPHBody, U_ref: float = 0.0):
        self.kind, self.body = kind, body
        self.params = fluid_params(body, U_ref=U_ref)
        self._fn = {AcousticTimeStep: "sphx_acoustic_time_step", AdvectionTimeStep: "sphx_advection_time_step"}[kind]

    def exec(self, dt: float = 0.0) -> float:
        out = C.c_double()
        N.call(self._fn, self.body.handle, C.byref(self.params), C.byref(out))
        return out.value


class SimpleDynamics:
    def __init__(self, kind, body: SPHBody, *args):
        self.kind, self.body, self.args = kind, body, args

    def exec(self, dt: float = 0.0) -> None:
        if self.kind is GravityForce:
            g = np.ascontiguousarray(self.args[0].g)
            N.call("sphx_gravity_force", self.body.handle, _dptr(g))
        elif self.kind is NormalDirectionFromBodyShape:
            pos = self.body.download("Position")
            self.body.upload("NormalDirection", self.body.shape.normal_direction(pos))
        else:
            raise ValueError("unsupported simple dynamics")


class ParticleSorting:
    def __init__(self, body: RealBody):
        self.body = body

    def exec(self, dt: float = 0.0) -> None:
        # getSortSequenceMesh(): the cell-linked-list mesh (cell_linked_list.cpp:131-136)
        N.call("sphx_particle_sorting", self.body.handle, C.byref(self.body.mesh))


class ObservedQuantityRecording:
    """ObservedQuantityRecording<Real>(name, observer_contact): interpolated values."""

    def __init__(self, name: str, contact: ContactRelation):
        self.name, self.contact = name, contact

    def exec(self) -> np.ndarray:
        out = np.zeros(max(1, self.contact.body.n))
        N.call("sphx_observe_quantity", self.contact.handle, self.name.encode(), _dptr(out))
        return out[: self.contact.body.n]


class TotalMechanicalEnergy:
    def __init__(self, body: SPHBody, gravity: Gravity):
        self.body, self.gravity = body, gravity

    def exec(self) -> float:
        out = C.c_double()
        g = np.ascontiguousarray(self.gravity.g)
        N.call("sphx_total_mechanical_energy", self.body.handle, _dptr(g), C.byref(out))
        return out.value


class UpperFrontInAxisDirection:
    def __init__(self, body: SPHBody, lower, upper, axis: int):
        self.body, self.axis = body, axis
        self.lo = np.zeros(3)
        self.up = np.zeros(3)
        self.lo[: body.dim] = lower
        self.up[: body.dim] = upper

    def exec(self) -> float:
        out = C.c_double()
        N.call("sphx_upper_front_in_axis_direction", self.body.handle, self.axis, _dptr(self.lo), _dptr(self.up),
               C.byref(out))
        return out.value


# ------------------------------------------------------------------ CK particle methods
# The dynamics the tests_sycl drivers add to their ParticleMethodContainer<par_ck>
# (dambreak_sycl.cpp:97-123), on the CUDA policy.  Their state variables are registered
# by the library on first use with the reference's initial values.
class LinearCorrectionMatrixCK:
    """addInteractionDynamics<LinearCorrectionMatrix, WithUpdate>(inner, alpha)
    .addPostContactInteraction(contact)."""

    def __init__(self, inner: InnerRelation, contact: Optional[ContactRelation], alpha: float = 0.5):
        self.inner, self.contact, self.alpha = inner, contact, float(alpha)

    def exec(self, dt: float = 0.0) -> None:
        N.call("sphx_ck_linear_correction_matrix", self.inner.handle,
               self.contact.handle if self.contact else None, self.alpha)


class _CKFluidDynamics:
    _fn = ""

    def __init__(self, inner: InnerRelation, contact: Optional[ContactRelation]):
        self.inner, self.contact = inner, contact
        self.params = fluid_params(inner.body)

    def exec(self, dt: float = 0.0) -> None:
        args = [self.inner.handle, self.contact.handle if self.contact else None, C.byref(self.params)]
        if self._fn != "sphx_ck_density_regularization":
            args.append(float(dt))
        N.call(self._fn, *args)


class AcousticStep1stHalfCK(_CKFluidDynamics):
    """AcousticStep1stHalf<OneLevel, AcousticRiemannSolverCK, LinearCorrectionCK> with its
    Contact<Wall, ...> part."""
    _fn = "sphx_ck_acoustic_step_1st_half"


class AcousticStep2ndHalfCK(_CKFluidDynamics):
    """AcousticStep2ndHalf<OneLevel, AcousticRiemannSolverCK, LinearCorrectionCK> with its
    Contact<Wall, ...> part."""
    _fn = "sphx_ck_acoustic_step_2nd_half"


class DensityRegularizationCK(_CKFluidDynamics):
    """CompressionSummation (inner + contact) with the post-state
    DensityRegularization<WeaklyCompressibleFluid, FreeSurface>."""
    _fn = "sphx_ck_density_regularization"


class FreeSurfaceIndicationCK:
    """InteractionDynamicsCK<FreeSurfaceIndicationComplexSpatialTemporalCK>(inner, contact):
    PositionDivergence and Indicator (1 at the free surface) of the fluid."""

    def __init__(self, inner: InnerRelation, contact: Optional[ContactRelation]):
        self.inner, self.contact = inner, contact

    def exec(self, dt: float = 0.0) -> None:
        N.call("sphx_ck_free_surface_indication", self.inner.handle, self.contact.handle if self.contact else None)


class AdvectionStepSetupCK:
    def __init__(self, body: SPHBody):
        self.body = body

    def exec(self, dt: float = 0.0) -> None:
        N.call("sphx_ck_advection_step_setup", self.body.handle)


class UpdateParticlePositionCK:
    def __init__(self, body: SPHBody):
        self.body = body

    def exec(self, dt: float = 0.0) -> None:
        N.call("sphx_ck_update_particle_position", self.body.handle)


class AcousticTimeStepCK:
    def __init__(self, body: SPHBody, acoustic_cfl: float = 0.6):
        self.body = body
        self.params = fluid_params(body, acoustic_cfl=acoustic_cfl)

    def exec(self, dt: float = 0.0) -> float:
        out = C.c_double()
        N.call("sphx_ck_acoustic_time_step", self.body.handle, C.byref(self.params), C.byref(out))
        return out.value


class AdvectionTimeStepCK:
    def __init__(self, body: SPHBody, U_ref: float, advection_cfl: float = 0.25):
        self.body = body
        self.params = fluid_params(body, U_ref=U_ref, advection_cfl=advection_cfl)

    def exec(self, dt: float = 0.0) -> float:
        out = C.c_double()
        N.call("sphx_ck_advection_time_step", self.body.handle, C.byref(self.params), C.byref(out))
        return out.value


class ObservingQuantityCK:
    """Interpolation<Contact<Real>> of a fluid variable at the observers (tabulated kernel,
    current volumes)."""

    def __init__(self, contact: ContactRelation, name: str):
        self.contact, self.name = contact, name

    def exec(self) -> np.ndarray:
        out = np.zeros(max(1, self.contact.body.n))
        N.call("sphx_ck_observe_quantity", self.contact.handle, self.name.encode(), _dptr(out))
        return out[: self.contact.body.n]


class TriggerByInterval:
    """TimeStepper::TriggerByInterval (sph_solver.cpp:53-80): fires once the physical time
    accumulated since it last fired exceeds the interval, then re-evaluates the interval."""

    def __init__(self, interval: float):
        self.present_time, self.interval = 0.0, float(interval)

    def increment(self, dt: float) -> None:
        self.present_time += dt

    def __call__(self, evaluator) -> bool:
        if self.present_time > self.interval:
            self.present_time = 0.0
            self.interval = evaluator.exec()
            return True
        return False


# ------------------------------------------------------------------ Taylor-Green pieces
class Viscosity:
    """addMaterialProperty<Viscosity>(mu): a fixed dynamic viscosity."""

    def __init__(self, mu: float):
        self.mu = float(mu)

    def ReferenceViscosity(self) -> float:
        return self.mu


def addMaterialProperty(body: SPHBody, prop) -> None:
    body.viscosity = prop


class PeriodicAlongAxis:
    """PeriodicAlongAxis(bounds, axis): the periodic box along one axis."""

    def __init__(self, lower: Sequence[float], upper: Sequence[float], axis: int):
        self.lower, self.upper, self.axis = float(lower[axis]), float(upper[axis]), int(axis)


class _PeriodicBounding:
    def __init__(self, body: RealBody, periodic: PeriodicAlongAxis):
        self.body, self.p = body, periodic

    def exec(self, dt: float = 0.0) -> None:
        N.call("sphx_periodic_bounding", self.body.handle, self.p.axis, self.p.lower, self.p.upper)


class _PeriodicCellLinkedList:
    """The images are inserted by every update of the body's cell list once the axis is
    registered; exec() is the reference's call site and does nothing further."""

    def __init__(self, body: RealBody, periodic: PeriodicAlongAxis):
        N.call("sphx_cell_list_set_periodic", body._cl_handle(), periodic.axis, periodic.lower, periodic.upper,
               body.cutoff_radius)

    def exec(self, dt: float = 0.0) -> None:
        pass


class PeriodicConditionUsingCellLinkedList:
    def __init__(self, body: RealBody, periodic: PeriodicAlongAxis):
        self.bounding_ = _PeriodicBounding(body, periodic)
        self.update_cell_linked_list_ = _PeriodicCellLinkedList(body, periodic)


class DensitySummationInner:
    """Tag: InteractionWithUpdate<fluid_dynamics::DensitySummationInner>."""


class ViscousForceInner:
    """InteractionWithUpdate<fluid_dynamics::ViscousForceInner>(inner)."""

    def __init__(self, inner: InnerRelation):
        self.inner = inner
        N.call("sphx_relation_keep_distances", inner.handle)

    def exec(self, dt: float = 0.0) -> None:
        N.call("sphx_viscous_force_inner", self.inner.handle, self.inner.body.viscosity.mu)


class TransportVelocityCorrectionInner:
    """InteractionWithUpdate<TransportVelocityCorrectionInner<TruncatedLinear, AllParticles>>."""

    def __init__(self, inner: InnerRelation, coefficient: float = 0.2):
        self.inner, self.coefficient = inner, float(coefficient)

    def exec(self, dt: float = 0.0) -> None:
        N.call("sphx_transport_velocity_correction_inner", self.inner.handle, self.coefficient)


class DensitySummationInnerDynamics:
    def __init__(self, inner: InnerRelation):
        self.inner = inner
        self.params = fluid_params(inner.body)

    def exec(self, dt: float = 0.0) -> None:
        N.call("sphx_density_summation_inner", self.inner.handle, C.byref(self.params))


class Integration1stHalfInnerRiemann:
    """Dynamics1Level<Integration1stHalfInnerRiemann>(inner)."""

    def __init__(self, inner: InnerRelation):
        self.inner = inner
        self.params = fluid_params(inner.body)

    def exec(self, dt: float = 0.0) -> None:
        N.call("sphx_integration_1st_half_with_wall_riemann", self.inner.handle, None, C.byref(self.params),
               float(dt))


class Integration2ndHalfInnerNoRiemann:
    """Dynamics1Level<Integration2ndHalfInnerNoRiemann>(inner): the 2nd half without the
    Riemann dissipation (limiter slope 0 makes DissipativePJump zero)."""

    def __init__(self, inner: InnerRelation):
        self.inner = inner
        self.params = fluid_params(inner.body)
        self.params.limiter_slope = 0.0

    def exec(self, dt: float = 0.0) -> None:
        N.call("sphx_integration_2nd_half_with_wall_riemann", self.inner.handle, None, C.byref(self.params),
               float(dt))


class AdvectionViscousTimeStep(ReduceDynamics):
    """ReduceDynamics<AdvectionViscousTimeStep>(body, U_ref): the reference speed is
    max(U_ref, mu / rho0 / h) (fluid_time_step.cpp:67-74)."""

    def __init__(self, body: SPHBody, U_ref: float):
        viscous_speed = body.viscosity.mu / body.material.ReferenceDensity() / body.h
        super().__init__(AdvectionTimeStep, body, max(viscous_speed, U_ref))


class TotalKineticEnergy:
    def __init__(self, body: SPHBody):
        self.body = body

    def exec(self) -> float:
        out = C.c_double()
        g = np.zeros(3)
        N.call("sphx_total_mechanical_energy", self.body.handle, _dptr(g), C.byref(out))
        return out.value


class MaximumSpeed:
    def __init__(self, body: SPHBody):
        self.body = body

    def exec(self) -> float:
        out = C.c_double()
        N.call("sphx_maximum_speed", self.body.handle, C.byref(out))
        return out.value
