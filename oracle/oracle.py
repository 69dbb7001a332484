"""ctypes wrapper of the FP64 CPU oracle (oracle/sphx_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, the smoke check and the benchmark's CPU
baseline legs.  The product library never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libsphx_oracle.so")

FLUID, WALL, OBSERVER = 0, 1, 2
INNER, CONTACT, OBSERVER_CONTACT = 0, 1, 2


class OrcCaseDesc(C.Structure):
    _fields_ = [
        ("dim", C.c_int), ("n_observers", C.c_int),
        ("sys_lower", C.c_double * 3), ("sys_upper", C.c_double * 3),
        ("dp", C.c_double), ("h_ratio", C.c_double),
        ("water_center", C.c_double * 3), ("water_halfsize", C.c_double * 3),
        ("outer_center", C.c_double * 3), ("outer_halfsize", C.c_double * 3),
        ("inner_center", C.c_double * 3), ("inner_halfsize", C.c_double * 3),
        ("rho0", C.c_double), ("c0", C.c_double), ("U_ref", C.c_double),
        ("gravity", C.c_double * 3),
        ("observers", (C.c_double * 3) * 16),
    ]


class OrcTGVDesc(C.Structure):
    _fields_ = [("dim", C.c_int), ("velocity_kind", C.c_int), ("L", C.c_double), ("dp", C.c_double),
                ("h_ratio", C.c_double), ("rho0", C.c_double), ("U", C.c_double), ("c0", C.c_double),
                ("Re", C.c_double)]


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (a second or two)."""
    src = os.path.join(HERE, "sphx_oracle.cpp")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", HERE])
    return LIB_PATH


_lib: Optional[C.CDLL] = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        vp, d, i, sz = C.c_void_p, C.c_double, C.c_int, C.c_size_t
        dp_, up_ = C.POINTER(C.c_double), C.POINTER(C.c_uint32)
        L.orc_case_create.restype = vp
        L.orc_case_create.argtypes = [C.POINTER(OrcCaseDesc)]
        L.orc_case_destroy.argtypes = [vp]
        L.orc_num_particles.restype = sz
        L.orc_num_particles.argtypes = [vp, i]
        L.orc_body_resize.argtypes = [vp, i, sz]
        L.orc_constant.restype = d
        L.orc_constant.argtypes = [vp, i]
        L.orc_get.restype = i
        L.orc_get.argtypes = [vp, i, C.c_char_p, dp_]
        L.orc_set.restype = i
        L.orc_set.argtypes = [vp, i, C.c_char_p, dp_]
        L.orc_get_ids.argtypes = [vp, i, up_, up_]
        L.orc_mesh.argtypes = [vp, dp_, dp_, C.POINTER(C.c_int)]
        L.orc_num_cells.restype = sz
        L.orc_num_cells.argtypes = [vp]
        L.orc_update_cell_linked_list.argtypes = [vp, i]
        L.orc_get_cell_list.argtypes = [vp, i, up_, up_]
        L.orc_update_configuration.argtypes = [vp]
        L.orc_update_observer_configuration.argtypes = [vp]
        L.orc_get_neighbors.restype = sz
        L.orc_get_neighbors.argtypes = [vp, i, up_, up_, dp_, dp_, dp_, dp_]
        L.orc_density_summation.argtypes = [vp]
        L.orc_integration_1st_half.argtypes = [vp, d]
        L.orc_integration_2nd_half.argtypes = [vp, d]
        L.orc_acoustic_time_step.restype = d
        L.orc_acoustic_time_step.argtypes = [vp]
        L.orc_advection_time_step.restype = d
        L.orc_advection_time_step.argtypes = [vp]
        L.orc_particle_sorting.argtypes = [vp]
        L.orc_observe_pressure.argtypes = [vp, dp_]
        L.orc_total_mechanical_energy.restype = d
        L.orc_total_mechanical_energy.argtypes = [vp]
        L.orc_upper_front.restype = d
        L.orc_upper_front.argtypes = [vp, i, dp_, dp_]
        L.orc_lattice_number_density.restype = d
        L.orc_lattice_number_density.argtypes = [i, d, d]
        L.orc_set_num_threads.argtypes = [i]
        L.orc_get_max_threads.restype = i
        L.orc_ck_kernel.restype = d
        L.orc_ck_kernel.argtypes = [vp, i, d]
        L.orc_ck_initialize.argtypes = [vp]
        L.orc_ck_acoustic_step.restype = i
        L.orc_ck_acoustic_step.argtypes = [vp, dp_]
        L.orc_ck_configuration.argtypes = [vp]
        L.orc_ck_free_surface_indication.argtypes = [vp]
        L.orc_ck_nested_advection_step.restype = i
        L.orc_ck_nested_advection_step.argtypes = [vp, dp_, dp_]
        L.orc_ck_density_regularization.argtypes = [vp]
        L.orc_ck_advection_step_setup.argtypes = [vp]
        L.orc_ck_linear_correction_matrix.argtypes = [vp, d]
        L.orc_ck_acoustic_1st_half.argtypes = [vp, d]
        L.orc_ck_acoustic_2nd_half.argtypes = [vp, d]
        L.orc_ck_acoustic_time_step.restype = d
        L.orc_ck_acoustic_time_step.argtypes = [vp]
        L.orc_ck_advection_time_step.restype = d
        L.orc_ck_advection_time_step.argtypes = [vp]
        L.orc_ck_update_particle_position.argtypes = [vp]
        L.orc_ck_advection_steps.restype = C.c_long
        L.orc_ck_advection_steps.argtypes = [vp]
        L.orc_ck_observe_pressure.argtypes = [vp, dp_]
        L.orc_ck_get.argtypes = [vp, i, dp_]
        L.orc_tgv_create.restype = vp
        L.orc_tgv_create.argtypes = [C.POINTER(OrcTGVDesc)]
        L.orc_tgv_advection_step.restype = i
        L.orc_tgv_advection_step.argtypes = [vp, dp_, dp_]
        L.orc_total_kinetic_energy.restype = d
        L.orc_total_kinetic_energy.argtypes = [vp]
        L.orc_maximum_speed.restype = d
        L.orc_maximum_speed.argtypes = [vp]
        L.orc_cell_entries.restype = sz
        L.orc_cell_entries.argtypes = [vp, i]
        L.orc_advection_step.restype = i
        L.orc_advection_step.argtypes = [vp, i, C.c_long, dp_, dp_, dp_, i, dp_, dp_]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    if a.dtype == np.float64:
        return a.ctypes.data_as(C.POINTER(C.c_double))
    if a.dtype == np.uint32:
        return a.ctypes.data_as(C.POINTER(C.c_uint32))
    raise TypeError(a.dtype)


def desc_of(case) -> OrcCaseDesc:
    d = OrcCaseDesc()
    d.dim = case.dim
    d.n_observers = len(case.observers)
    for name in ("sys_lower", "sys_upper", "water_center", "water_halfsize", "outer_center",
                 "outer_halfsize", "inner_center", "inner_halfsize", "gravity"):
        getattr(d, name)[:] = list(getattr(case, name))
    d.dp, d.h_ratio = case.dp, case.h_ratio
    d.rho0, d.c0, d.U_ref = case.rho0, case.c0, case.U_ref
    for k, o in enumerate(case.observers):
        d.observers[k][:] = list(o)
    return d


def set_num_threads(n: int) -> None:
    lib().orc_set_num_threads(int(n))


def max_threads() -> int:
    return int(lib().orc_get_max_threads())


class OracleCase:
    """One dam-break case held by the oracle (fluid, wall and observer bodies)."""

    CONSTANTS = ("sigma0", "W0", "h", "rc", "contact_depth", "inv_rho0c0_ave", "rho0c0_geo_ave",
                 "inv_c0_ave", "p0", "factor_W", "factor_dW")

    def __init__(self, case):
        self.case = case
        self.dim = case.dim
        self._desc = desc_of(case)
        self.h = lib().orc_case_create(C.byref(self._desc))
        self.iteration = 0
        self.physical_time = C.c_double(0.0)
        self.acoustic_dt = C.c_double(0.0)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_case_destroy(self.h)
            self.h = None

    def resize(self, body: int, n: int) -> None:
        """Zeroed body of n particles (set its variables, then rebuild lists and relations)."""
        lib().orc_body_resize(self.h, body, int(n))

    def n(self, body: int = FLUID) -> int:
        return int(lib().orc_num_particles(self.h, body))

    def constant(self, name: str) -> float:
        return float(lib().orc_constant(self.h, self.CONSTANTS.index(name)))

    def get(self, name: str, body: int = FLUID) -> np.ndarray:
        n = self.n(body)
        out = np.zeros(n * self.dim, dtype=np.float64)
        nc = lib().orc_get(self.h, body, name.encode(), _p(out))
        if nc == 0:
            raise KeyError(name)
        return out.reshape(n, self.dim) if nc > 1 else out[:n].copy()

    def set(self, name: str, values: np.ndarray, body: int = FLUID) -> None:
        a = np.ascontiguousarray(values, dtype=np.float64).ravel()
        if lib().orc_set(self.h, body, name.encode(), _p(a)) == 0:
            raise KeyError(name)

    def ids(self, body: int = FLUID):
        n = self.n(body)
        o = np.zeros(n, dtype=np.uint32)
        s = np.zeros(n, dtype=np.uint32)
        lib().orc_get_ids(self.h, body, _p(o), _p(s))
        return o, s

    def mesh(self):
        lo = np.zeros(3)
        gs = np.zeros(1)
        ac = (C.c_int * 3)()
        lib().orc_mesh(self.h, _p(lo), _p(gs), ac)
        return lo, float(gs[0]), tuple(ac)

    def cell_list(self, body: int = FLUID):
        nc = int(lib().orc_num_cells(self.h))
        off = np.zeros(nc + 1, dtype=np.uint32)
        idx = np.zeros(self.n(body), dtype=np.uint32)
        lib().orc_get_cell_list(self.h, body, _p(off), _p(idx))
        return off, idx

    def update_cell_linked_list(self, body: int = FLUID) -> None:
        lib().orc_update_cell_linked_list(self.h, body)

    def update_configuration(self) -> None:
        lib().orc_update_configuration(self.h)
        lib().orc_update_observer_configuration(self.h)

    def neighbors(self, which: int = INNER):
        nsrc = self.n(OBSERVER if which == OBSERVER_CONTACT else FLUID)
        counts = np.zeros(nsrc, dtype=np.uint32)
        total = int(lib().orc_get_neighbors(self.h, which, _p(counts), None, None, None, None, None))
        j = np.zeros(total, dtype=np.uint32)
        W, dW, r = (np.zeros(total) for _ in range(3))
        e = np.zeros(total * self.dim)
        lib().orc_get_neighbors(self.h, which, _p(counts), _p(j), _p(W), _p(dW), _p(r), _p(e))
        return dict(counts=counts, j=j, W=W, dW=dW, r=r, e=e.reshape(total, self.dim))

    def density_summation(self) -> None:
        lib().orc_density_summation(self.h)

    def integration_1st_half(self, dt: float) -> None:
        lib().orc_integration_1st_half(self.h, float(dt))

    def integration_2nd_half(self, dt: float) -> None:
        lib().orc_integration_2nd_half(self.h, float(dt))

    def acoustic_time_step(self) -> float:
        return float(lib().orc_acoustic_time_step(self.h))

    def advection_time_step(self) -> float:
        return float(lib().orc_advection_time_step(self.h))

    def particle_sorting(self) -> None:
        lib().orc_particle_sorting(self.h)

    def observe_pressure(self) -> np.ndarray:
        out = np.zeros(max(1, self.n(OBSERVER)))
        lib().orc_observe_pressure(self.h, _p(out))
        return out[: self.n(OBSERVER)]

    def total_mechanical_energy(self) -> float:
        return float(lib().orc_total_mechanical_energy(self.h))

    def upper_front(self, axis: int, lo, up) -> float:
        lo = np.asarray(lo, dtype=np.float64)
        up = np.asarray(up, dtype=np.float64)
        return float(lib().orc_upper_front(self.h, axis, _p(lo), _p(up)))

    def advection_step(self, observe: bool = False):
        """One advection step of the case's driver loop; returns (substeps, Dt, obs, energy)."""
        Dt = C.c_double(0.0)
        nobs = max(1, self.n(OBSERVER))
        obs = np.zeros(nobs)
        en = np.zeros(1)
        sub = lib().orc_advection_step(self.h, self.case.loop_style, self.iteration,
                                       C.byref(self.physical_time), C.byref(self.acoustic_dt),
                                       C.byref(Dt), int(observe), _p(obs), _p(en))
        self.iteration += 1
        return sub, Dt.value, obs[: self.n(OBSERVER)], float(en[0])

    # ------------------------------------------------------------------ CK numerics
    CK_FIELDS = ("Compression", "CompressionRate", "VolumetricMeasureRef", "CompressionSummation",
                 "Displacement", "LinearCorrectionMatrix", "PositionDivergence", "Indicator")

    def ck_kernel(self, which: str, r: float = 0.0) -> float:
        """Tabulated Wendland C2 of this case: which in ("W", "dW", "W0")."""
        return float(lib().orc_ck_kernel(self.h, ("W", "dW", "W0").index(which), float(r)))

    def ck_initialize(self) -> None:
        lib().orc_ck_initialize(self.h)

    def ck_acoustic_step(self) -> bool:
        """One loop pass of dambreak_sycl.cpp; True when an advection step fell due (the
        positions were moved; call ck_configuration after observing)."""
        return bool(lib().orc_ck_acoustic_step(self.h, C.byref(self.physical_time)))

    def ck_configuration(self) -> None:
        lib().orc_ck_configuration(self.h)

    def ck_free_surface_indication(self) -> None:
        lib().orc_ck_free_surface_indication(self.h)

    def ck_nested_advection_step(self):
        """One advection step of the 3D SYCL dam-break loop (nested advection / acoustic
        loops, acoustic dt first); returns (sub-steps, advection dt)."""
        Dt = C.c_double()
        sub = lib().orc_ck_nested_advection_step(self.h, C.byref(self.physical_time), C.byref(Dt))
        self.iteration += 1
        return sub, Dt.value

    def ck_advection_steps(self) -> int:
        return int(lib().orc_ck_advection_steps(self.h))

    def ck_observe_pressure(self) -> np.ndarray:
        out = np.zeros(max(self.n(OBSERVER), 1))
        lib().orc_ck_observe_pressure(self.h, _p(out))
        return out[: self.n(OBSERVER)]

    def ck_get(self, name: str) -> np.ndarray:
        which = self.CK_FIELDS.index(name)
        n, d = self.n(FLUID), self.dim
        scalar = which < 4 or which >= 6
        size = n * (1 if scalar else (d if which == 4 else d * d))
        out = np.zeros(max(size, 1))
        lib().orc_ck_get(self.h, which, _p(out))
        out = out[:size]
        return out if scalar else (out.reshape(n, d) if which == 4 else out.reshape(n, d, d))


class OracleTGV(OracleCase):
    """A Taylor-Green vortex held by the oracle (periodic box, no wall or observer)."""

    def __init__(self, tgv):
        self.case = tgv
        self.dim = tgv.dim
        self._desc = OrcTGVDesc(tgv.dim, tgv.velocity_kind, tgv.L, tgv.dp, tgv.h_ratio, tgv.rho0, tgv.U, tgv.c0,
                                tgv.Re)
        self.h = lib().orc_tgv_create(C.byref(self._desc))
        self.iteration = 0
        self.physical_time = C.c_double(0.0)
        self.acoustic_dt = C.c_double(0.0)

    def advection_step(self, observe: bool = False):
        Dt = C.c_double()
        sub = lib().orc_tgv_advection_step(self.h, C.byref(self.physical_time), C.byref(Dt))
        self.iteration += 1
        return sub, Dt.value

    def kinetic_energy(self) -> float:
        return float(lib().orc_total_kinetic_energy(self.h))

    def maximum_speed(self) -> float:
        return float(lib().orc_maximum_speed(self.h))

    def cell_entries(self) -> int:
        return int(lib().orc_cell_entries(self.h, FLUID))
