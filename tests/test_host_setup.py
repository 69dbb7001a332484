"""Host-side set-up (lattice generator, wall normals, kernel constants) against the oracle."""
import numpy as np
import pytest

from oracle import oracle as O
from sphinxsys_gb300 import cases
from sphinxsys_gb300 import sph as S


def host_bodies(case):
    d = case.dim
    water = S.ComplexShape().add(S.GeometricShapeBox(case.water_center[:d], case.water_halfsize[:d]))
    wall = S.ComplexShape()
    wall.add(S.GeometricShapeBox(case.outer_center[:d], case.outer_halfsize[:d]))
    wall.subtract(S.GeometricShapeBox(case.inner_center[:d], case.inner_halfsize[:d]))
    fp = S.lattice_positions(d, case.sys_lower, case.sys_upper, case.dp, water)
    wp = S.lattice_positions(d, case.sys_lower, case.sys_upper, case.dp, wall)
    return fp, wp, wall.normal_direction(wp)


@pytest.mark.parametrize("case", [cases.dambreak_2d(), cases.dambreak_3d_reference(), cases.dambreak_3d(0.05)],
                         ids=lambda c: c.name)
def test_lattice_and_normals_match_oracle_bitwise(case):
    fp, wp, wn = host_bodies(case)
    oc = O.OracleCase(case)
    assert np.array_equal(fp, oc.get("Position", O.FLUID))
    assert np.array_equal(wp, oc.get("Position", O.WALL))
    assert np.array_equal(wn, oc.get("NormalDirection", O.WALL))


def test_dambreak_2d_particle_counts():
    fp, wp, _ = host_bodies(cases.dambreak_2d())
    assert len(fp) == 3200 and len(wp) == 3504


def test_benchmark_3d_fluid_counts_follow_lattice_rule():
    # fluid lattice counts of the benchmark tank (cell centres inside the water block)
    for dp, expect in ((0.0075, 160 * 133 * 80), (0.006, 200 * 167 * 100)):
        c = cases.dambreak_3d(dp)
        water = S.GeometricShapeBox(c.water_center, c.water_halfsize)
        counts = []
        for a in range(3):
            n = int(np.ceil((c.sys_upper[a] - c.sys_lower[a]) / dp))
            x = (c.sys_lower[a] + np.arange(n) * dp) + 0.5 * dp
            counts.append(int(np.sum(np.abs(x - water.c[a]) <= water.hs[a])))
        assert counts[0] * counts[1] * counts[2] == expect


def test_kernel_constants_match_oracle():
    import ctypes
    from sphinxsys_gb300 import native
    case = cases.dambreak_2d()
    oc = O.OracleCase(case)
    s = ctypes.c_double()
    native.call("sphx_lattice_number_density", 2, case.h, case.dp, ctypes.byref(s))
    assert s.value == oc.constant("sigma0")
    s3 = ctypes.c_double()
    native.call("sphx_lattice_number_density", 3, 1.3 * 0.05, 0.05, ctypes.byref(s3))
    assert abs(s3.value - O.lib().orc_lattice_number_density(3, 1.3 * 0.05, 0.05)) <= 1e-12 * s3.value
    lo, gs, ac = oc.mesh()
    md = native.MeshDesc()
    l3 = (ctypes.c_double * 3)(*case.sys_lower)
    u3 = (ctypes.c_double * 3)(*case.sys_upper)
    native.call("sphx_mesh_from_bounds", 2, l3, u3, 2 * case.h, 2, ctypes.byref(md))
    assert tuple(md.all_cells)[:2] == ac[:2] and md.grid_spacing == gs
    assert list(md.lower)[:2] == list(lo[:2])
    assert oc.constant("contact_depth") == 2
