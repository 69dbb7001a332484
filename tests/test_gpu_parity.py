"""Parity of the CUDA path (through the C ABI) with the FP64 oracle.

Bit-exact: cell linked lists (CellOffset and ParticleIndex), neighbour pair sets and
their order, the Morton particle sort.  FP64 fields: relative error at most 1e-10
(max |gpu - oracle| / max |oracle| per variable) after the stated number of steps.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from sphinxsys_gb300 import cases, native
from sphinxsys_gb300.dambreak import DamBreak

pytestmark = pytest.mark.gpu

FIELD_RTOL = 1e-10
GEOM_RTOL = 1e-13


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = max(np.max(np.abs(b)), 1e-300) if b.size else 1.0
    return float(np.max(np.abs(a - b)) / scale) if b.size else 0.0


def compare_fields(sim, oc, names=("Position", "Velocity", "Density", "Pressure", "DensityChangeRate", "Force")):
    errs = {}
    for n in names:
        errs[n] = rel_err(sim.water_block.download(n), oc.get(n))
    return errs


def compare_neighbors(g, o, dim, contact=False):
    assert np.array_equal(g["counts"], o["counts"])
    assert np.array_equal(g["j"], o["j"])
    for k in ("dW", "r") if contact else ("dW",):
        assert rel_err(g[k], o[k]) < GEOM_RTOL, k
    assert rel_err(g["e"], o["e"]) < GEOM_RTOL


@pytest.fixture(scope="module")
def pair_2d():
    case = cases.dambreak_2d()
    return DamBreak(case), O.OracleCase(case)


def test_initial_state_matches(pair_2d):
    sim, oc = pair_2d
    assert sim.water_block.n == oc.n(O.FLUID) == 3200
    assert sim.wall_boundary.n == oc.n(O.WALL) == 3504
    assert np.array_equal(sim.water_block.download("Position"), oc.get("Position"))
    assert np.array_equal(sim.wall_boundary.download("NormalDirection"), oc.get("NormalDirection", O.WALL))
    assert np.array_equal(sim.water_block.download("ForcePrior"), oc.get("ForcePrior"))


def test_cell_lists_bit_exact(pair_2d):
    sim, oc = pair_2d
    for body, b in ((sim.water_block, O.FLUID), (sim.wall_boundary, O.WALL)):
        off, idx = body.cell_list_arrays()
        ooff, oidx = oc.cell_list(b)
        assert np.array_equal(off, ooff)
        assert np.array_equal(idx, oidx)


def test_neighbor_pairs_bit_exact(pair_2d):
    sim, oc = pair_2d
    compare_neighbors(sim.water_block_inner.neighbors(), oc.neighbors(O.INNER), 2)
    compare_neighbors(sim.water_wall_contact.neighbors(), oc.neighbors(O.CONTACT), 2, contact=True)
    g = sim.fluid_observer_contact.neighbors()
    o = oc.neighbors(O.OBSERVER_CONTACT)
    assert np.array_equal(g["j"], o["j"])
    assert rel_err(g["W"], o["W"]) < GEOM_RTOL


def test_time_steps_match(pair_2d):
    sim, oc = pair_2d
    assert abs(sim.fluid_advection_time_step.exec() / oc.advection_time_step() - 1) < 1e-14
    assert abs(sim.fluid_acoustic_time_step.exec() / oc.acoustic_time_step() - 1) < 1e-14


def run_both(sim, oc, steps):
    subs = []
    for _ in range(steps):
        s_g, dt_g, _, _ = sim.advection_step()
        s_o, dt_o, _, _ = oc.advection_step()
        assert s_g == s_o
        assert abs(dt_g / dt_o - 1) < 1e-12
        subs.append(s_g)
    return subs


def test_fields_after_100_acoustic_steps_2d():
    case = cases.dambreak_2d()
    sim, oc = DamBreak(case), O.OracleCase(case)
    subs = run_both(sim, oc, 20)
    assert sum(subs) >= 100
    errs = compare_fields(sim, oc)
    assert max(errs.values()) < FIELD_RTOL, errs
    assert abs(sim.physical_time / oc.physical_time.value - 1) < 1e-13
    # observer probe and mechanical energy
    assert rel_err(sim.recorded_pressure.exec(), oc.observe_pressure()) < 1e-9
    assert abs(sim.mechanical_energy.exec() / oc.total_mechanical_energy() - 1) < 1e-12


def test_particle_sort_and_long_run_2d():
    """101 advection steps: the Morton re-sort at step 100 permutes identically."""
    case = cases.dambreak_2d()
    sim, oc = DamBreak(case), O.OracleCase(case)
    run_both(sim, oc, 101)
    oid, sid = oc.ids(O.FLUID)
    assert np.array_equal(sim.water_block.download("OriginalID"), oid)
    assert np.array_equal(sim.water_block.download("SortedID"), sid)
    assert not np.array_equal(oid, np.arange(len(oid)))
    errs = compare_fields(sim, oc)
    assert max(errs.values()) < 1e-8, errs


def test_particle_sorting_bit_exact_on_shuffled_state():
    case = cases.dambreak_2d()
    sim, oc = DamBreak(case), O.OracleCase(case)
    rng = np.random.default_rng(0)
    x = oc.get("Position") + rng.uniform(-0.5, 0.5, size=(oc.n(O.FLUID), 2))
    oc.set("Position", x)
    sim.water_block.upload("Position", x)
    oc.particle_sorting()
    sim.particle_sorting.exec()
    oid, sid = oc.ids(O.FLUID)
    assert np.array_equal(sim.water_block.download("OriginalID"), oid)
    assert np.array_equal(sim.water_block.download("SortedID"), sid)
    assert np.array_equal(sim.water_block.download("Position"), oc.get("Position"))
    assert np.array_equal(sim.water_block.download("Mass"), oc.get("Mass"))


def test_out_of_domain_and_clustered_positions():
    """Clamped cell hashing for particles outside the mesh, and list growth beyond the
    initial capacity for a compressed cluster."""
    case = cases.dambreak_2d()
    sim, oc = DamBreak(case), O.OracleCase(case)
    rng = np.random.default_rng(1)
    x = oc.get("Position")
    x[:50] += np.array([7.0, -3.0])          # far outside the mesh
    x[100:400] = rng.uniform(1.0, 1.05, size=(300, 2))  # dense cluster: > 24 neighbours
    oc.set("Position", x)
    sim.water_block.upload("Position", x)
    oc.update_cell_linked_list(O.FLUID)
    oc.update_configuration()
    sim.water_block.updateCellLinkedList()
    sim.water_wall_complex.updateConfiguration()
    off, idx = sim.water_block.cell_list_arrays()
    ooff, oidx = oc.cell_list(O.FLUID)
    assert np.array_equal(off, ooff) and np.array_equal(idx, oidx)
    g, o = sim.water_block_inner.neighbors(), oc.neighbors(O.INNER)
    assert o["counts"].max() > 24
    compare_neighbors(g, o, 2)


def test_deterministic_rerun():
    case = cases.dambreak_2d()
    outs = []
    for _ in range(2):
        sim = DamBreak(case)
        for _ in range(5):
            sim.advection_step()
        outs.append([sim.water_block.download(n) for n in ("Position", "Velocity", "Density")])
    for a, b in zip(*outs):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("case", [cases.dambreak_3d_reference(0.05), cases.dambreak_3d(0.04)],
                         ids=lambda c: c.name)
def test_fields_3d(case):
    sim, oc = DamBreak(case), O.OracleCase(case)
    for body, b in ((sim.water_block, O.FLUID), (sim.wall_boundary, O.WALL)):
        off, idx = body.cell_list_arrays()
        ooff, oidx = oc.cell_list(b)
        assert np.array_equal(off, ooff) and np.array_equal(idx, oidx)
    compare_neighbors(sim.water_block_inner.neighbors(), oc.neighbors(O.INNER), 3)
    compare_neighbors(sim.water_wall_contact.neighbors(), oc.neighbors(O.CONTACT), 3, contact=True)
    subs = run_both(sim, oc, 10)
    while sum(subs) < 100:  # at least 100 acoustic steps
        subs += run_both(sim, oc, 1)
    errs = compare_fields(sim, oc)
    assert max(errs.values()) < FIELD_RTOL, errs
    assert rel_err(sim.recorded_pressure.exec(), oc.observe_pressure()) < 1e-9


def pair_lists(counts_len, gpu_relation=None, oracle=None, which=None):
    """Neighbour counts and indices only (the per-pair kernel values of a 1.7M-particle
    relation would take several GB)."""
    counts = np.zeros(counts_len, dtype=np.uint32)
    u32 = C.POINTER(C.c_uint32)
    if gpu_relation is not None:
        total = C.c_size_t()
        native.call("sphx_relation_download", gpu_relation.handle, counts.ctypes.data_as(u32), None, None, None,
                    None, None, C.byref(total))
        j = np.zeros(int(counts.sum()), dtype=np.uint32)
        native.call("sphx_relation_download", gpu_relation.handle, counts.ctypes.data_as(u32), j.ctypes.data_as(u32),
                    None, None, None, None, C.byref(total))
    else:
        O.lib().orc_get_neighbors(oracle.h, which, O._p(counts), None, None, None, None, None)
        j = np.zeros(int(counts.sum()), dtype=np.uint32)
        O.lib().orc_get_neighbors(oracle.h, which, O._p(counts), O._p(j), None, None, None, None)
    return counts, j


def test_fields_at_fp64_config_size():
    """The FP64 drop-in against the oracle on the 3D dam break at dp = 0.0075 (tank
    3.2 x 1.0 x 1.8, 1,702,400 fluid particles): cell lists, inner and wall pair lists equal
    at the start and after 20 advection steps (100+ acoustic steps), fields within 1e-10."""
    import os
    O.set_num_threads(os.cpu_count() or 1)
    case = cases.dambreak_3d(0.0075)
    sim, oc = DamBreak(case), O.OracleCase(case)
    n = sim.water_block.n
    assert n == oc.n(O.FLUID) == 1_702_400

    def same_pairs():
        for rel, which in ((sim.water_block_inner, O.INNER), (sim.water_wall_contact, O.CONTACT)):
            cg, jg = pair_lists(n, gpu_relation=rel)
            co, jo = pair_lists(n, oracle=oc, which=which)
            assert np.array_equal(cg, co) and np.array_equal(jg, jo), which
        off, idx = sim.water_block.cell_list_arrays()
        ooff, oidx = oc.cell_list(O.FLUID)
        assert np.array_equal(off, ooff) and np.array_equal(idx, oidx)

    same_pairs()
    subs = run_both(sim, oc, 20)
    assert sum(subs) >= 100, subs
    errs = compare_fields(sim, oc)
    print(case.name, sum(subs), errs)
    assert max(errs.values()) < FIELD_RTOL, errs
    same_pairs()
    assert rel_err(sim.recorded_pressure.exec(), oc.observe_pressure()) < 1e-9


def test_upper_front_matches_oracle(pair_2d):
    sim, oc = pair_2d
    from sphinxsys_gb300 import sph as S
    lo, up = (1.5, -1.0), (2.5, 6.0)
    g = S.UpperFrontInAxisDirection(sim.water_block, lo, up, 1).exec()
    assert g == oc.upper_front(1, np.array([1.5, -1.0, 0]), np.array([2.5, 6.0, 0]))


def test_exclusive_scan_known_answer(golden):
    torch = pytest.importorskip("torch")
    sim_ctx = DamBreak(cases.dambreak_2d()).ctx
    inp = torch.tensor(golden["exclusive_scan/input"].astype(np.int64), dtype=torch.int32, device="cuda")
    out = torch.zeros_like(inp)
    torch.cuda.synchronize()
    total = C.c_uint32()
    native.call("sphx_exclusive_scan_u32", sim_ctx.h, C.c_void_p(inp.data_ptr()), C.c_void_p(out.data_ptr()),
                inp.numel(), C.byref(total))
    sim_ctx.synchronize()
    assert np.array_equal(out.cpu().numpy(), golden["exclusive_scan/expected"])
    assert total.value == int(golden["exclusive_scan/input"].sum())
    # large ragged scan against numpy
    rng = np.random.default_rng(3)
    v = rng.integers(0, 40, size=1_234_567).astype(np.int32)
    big = torch.tensor(v, device="cuda")
    res = torch.zeros_like(big)
    torch.cuda.synchronize()
    native.call("sphx_exclusive_scan_u32", sim_ctx.h, C.c_void_p(big.data_ptr()), C.c_void_p(res.data_ptr()),
                big.numel(), C.byref(total))
    sim_ctx.synchronize()
    expect = np.concatenate([[0], np.cumsum(v[:-1], dtype=np.int64)])
    assert np.array_equal(res.cpu().numpy().astype(np.int64), expect)


def test_empty_fluid_body():
    from sphinxsys_gb300 import sph as S
    sys_ = S.SPHSystem((-0.1, -0.1), (1.0, 1.0), 0.025)
    empty = S.FluidBody(sys_, S.ComplexShape().add(S.GeometricShapeBox((5.0, 5.0), (0.1, 0.1))))
    empty.defineMatterMaterial(S.WeaklyCompressibleFluid(1.0, 20.0))
    empty.generateParticles(S.Lattice)
    assert empty.n == 0
    inner = S.InnerRelation(empty)
    empty.updateCellLinkedList()
    inner.updateConfiguration()
    off, idx = empty.cell_list_arrays()
    assert off[-1] == 0 and len(idx) == 0
    dt = S.ReduceDynamics(S.AcousticTimeStep, empty).exec()
    assert dt < 0  # ReduceMax over nothing stays at MinReal, as in the reference
