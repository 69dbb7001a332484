"""Batched dam breaks (sphx_batch_*) against the single-case mixed-precision solver.

Each instance of a batch runs the same arithmetic as sphx_mp_* on that case alone (same
cell order, same neighbour order, same per-instance time steps), so its sub-step counts
must be equal and its fields equal within 1e-6 relative (on GB300: bit for bit).  The
graph-driven loop and the host-driven loop run the same kernels and must agree bit for
bit, and an instance's result must not depend on the other instances of its batch."""
import numpy as np
import pytest

from sphinxsys_gb300 import cases
from sphinxsys_gb300.batch import BatchDamBreak
from sphinxsys_gb300.dambreak import MixedPrecisionDamBreak

pytestmark = pytest.mark.gpu

STEPS = 6


def small_instances(dim, count, seed):
    out = [c for c in cases.batch_instances(4 * count, seed=seed, n_min=1500, n_max=9000) if c.dim == dim]
    assert len(out) >= count
    return out[:count]


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def run_single(case, steps):
    mp = MixedPrecisionDamBreak(case)
    subs = [mp.advection_step()[0] for _ in range(steps)]
    mp.sync_fp64()
    body = mp.fp64.water_block
    ids = body.download("OriginalID").astype(np.int64)
    order = np.argsort(ids)
    fields = [body.download(n)[order] for n in ("Position", "Velocity", "Density", "Pressure")]
    return subs, fields, mp.physical_time


@pytest.mark.parametrize("dim", [2, 3])
def test_batch_instances_match_single_case_solver(dim):
    insts = small_instances(dim, 3, seed=1)
    batch = BatchDamBreak(insts)
    subs = np.array([batch.advection_step() for _ in range(STEPS)])
    assert batch.graph_launches() == STEPS
    for q, case in enumerate(insts):
        s_ref, f_ref, t_ref = run_single(case, STEPS)
        assert list(subs[:, q]) == s_ref, (q, subs[:, q], s_ref)
        assert abs(batch.physical_time[q] - t_ref) <= 1e-12 * t_ref
        got = batch.download(q)
        errs = [rel(g, r) for g, r in zip(got, f_ref)]
        print(case.name, len(f_ref[2]), errs)
        assert max(errs[:3]) < 1e-6, errs
        assert errs[3] < 1e-5, errs


def test_graph_and_host_loop_agree_bitwise():
    insts = small_instances(2, 3, seed=2)
    a = BatchDamBreak(insts, use_graph=True)
    b = BatchDamBreak(insts, use_graph=False)
    for _ in range(4):
        sa = a.advection_step()
        sb = b.advection_step()
        assert np.array_equal(sa, sb)
    assert a.graph_launches() == 4 and b.graph_launches() == 0
    assert np.array_equal(a.physical_time, b.physical_time)
    for q in range(len(insts)):
        for x, y in zip(a.download(q), b.download(q)):
            assert np.array_equal(x, y)


def test_instance_independent_of_its_batch():
    insts = small_instances(3, 3, seed=3)
    full = BatchDamBreak(insts)
    alone = BatchDamBreak(insts[1:2])
    for _ in range(4):
        s_full = full.advection_step()
        s_alone = alone.advection_step()
        assert s_full[1] == s_alone[0]
    for x, y in zip(full.download(1), alone.download(0)):
        assert np.array_equal(x, y)


def test_block_sizes_bitwise_equal():
    insts = small_instances(2, 2, seed=4)
    outs = []
    for block in (64, 128, 256):
        b = BatchDamBreak(insts, block=block)
        for _ in range(3):
            b.advection_step()
        outs.append([b.download(q) for q in range(len(insts))])
    for other in outs[1:]:
        for inst_a, inst_b in zip(outs[0], other):
            for x, y in zip(inst_a, inst_b):
                assert np.array_equal(x, y)


def test_batch_rejects_mixed_dimensions():
    insts = [small_instances(2, 1, seed=5)[0], small_instances(3, 1, seed=5)[0]]
    with pytest.raises(ValueError):
        BatchDamBreak(insts)


@pytest.mark.parametrize("use_graph", [True, False])
def test_substep_cap_ends_the_step_with_timeout(use_graph):
    """An instance that needs more acoustic sub-steps than the cap allows stops relaxing; the
    step finishes its configuration update and reports SPHX_ERR_TIMEOUT (the graph's WHILE
    loop ends on the cap, so nothing waits).  Lifting the cap, the batch steps on."""
    from sphinxsys_gb300.native import SphxError
    insts = small_instances(2, 2, seed=6)
    b = BatchDamBreak(insts, use_graph=use_graph)
    first = b.advection_step()
    assert int(first.min()) >= 3, first  # dam breaks take ~5 sub-steps per advection step
    b.set_substep_cap(2)
    with pytest.raises(SphxError) as e:
        b.advection_step()
    assert e.value.code == 6, e.value  # SPHX_ERR_TIMEOUT
    b.set_substep_cap(int(first.max()) + 50)
    again = b.advection_step()
    assert int(again.min()) >= 1
    for q in range(len(insts)):
        for x in b.download(q):
            assert np.all(np.isfinite(x))
    for bad in (0, -1, (1 << 20) + 1):
        with pytest.raises(SphxError):
            b.set_substep_cap(bad)
