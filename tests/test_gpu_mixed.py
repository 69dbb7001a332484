"""Mixed-precision solver against the FP64 GPU path, and its internal consistency.

Tolerance: fields within 1e-4 relative (max |mp - fp64| / max |fp64|) after 20 advection
steps; the stored-list and cell-sweep strategies, and every block size, agree bit for bit
(same pair set, same summation order)."""
import numpy as np
import pytest

from sphinxsys_gb300 import cases
from sphinxsys_gb300.dambreak import DamBreak, MixedPrecisionDamBreak

pytestmark = pytest.mark.gpu

MP_RTOL = 1e-4


def rel_err(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


def run_pair(case, steps):
    ref = DamBreak(case)
    mp = MixedPrecisionDamBreak(case)
    subs = []
    for _ in range(steps):
        s_r, dt_r, _, _ = ref.advection_step()
        s_m, dt_m = mp.advection_step()
        subs.append((s_r, s_m, dt_r, dt_m))
    mp.sync_fp64()
    return ref, mp, subs


@pytest.mark.parametrize("case", [cases.dambreak_2d(), cases.dambreak_3d(0.04)], ids=lambda c: c.name)
def test_mixed_precision_tracks_fp64(case):
    ref, mp, subs = run_pair(case, 20)
    for s_r, s_m, dt_r, dt_m in subs:
        assert abs(s_r - s_m) <= 1
        assert abs(dt_m / dt_r - 1) < 1e-5
    errs = {}
    for name in ("Position", "Velocity", "Density"):
        errs[name] = rel_err(mp.fp64.water_block.download(name), ref.water_block.download(name))
    # pressure error relative to the pressure scale rho0 c0^2 * max |rho/rho0 - 1|
    p_m = mp.fp64.water_block.download("Pressure")
    p_r = ref.water_block.download("Pressure")
    errs["Pressure"] = rel_err(p_m, p_r)
    print(case.name, errs)
    assert errs["Position"] < 1e-6, errs
    assert errs["Velocity"] < MP_RTOL, errs
    assert errs["Density"] < 1e-6, errs
    assert errs["Pressure"] < 1e-3, errs
    cons = mp.conservation()
    m_ref = ref.water_block.download("Mass").sum()
    assert abs(cons[0] / m_ref - 1) < 1e-6
    assert abs(cons[4] / ref.mechanical_energy.exec() - 1) < 1e-5


def test_strategies_and_block_sizes_bitwise_equal():
    case = cases.dambreak_2d()
    outs = []
    for block, strategy in ((128, 0), (64, 0), (256, 1), (96, 1)):
        mp = MixedPrecisionDamBreak(case, block=block, strategy=strategy)
        for _ in range(5):
            mp.advection_step()
        mp.sync_fp64()
        outs.append([mp.fp64.water_block.download(n) for n in ("Position", "Velocity", "Density")])
    for other in outs[1:]:
        for a, b in zip(outs[0], other):
            assert np.array_equal(a, b)


@pytest.mark.parametrize("case, tiles", [
    (cases.dambreak_2d(), [(4, 4, 0), (8, 8, 0), (2, 8, 0)]),
    (cases.dambreak_3d(0.04), [(4, 4, 4), (2, 2, 8), (8, 8, 2), (1, 3, 5)]),
], ids=["2d", "3d"])
def test_tiled_and_async_strategies_bitwise_equal(case, tiles):
    """Strategy 2 (tile windows staged in shared memory, lists of staged indices) and
    strategy 3 (the stored lists with records gathered by cp.async into a shared-memory
    ring) and strategy 4 (the stored lists on persistent warps taking chunks of particles)
    visit the same neighbours in the same order with the same arithmetic as the
    stored lists of strategy 0: equal bit for bit, for every tile shape and block size; so
    does the tile-grouped traversal of strategy 0."""
    def run(block, strategy, tile):
        mp = MixedPrecisionDamBreak(case, block=block, strategy=strategy)
        if tile is not None:
            mp.set_tile(*tile)
        subs = [mp.advection_step()[0] for _ in range(5)]
        mp.sync_fp64()
        return subs, [mp.fp64.water_block.download(n) for n in ("Position", "Velocity", "Density", "Pressure")]

    ref_subs, ref = run(128, 0, None)
    runs = [(128, 0, tiles[0])] + [(b, 2, t) for t in tiles for b in (64, 256)] + [(b, s_, None) for b in (64, 256) for s_ in (3, 4)]
    for block, strategy, tile in runs:
        subs, out = run(block, strategy, tile)
        assert subs == ref_subs, (block, strategy, tile)
        for a, b in zip(ref, out):
            assert np.array_equal(a, b), (block, strategy, tile)


@pytest.mark.parametrize("case", [cases.dambreak_2d(), cases.dambreak_3d(0.04)], ids=lambda c: c.name)
def test_lane_split_strategies_agree_with_stored_lists(case):
    """Strategies 5 and 6 put 2 and 4 lanes on each particle (each lane takes every 2nd /
    4th slot of the stored lists; the lanes' compensated sums are combined by warp
    shuffles): the same pairs summed in another order.  After 5 advection steps the state
    agrees with strategy 0 to the rounding of a re-ordered FP32 sum (1e-5 relative, the
    bound of the re-imported state, whose cells order their particles differently), with
    the same sub-step counts; each lane count gives the same bits for every block size."""
    def run(block, strategy):
        mp = MixedPrecisionDamBreak(case, block=block, strategy=strategy)
        subs = [mp.advection_step()[0] for _ in range(5)]
        mp.sync_fp64()
        return subs, [mp.fp64.water_block.download(n) for n in ("Position", "Velocity", "Density")]

    ref_subs, ref = run(128, 0)
    for strategy in (5, 6):
        subs, out = run(128, strategy)
        assert subs == ref_subs, strategy
        errs = [rel_err(o, r) for o, r in zip(out, ref)]
        print(case.name, strategy, errs)
        assert max(errs) < 1e-5, (strategy, errs)
        subs2, out2 = run(64, strategy)
        assert subs2 == subs
        for a, b in zip(out, out2):
            assert np.array_equal(a, b), strategy


def test_tiled_strategy_rejects_large_tiles():
    from sphinxsys_gb300.native import SphxError
    mp = MixedPrecisionDamBreak(cases.dambreak_2d(), strategy=2)
    with pytest.raises(SphxError):
        mp.set_tile(16, 16, 0)
    mp.set_tile(8, 8, 0)
    mp.advection_step()


def test_mixed_precision_upper_front_and_probe():
    case = cases.dambreak_2d()
    ref, mp, _ = run_pair(case, 10)
    lo, up = (1.5, -1.0), (2.5, 6.0)
    from sphinxsys_gb300 import sph as S
    f_ref = S.UpperFrontInAxisDirection(ref.water_block, lo, up, 1).exec()
    f_mp = mp.upper_front(1, lo, up)
    assert abs(f_mp - f_ref) < 1e-6
    ref.water_block.updateCellLinkedList()
    ref.fluid_observer_contact.updateConfiguration()
    assert np.allclose(mp.observe_pressure(), ref.recorded_pressure.exec(), rtol=1e-3, atol=1e-6)


def test_upload_restores_downloaded_state():
    """sphx_mp_upload of a state written by sphx_mp_download continues the same run.

    Not bit for bit: the re-import orders the particles of a cell by their body index,
    the running solver by their previous position, so FP32 neighbour sums are added in
    another order (a few 1e-7 relative per step)."""
    case = cases.dambreak_2d()
    a = MixedPrecisionDamBreak(case)
    b = MixedPrecisionDamBreak(case)
    for _ in range(3):
        a.advection_step()
        b.advection_step()
    a.sync_fp64()
    b.upload(a.fp64.water_block)  # same state, re-imported
    a.advection_step()
    b.advection_step()
    a.sync_fp64()
    b.sync_fp64()
    for name in ("Position", "Velocity"):
        assert rel_err(b.fp64.water_block.download(name), a.fp64.water_block.download(name)) < 1e-5


def test_configuration_update_deferred_to_next_step():
    """The configuration for the moved positions is built at the start of the next step:
    a download in between leaves the run bit for bit unchanged, and a step that follows an
    upload (whose import already built the configuration) launches no second one."""
    case = cases.dambreak_2d()
    a = MixedPrecisionDamBreak(case)
    b = MixedPrecisionDamBreak(case)
    for _ in range(4):
        a.advection_step()
        b.advection_step()
        b.sync_fp64()
    a.sync_fp64()
    for name in ("Position", "Velocity", "Density"):
        assert np.array_equal(a.fp64.water_block.download(name), b.fp64.water_block.download(name)), name
    ctx = a.ctx
    n0 = ctx.launch_count()
    s_plain, _ = a.advection_step()
    plain = ctx.launch_count() - n0
    a.sync_fp64()
    a.upload(a.fp64.water_block)
    n0 = ctx.launch_count()
    s_up, _ = a.advection_step()
    after_upload = ctx.launch_count() - n0
    # same sub-step count: the launch difference is the configuration update alone
    if s_plain == s_up:
        assert after_upload < plain, (after_upload, plain)


@pytest.mark.parametrize("case", [cases.dambreak_2d(), cases.dambreak_3d(0.04)], ids=lambda c: c.name)
def test_host_rows_load_and_store_like_the_body_path(case):
    """sphx_mp_upload_host loads the state sphx_body_upload + sphx_mp_upload load, and
    sphx_mp_download_host returns the rows sphx_mp_download + sphx_body_download return,
    bit for bit (the copies overlap the configuration build only in time)."""
    a = MixedPrecisionDamBreak(case)
    b = MixedPrecisionDamBreak(case)
    for _ in range(2):  # same history: the last acoustic dt is kept across a load
        a.advection_step()
        b.advection_step()
    a.sync_fp64()
    body = a.fp64.water_block
    rows = {nm: np.ascontiguousarray(body.download(nm)) for nm in
            ("Position", "Velocity", "Force", "Density", "DensityChangeRate")}
    a.upload(body)
    b.upload_host(rows["Position"], rows["Velocity"], rows["Force"], rows["Density"], rows["DensityChangeRate"])
    assert a.advection_step() == b.advection_step()
    a.sync_fp64()
    n, d = a.n_fluid, case.dim
    out = {"Position": np.zeros((n, d)), "Velocity": np.zeros((n, d)), "Density": np.zeros(n),
           "Pressure": np.zeros(n)}
    b.download_host(out["Position"], out["Velocity"], out["Density"], out["Pressure"])
    for name, v in out.items():
        assert np.array_equal(v, a.fp64.water_block.download(name)), name
    again = {k: np.zeros_like(v) for k, v in out.items()}
    a.download_host(again["Position"], again["Velocity"], again["Density"], again["Pressure"])
    for name, v in again.items():
        assert np.array_equal(v, a.fp64.water_block.download(name)), name


@pytest.mark.parametrize("case", [cases.dambreak_2d(), cases.dambreak_3d(0.04)], ids=lambda c: c.name)
def test_registered_host_rows_hold_each_step_result(case):
    """Rows registered with sphx_mp_set_host_rows hold, after every advection step, what
    sphx_mp_download_host returns after it, bit for bit (velocity and pressure copied
    during the last 2nd half, position and density after it); the run itself is the
    same as without rows; unregistered, the rows stay as the last step left them."""
    a = MixedPrecisionDamBreak(case)
    b = MixedPrecisionDamBreak(case)
    n, d = a.n_fluid, case.dim
    rows = {"Position": np.zeros((n, d)), "Velocity": np.zeros((n, d)), "Density": np.zeros(n),
            "Pressure": np.zeros(n)}
    b.set_host_rows(rows["Position"], rows["Velocity"], rows["Density"], rows["Pressure"])
    for _ in range(3):
        assert a.advection_step() == b.advection_step()
        ref = {k: np.zeros_like(v) for k, v in rows.items()}
        a.download_host(ref["Position"], ref["Velocity"], ref["Density"], ref["Pressure"])
        for name, v in rows.items():
            assert np.array_equal(v, ref[name]), name
    kept = {k: v.copy() for k, v in rows.items()}
    b.set_host_rows()
    b.advection_step()
    for name, v in rows.items():
        assert np.array_equal(v, kept[name]), name
    with pytest.raises(ValueError):
        b.set_host_rows(rows["Position"], None, rows["Density"], rows["Pressure"])


def test_autotune_keeps_state():
    """The autotuner restores the state it advanced (whichever of the strategies 0-6 it
    keeps: on this 3,200-particle case the lane-split ones can win, their extra lanes
    filling more of the GPU)."""
    case = cases.dambreak_2d()
    a = MixedPrecisionDamBreak(case)
    b = MixedPrecisionDamBreak(case)
    block, strategy, ms = b.autotune(reps=1)
    assert block in (64, 128, 256) and strategy in range(7) and ms > 0
    b.set_tuning(128, 0)
    for _ in range(3):
        a.advection_step()
        b.advection_step()
    a.sync_fp64()
    b.sync_fp64()
    assert np.array_equal(a.fp64.water_block.download("Position"), b.fp64.water_block.download("Position"))


@pytest.mark.parametrize("case", [cases.dambreak_2d(), cases.dambreak_3d(0.04)], ids=lambda c: c.name)
def test_pruned_search_finds_every_neighbour(case):
    """The mixed solver's lists, built by the pruned sub-cell search from the same positions,
    hold the FP64 relations' pairs: the counts agree up to pairs within rounding of the
    cut-off (FP32 against FP64 membership)."""
    mp = MixedPrecisionDamBreak(case)
    sizes = mp.list_sizes()
    ref = mp.fp64
    n_in = int(ref.water_block_inner.neighbors()["counts"].sum())
    n_w = int(ref.water_wall_contact.neighbors()["counts"].sum())
    assert abs(sizes["nnz_inner"] - n_in) <= max(2, n_in // 100000), (sizes, n_in)
    assert abs(sizes["nnz_wall"] - n_w) <= max(2, n_w // 100000), (sizes, n_w)
