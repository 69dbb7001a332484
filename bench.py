"""Benchmark: particle-steps/s of the weakly-compressible dam-break step on one GB300.

Headline workload: the 3D dam break of a 3.2 x 1.0 x 1.8 tank with a 1.2 x 1.0 x 0.6
water block at dp = 0.006 (3,340,000 fluid particles, 2,456,600 wall particles), advanced
by the mixed-precision solver (FP32 pair arithmetic with compensated sums on FP32
positions relative to integer sub-cells; FP64 position integration, re-hash, dt
reductions and conservation sums), timed beside the FP64 path on the same
case from the same initial state, with the field / probe / free-surface errors of mixed
against FP64.  The FP64 drop-in is also measured on dp = 0.0075 (1,702,400 fluid
particles) through the reference-shaped API (``fp64_drop_in``), a seeded batch of 64
independent dam breaks against the same instances run one by one in FP64 (``batch``), and
the 3D periodic Taylor-Green vortex at 256^3 in mixed precision with its kinetic-energy
decay and a few FP64 steps of the same case (``taylor_green``).  ``accuracy_vs_fp64``
runs the headline geometry at dp = 0.02 in both precisions to t = 0.75 and reports the
wall-probe and free-surface errors the 1e-4 bound refers to (the probe on the near wall,
wetted from t = 0).

One bench step is one advection step of the Dambreak.cpp loop: advection dt, density
summation, the acoustic sub-steps (1st + 2nd half each) and the cell-list / configuration
update.  particle-steps/s = fluid particles x acoustic sub-steps / time.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun each rank advances its own dam break (replicas, weak scaling).
`--impl reference` times the FP64 CPU restatement of the reference (the oracle, OpenMP
over all host cores) on the headline case; it never touches a GPU.
"""
from __future__ import annotations

import argparse
import csv
import io
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
DTYPE_MIXED = "f32 pairs, cell-relative f32 positions / f64 position integration, re-hash, dt, sums"
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s (1 GB300): mixed-prec vs FP64 at <=1e-4 rel err; %HBM roofline"
UNIT = "particle-steps/s"


def to_json(obj) -> str:
    """One JSON line; numpy scalars (and anything else with .item()) become Python values."""
    return json.dumps(obj, default=lambda o: o.item() if hasattr(o, "item") else str(o))


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.tmp = None

    def start(self):
        """Starts sampling every 50 ms and returns once the first sample is written (the
        tool takes a while to start), so that the timed region that follows is covered."""
        try:
            self.tmp = tempfile.NamedTemporaryFile(mode="w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=self.tmp, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < 5.0 and self.proc.poll() is None:
            if os.path.getsize(self.tmp.name) > 0:
                break
            time.sleep(0.01)

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.tmp.flush()
        self.tmp.seek(0)
        rows = [r for r in csv.reader(io.StringIO(self.tmp.read())) if len(r) >= 9]
        os.unlink(self.tmp.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if "Active" in r[5 + k] and "Not" not in r[5 + k]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def hbm_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def traffic_of(key):
    """ncu DRAM bytes per launch recorded under profiles/traffic.json, if any."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            return json.load(f).get(key)
    except (OSError, ValueError):
        return None


def bytes_fp64_second(n_fluid: int, n_wall_active: int, nnz: int) -> int:
    """Integration2ndHalf, FP64 3D: 136 B per fluid particle (read x, v, rho, drho, Vol;
    write x, rho, drho, F), 80 B per active wall particle (x, V, v_ave, n), 36 B per stored
    pair: the neighbour index and the configuration-time dW (8 B) and e (24 B) the classic
    neighbourhood keeps for the whole advection step."""
    return 136 * n_fluid + 80 * n_wall_active + 36 * nnz


def bytes_mp_second(n_fluid: int, n_wall_active: int, nnz: int) -> int:
    """Mixed 2nd half, 3D: per fluid particle read geo0 (16), dyn (16), the offset pair
    off + off_lo (24), drho (4), drho_dt (4), write the offset pair (24), drho (4),
    drho_dt (4), force (12) = 108 B; per active wall particle geo (16) and normal (16) =
    32 B; 4 B per stored neighbour index."""
    return 108 * n_fluid + 32 * n_wall_active + 4 * nnz


def timed_steps(torch, ctx, step_fn, steps, warmup, sampler=None):
    ext = torch.cuda.ExternalStream(ctx.stream())
    for _ in range(warmup):
        step_fn()
    ctx.synchronize()
    torch.cuda.synchronize()
    launches0 = ctx.launch_count()
    if sampler:
        sampler.start()
    with torch.cuda.stream(ext):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
    subs = 0
    for _ in range(steps):
        subs += step_fn()[0]
    with torch.cuda.stream(ext):
        b.record()
    ctx.synchronize()
    torch.cuda.synchronize()
    clocks = sampler.stop() if sampler else None
    return a.elapsed_time(b) / 1e3, subs, ctx.launch_count() - launches0, clocks


def mixed_leg(args, torch, local, world):
    from sphinxsys_gb300 import cases
    from sphinxsys_gb300 import sph as S
    from sphinxsys_gb300.dambreak import MixedPrecisionDamBreak
    case = cases.dambreak_3d(args.mp_dp)
    mp = MixedPrecisionDamBreak(case, device=local)
    ref = mp.fp64  # the FP64 set-up is also the FP64 reference run (same initial state)
    n = ref.water_block.n
    tuned = None
    if args.autotune:
        b, st, ms = mp.autotune(reps=2)
        tuned = dict(mp.tuning(), ms_per_substep=ms)
    mp.set_profiling(True)
    el, subs, launches, clocks = timed_steps(torch, mp.ctx, mp.advection_step, args.steps, args.warmup,
                                             ClockSampler(local))
    t1, t2, nsweeps = mp.kernel_times()
    sizes = mp.list_sizes()
    mp.set_profiling(False)
    fp_el, fp_subs, _, _ = timed_steps(torch, mp.ctx, lambda: ref.advection_step()[:2], args.steps, args.warmup)
    # errors of mixed against FP64 after the same advection steps from the same start
    errs = {}
    for name in ("Position", "Velocity", "Density", "Pressure"):
        a = mp.fp64_view(name)
        b = ref.water_block.download(name)
        errs[name] = float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))
    p_mp = mp.observe_pressure_view()
    p_fp = ref.recorded_pressure.exec()
    # a probe the water has not reached reads 0 in both runs: no relative error there
    probes = []
    for pos, a, b in zip(case.observers, p_mp, p_fp):
        wetted = bool(abs(b) > 0.0)
        probes.append({"position": list(pos), "mixed": float(a), "fp64": float(b), "wetted": wetted,
                       "abs_err": abs(float(a) - float(b)),
                       "rel_err": abs(float(a) - float(b)) / abs(float(b)) if wetted else None})
    vert = case.vertical_axis
    lo = list(case.sys_lower)
    up = list(case.sys_upper)
    lo[0], up[0] = case.water_center[0] - case.water_halfsize[0], case.water_center[0] + case.water_halfsize[0]
    h_mp = mp.upper_front(vert, lo, up)
    h_fp = S.UpperFrontInAxisDirection(ref.water_block, lo, up, vert).exec()
    n_wall_active = int(np.unique(ref.water_wall_contact.neighbors()["j"]).size)
    hbm, src = hbm_peak()
    alg = bytes_mp_second(n, n_wall_active, sizes["nnz_inner"] + sizes["nnz_wall"])
    achieved = alg / (t2 / 1e3) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                "traffic": traffic_of("k_mp_second"), "kernel": "k_mp_second<3,lists>", "algorithmic_bytes": alg,
                "kernel_ms": t2, "first_half_ms": t1, "sweeps_timed": nsweeps, "peak_source": src}
    # end to end through the public API: host FP64 state in, one advection step, state out
    e2e = None
    if args.e2e_steps > 0:
        names = ("Position", "Velocity", "Force", "Density", "DensityChangeRate")

        def pinned_like(a):
            t = torch.empty(a.shape, dtype=torch.float64, pin_memory=True).numpy()
            t[...] = a
            return t

        # the caller's state lives in pinned host memory; each step loads it
        # (sphx_mp_upload_host), advances, and the step itself writes the results back
        # into the same buffers (rows registered with sphx_mp_set_host_rows: the velocity
        # and pressure rows copy during the last 2nd half)
        host = {nm: pinned_like(mp.fp64_view(nm)) for nm in names}
        pressure = pinned_like(np.zeros(n))
        outs = {"Position": host["Position"], "Velocity": host["Velocity"], "Density": host["Density"],
                "Pressure": pressure}
        h2d = sum(a.nbytes for a in host.values())
        d2h = sum(a.nbytes for a in outs.values())
        mp.set_host_rows(outs["Position"], outs["Velocity"], outs["Density"], outs["Pressure"])
        for _ in range(2):  # untimed warm-up of the same calls
            mp.upload_host(*(host[nm] for nm in names))
            mp.advection_step()
        mp.ctx.synchronize()
        t0 = time.perf_counter()
        esubs = 0
        for _ in range(args.e2e_steps):
            mp.upload_host(*(host[nm] for nm in names))
            s, _ = mp.advection_step()
            esubs += s
        e_el = time.perf_counter() - t0
        mp.set_host_rows()
        e2e = {"value": n * esubs / e_el * world, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "ms_per_step": 1e3 * e_el / args.e2e_steps,
               "calls": "sphx_mp_upload_host, sphx_mp_advection_step (host rows registered with "
                        "sphx_mp_set_host_rows)"}
    out = {
        "case": case, "n": n, "n_wall": ref.wall_boundary.n, "elapsed": el, "subs": subs, "launches": launches,
        "clocks": clocks, "roofline": roofline, "e2e": e2e, "tuning": tuned,
        "fp64_same_case": {"value": n * fp_subs / fp_el, "ms_per_step": 1e3 * fp_el / args.steps,
                           "acoustic_substeps": fp_subs},
        "speedup_vs_fp64": (n * subs / el) / (n * fp_subs / fp_el),
        "errors_vs_fp64": {"t": ref.physical_time, "fields_max_rel": errs, "probes": probes,
                           "free_surface_height": h_mp, "free_surface_height_fp64": h_fp,
                           "free_surface_rel_err": abs(h_mp - h_fp) / max(abs(h_fp), 1e-300)},
        "lists": sizes,
    }
    del mp, ref
    return out


def accuracy_leg(args):
    """Mixed precision against FP64 where the headline's 1e-4 bound applies: the same
    geometry at dp = args.acc_dp, both solvers from one initial state to t = args.acc_t,
    recorded every 5 advection steps; the near-wall probe at (0, 0.5, 0.2) (wetted from
    t = 0) relative to max(|p_fp64|, 0.1 rho0 g (H - z)), and the free-surface height over
    the initial column (the criteria of tests/test_gpu_accuracy.py)."""
    from sphinxsys_gb300 import cases
    from sphinxsys_gb300 import sph as S
    from sphinxsys_gb300.dambreak import DamBreak, MixedPrecisionDamBreak
    case = cases.dambreak_3d(args.acc_dp)
    k = case.observers.index((0.0, 0.5, 0.2))
    lo, up = list(case.sys_lower), list(case.sys_upper)
    lo[0] = case.water_center[0] - case.water_halfsize[0]
    up[0] = case.water_center[0] + case.water_halfsize[0]
    mp = MixedPrecisionDamBreak(case)
    rows_m, steps = [], 0
    while mp.physical_time < args.acc_t:
        mp.advection_step()
        steps += 1
        if steps % 5 == 0:
            rows_m.append((float(mp.observe_pressure_view()[k]), mp.upper_front(case.vertical_axis, lo, up)))
    del mp
    sim = DamBreak(case)
    rows_f = []
    for s_ in range(1, steps + 1):
        sim.advection_step()
        if s_ % 5 == 0:
            rows_f.append((float(sim.recorded_pressure.exec()[k]),
                           S.UpperFrontInAxisDirection(sim.water_block, lo, up, case.vertical_axis).exec()))
    floor = 0.1 * case.rho0 * case.gravity_g * (2.0 * case.water_halfsize[2] - case.observers[k][2])
    p_rel = [abs(a[0] - b[0]) / max(abs(b[0]), floor) for a, b in zip(rows_m, rows_f)]
    fs_rel = [abs(a[1] / b[1] - 1.0) for a, b in zip(rows_m, rows_f)]
    return {"workload": case.name, "t_end": sim.physical_time, "advection_steps": steps, "records": len(p_rel),
            "probe": list(case.observers[k]), "probe_max_rel_err": max(p_rel), "probe_max_abs_err":
            max(abs(a[0] - b[0]) for a, b in zip(rows_m, rows_f)), "free_surface_max_rel_err": max(fs_rel),
            "bound": 1e-4, "within_bound": max(p_rel) <= 1e-4 and max(fs_rel) <= 1e-4}


def fp64_leg(args, torch, local):
    """The FP64 drop-in (reference-shaped calls) on dp = args.dp; per-launch CUDA events
    around every 2nd-half call inside the timed region give the roofline kernel time."""
    from sphinxsys_gb300 import cases
    from sphinxsys_gb300.dambreak import DamBreak
    case = cases.dambreak_3d(args.dp)
    sim = DamBreak(case, device=local)
    n = sim.water_block.n
    ext = torch.cuda.ExternalStream(sim.ctx.stream())
    for _ in range(args.warmup):
        sim.advection_step()
    wn = sim.water_wall_contact.neighbors()
    n_wall_active = int(np.unique(wn["j"]).size)
    nnz = int(sim.water_block_inner.neighbors()["counts"].sum()) + int(wn["counts"].sum())
    events = []
    orig = sim.fluid_density_relaxation.exec

    def timed_exec(dt=0.0):
        with torch.cuda.stream(ext):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record()
            orig(dt)
            b.record()
        events.append((a, b))

    sim.fluid_density_relaxation.exec = timed_exec
    el, subs, launches, _ = timed_steps(torch, sim.ctx, lambda: sim.advection_step()[:2], args.fp64_steps, 0)
    sim.fluid_density_relaxation.exec = orig
    k_ms = sum(a.elapsed_time(b) for a, b in events) / max(len(events), 1)
    hbm, src = hbm_peak()
    alg = bytes_fp64_second(n, n_wall_active, nnz)
    achieved = alg / (k_ms / 1e3) / 1e9
    out = {"workload": case.name, "n_fluid": n, "dtype": "f64", "value": n * subs / el,
           "ms_per_step": 1e3 * el / args.fp64_steps, "steps": args.fp64_steps, "acoustic_substeps": subs,
           "gpu_launches": int(launches),
           "roofline": {"bound": "fp64 pipe (reported against hbm)", "achieved": achieved, "peak": hbm,
                        "unit": "GB/s", "frac": achieved / hbm, "traffic": traffic_of("k_interact_2nd"),
                        "kernel": "k_interact_2nd<3>", "algorithmic_bytes": alg, "kernel_ms": k_ms,
                        "peak_source": src}}
    del sim
    return out


def batch_leg(args, torch, local):
    """Seeded batch of independent 2D / 3D dam breaks (N log-uniform in [2e4, 5e5], aspect
    H/L uniform in [0.25, 1], std::mt19937_64 seed 0), one BatchDamBreak per dimension,
    each advection step one CUDA graph launch.  Aggregate particle-steps/s = sum over
    instances of fluid particles x acoustic sub-steps / time, against the same instances
    run one after another through the FP64 drop-in path (a bounded sample of steps)."""
    from sphinxsys_gb300 import cases
    from sphinxsys_gb300.batch import BatchDamBreak
    from sphinxsys_gb300.dambreak import DamBreak
    insts = cases.batch_instances(args.batch_count, seed=0)
    groups = {}
    ps_graph = el_graph = ps_host = el_host = 0.0
    launches = 0
    for d in (2, 3):
        cs = [c for c in insts if c.dim == d]
        if not cs:
            continue
        b = BatchDamBreak(cs, device=local)
        nq = np.asarray(b.n_fluid, dtype=np.float64)
        stream = torch.cuda.ExternalStream(b.ctx.stream())

        def run(k, use_graph):
            b.ctx.synchronize()
            l0 = b.ctx.launch_count()
            with torch.cuda.stream(stream):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record()
            ps = 0.0
            for _ in range(k):
                ps += float(np.dot(nq, b.advection_step(use_graph)))
            with torch.cuda.stream(stream):
                e1.record()
            b.ctx.synchronize()
            torch.cuda.synchronize()
            return ps, e0.elapsed_time(e1) / 1e3, b.ctx.launch_count() - l0

        tune = {}
        for blk in (64, 128, 256):  # block-size autotune, one step each after a graph build
            b.set_tuning(blk)
            b.advection_step()
            ps, el, _ = run(1, True)
            tune[blk] = el / max(ps, 1.0)
        blk = min(tune, key=tune.get)
        b.set_tuning(blk)
        for _ in range(max(args.warmup - 3, 1)):
            b.advection_step()
        ps, el, ln = run(args.batch_steps, True)
        ps_graph += ps
        el_graph += el
        launches += ln
        hps, hel, _ = run(args.batch_steps, False)
        ps_host += hps
        el_host += hel
        nf, nw = b.size()
        groups[f"{d}d"] = {"instances": len(cs), "n_fluid": int(nf), "n_wall": int(nw), "block": blk,
                           "graph": {"value": ps / el, "ms_per_step": 1e3 * el / args.batch_steps},
                           "host_loop": {"value": hps / hel, "ms_per_step": 1e3 * hel / args.batch_steps}}
        del b
    # the same instances, one after another, through the FP64 drop-in path
    fp_ps = fp_el = 0.0
    for c in insts:
        sim = DamBreak(c, device=local)
        n = sim.water_block.n
        for _ in range(args.batch_fp64_warmup):
            sim.advection_step()
        el, subs, _, _ = timed_steps(torch, sim.ctx, lambda: sim.advection_step()[:2], args.batch_fp64_steps, 0)
        fp_ps += n * subs
        fp_el += el
        del sim
    value = ps_graph / el_graph
    return {"workload": f"batch{len(insts)}_seed0", "instances": len(insts), "value": value, "unit": UNIT,
            "steps": args.batch_steps, "gpu_launches": int(launches), "groups": groups,
            "host_loop_value": ps_host / el_host,
            "fp64_sequential": {"value": fp_ps / fp_el, "steps_per_instance": args.batch_fp64_steps,
                                "sample": f"{args.batch_fp64_steps} advection steps of each instance"},
            "speedup_vs_fp64_sequential": value / (fp_ps / fp_el)}


def bytes_mp_second_periodic(n_fluid: int, nnz: int) -> int:
    """Mixed 2nd half of the periodic flow, 3D: per particle read geo0 (16), dyn (16), the
    offset pair (24), drho (4), drho_dt (4), prior force (12), write the offset pair (24),
    drho (4), drho_dt (4), force (12) = 120 B; 4 B per stored neighbour entry."""
    return 120 * n_fluid + 4 * nnz


def taylor_green_leg(args, torch, local):
    """The 3D periodic Taylor-Green vortex on [0, 2 pi]^3 at args.tg_resolution^3 particles
    (Re = 100, rho0 = 1, c0 = 10, transport-velocity correction), mixed precision: warm-up
    and timed advection steps, the kinetic energy after each, its decay against
    exp(-6 nu t) (the linearised decay, |k|^2 = 3), then the FP64 drop-in on the same case
    from the same initial state for args.tg_fp64_steps steps (kinetic-energy error of mixed
    against FP64 at equal step counts, and the FP64 throughput)."""
    from sphinxsys_gb300 import cases
    from sphinxsys_gb300.taylor_green import MixedPrecisionTaylorGreen, TaylorGreen
    case = cases.taylor_green_3d(args.tg_resolution)
    t0 = time.perf_counter()
    mp = MixedPrecisionTaylorGreen(case, device=local)
    setup_s = time.perf_counter() - t0
    n = mp.n_fluid
    ctx = mp.water_block.system.ctx
    nu = case.mu / case.rho0
    ke = [mp.kinetic_energy()]
    times = [0.0]
    tuned = mp.autotune(reps=1) if args.autotune else None

    def step():
        r = mp.advection_step()
        return r

    for _ in range(args.warmup):
        step()
        ke.append(mp.kinetic_energy())
        times.append(mp.physical_time)
    mp.set_profiling(True)
    el, subs, launches, _ = timed_steps(torch, ctx, step, args.tg_steps, 0)
    t1, t2, nsweeps = mp.kernel_times()
    mp.set_profiling(False)
    ke.append(mp.kinetic_energy())
    times.append(mp.physical_time)
    sizes = mp.list_sizes()
    hbm, src = hbm_peak()
    alg = bytes_mp_second_periodic(n, sizes["nnz_inner"])
    achieved = alg / (t2 / 1e3) / 1e9
    decay = {"t": times[-1], "ke_ratio": ke[-1] / ke[0], "analytic": float(np.exp(-6.0 * nu * times[-1]))}
    decay["rel_err"] = decay["ke_ratio"] / decay["analytic"] - 1.0
    total_steps = args.warmup + args.tg_steps
    del mp
    fp64 = None
    if args.tg_fp64_steps > 0:
        ref = TaylorGreen(case, device=local)
        ke_fp = [ref.kinetic_energy.exec()]
        fsteps = min(args.tg_fp64_steps, total_steps)
        fel, fsubs, _, _ = timed_steps(torch, ref.water_block.system.ctx, ref.advection_step, fsteps, 0)
        ke_fp.append(ref.kinetic_energy.exec())
        # the mixed run's energy after the same number of advection steps
        ke_mp = ke[fsteps] if fsteps <= args.warmup else None
        fp64 = {"value": n * fsubs / fel, "ms_per_step": 1e3 * fel / fsteps, "steps": fsteps,
                "ke_rel_err_mixed_vs_fp64": (abs(ke_mp / ke_fp[-1] - 1.0) if ke_mp is not None else None)}
        del ref
    return {"workload": case.name, "n_fluid": n, "dtype": DTYPE_MIXED, "value": n * subs / el,
            "unit": UNIT, "ms_per_step": 1e3 * el / args.tg_steps, "steps": args.tg_steps, "warmup": args.warmup,
            "acoustic_substeps": subs, "gpu_launches": int(launches), "tuning": tuned, "setup_s": setup_s,
            "kinetic_energy_decay": decay,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                         "kernel": "k_mp_second_periodic<3,lists>", "algorithmic_bytes": alg, "kernel_ms": t2,
                         "first_half_ms": t1, "sweeps_timed": nsweeps, "peak_source": src,
                         "traffic": traffic_of("k_mp_second_periodic")},
            "fp64_same_case": fp64,
            "speedup_vs_fp64": (n * subs / el) / fp64["value"] if fp64 else None}


def run_cpu_sample(case, threads: int):
    """One advection step of the oracle (OpenMP FP64 restatement) on the same case."""
    from oracle import oracle as O
    O.set_num_threads(threads)
    oc = O.OracleCase(case)
    t0 = time.perf_counter()
    sub, _, _, _ = oc.advection_step()
    dt = time.perf_counter() - t0
    return oc.n(O.FLUID) * sub / dt, sub, dt


def reference_arm(args, rank, world):
    """The reference's CPU path: the FP64 oracle over all host cores on the headline case."""
    from sphinxsys_gb300 import cases
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    case = cases.dambreak_3d(args.mp_dp)
    from oracle import oracle as O
    O.set_num_threads(threads)
    oc = O.OracleCase(case)
    n = oc.n(O.FLUID)
    for _ in range(args.warmup):
        oc.advection_step()
    t0 = time.perf_counter()
    subs = 0
    for _ in range(args.steps):
        s, _, _, _ = oc.advection_step()
        subs += s
    el = time.perf_counter() - t0
    v = n * subs / el
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * el / max(args.steps, 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic dam-break lattice",
        "config": {"workload": case.name, "n_fluid": n, "n_wall": oc.n(O.WALL), "dp": args.mp_dp,
                   "precision": "fp64", "parallelism": "rank 0 only, OpenMP over the host cores"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{args.steps} advection steps ({subs} acoustic sub-steps) of {case.name}"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(to_json(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--mp-dp", type=float, default=0.006, help="headline (mixed-precision) case spacing")
    ap.add_argument("--dp", type=float, default=0.0075, help="FP64 drop-in case spacing")
    ap.add_argument("--fp64-steps", type=int, default=5)
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--cpu-threads", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--autotune", type=int, default=1)
    ap.add_argument("--batch-count", type=int, default=64, help="instances of the batched leg (0 = skip)")
    ap.add_argument("--batch-steps", type=int, default=5)
    ap.add_argument("--batch-fp64-steps", type=int, default=3)
    ap.add_argument("--batch-fp64-warmup", type=int, default=1)
    ap.add_argument("--tg-resolution", type=int, default=256, help="Taylor-Green particles per side (0 = skip)")
    ap.add_argument("--tg-steps", type=int, default=10)
    ap.add_argument("--tg-fp64-steps", type=int, default=3)
    ap.add_argument("--acc-dp", type=float, default=0.02, help="accuracy leg spacing (0 = skip)")
    ap.add_argument("--acc-t", type=float, default=0.75, help="accuracy leg end time")
    args = ap.parse_args()
    rank, world, local = dist_info()

    if args.impl == "reference":
        reference_arm(args, rank, world)
        return

    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        dist.barrier()
    torch.cuda.set_device(local)

    mixed = mixed_leg(args, torch, local, world)
    el = mixed["elapsed"]
    ps = float(mixed["n"] * mixed["subs"])
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ps], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        m = torch.tensor([el], dtype=torch.float64, device="cuda")
        dist.all_reduce(m, op=dist.ReduceOp.MAX)
        ps, el = float(t[0]), float(m[0])
    fp64 = None if args.no_fp64 else fp64_leg(args, torch, local)
    batch = batch_leg(args, torch, local) if args.batch_count > 0 else None
    taylor_green = taylor_green_leg(args, torch, local) if args.tg_resolution > 0 else None
    accuracy = accuracy_leg(args) if args.acc_dp > 0 and rank == 0 else None

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        from sphinxsys_gb300 import cases
        threads = args.cpu_threads or (os.cpu_count() or 1)
        v, sub, dt = run_cpu_sample(cases.dambreak_3d(args.mp_dp), threads)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"1 advection step ({sub} acoustic sub-steps, {dt:.1f} s) of {mixed['case'].name}"}

    if rank == 0:
        case = mixed["case"]
        line = {
            "metric": METRIC, "value": ps / el, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": DTYPE_MIXED,
            "data": "synthetic dam-break lattice",
            "config": {"workload": case.name, "n_fluid": mixed["n"], "n_wall": mixed["n_wall"], "dp": args.mp_dp,
                       "precision": "mixed", "acoustic_substeps": mixed["subs"], "l2": "inputs larger than L2",
                       "parallelism": f"replicas{world}", "tuning": mixed["tuning"]},
            "roofline": mixed["roofline"], "cpu_baseline": cpu, "e2e": mixed["e2e"],
            "gpu_launches": int(mixed["launches"]), "clocks": mixed["clocks"],
            "mixed_precision": {"speedup_vs_fp64_same_case": mixed["speedup_vs_fp64"],
                                "fp64_same_case": mixed["fp64_same_case"],
                                "errors_vs_fp64": mixed["errors_vs_fp64"], "lists": mixed["lists"],
                                "accuracy_vs_fp64": accuracy},
            "fp64_drop_in": fp64,
            "batch": batch,
            "taylor_green": taylor_green,
        }
        print(to_json(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
