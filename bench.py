"""Benchmark: particle-steps/s of the weakly-compressible dam-break step on one GB300.

Workload (default): the 3D dam break of a 3.2 x 1.0 x 1.8 tank with a 1.2 x 1.0 x 0.6
water block, dp = 0.0075 (1,702,400 fluid particles, 4 wall layers), FP64, the
Dambreak.cpp loop.  One bench step is one advection step: advection dt, density
summation, the acoustic sub-steps (1st + 2nd half each), the Morton re-sort every 100
steps, the cell-list rebuild and the configuration update.  particle-steps/s counts
fluid particles x acoustic sub-steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--dp DP]

Under torchrun each rank advances its own dam break (replicas, weak scaling).
`--impl reference` times the FP64 CPU restatement of the reference (the oracle, OpenMP
over all host cores) on the same workload.
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
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s (1 GB300): mixed-prec vs FP64 at <=1e-4 rel err; %HBM roofline"
UNIT = "particle-steps/s"


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
        try:
            self.tmp = tempfile.NamedTemporaryFile(mode="w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.tmp, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

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


def algorithmic_bytes_2nd_half(n_fluid: int, n_wall_active: int, nnz: int) -> int:
    """Integration2ndHalf, FP64 3D: 136 B per fluid particle (read x, v, rho, drho, Vol;
    write x, rho, drho, F), 80 B per active wall particle (x, V, v_ave, n) and 4 B per
    stored neighbour index."""
    return 136 * n_fluid + 80 * n_wall_active + 4 * nnz


def algorithmic_bytes_mp_second(n_fluid: int, n_wall_active: int, nnz: int) -> int:
    """Mixed-precision 2nd half, 3D: per fluid particle read cell+off0 (16), vel (12),
    off (12), drho (4), drho_dt (4) and write off (12), drho (4), drho_dt (4), force (12)
    = 80 B; per active wall particle cell+off (16) and normal (12) = 28 B; 4 B per stored
    neighbour index."""
    return 80 * n_fluid + 28 * n_wall_active + 4 * nnz


def mixed_precision_leg(args, torch, local):
    """FP64 and mixed precision on the same case (default dp = 0.006, 3,340,000 fluid
    particles) from the same initial state: particle-steps/s of both, the sweep-kernel
    roofline of the mixed solver, and the field / probe errors of mixed against FP64."""
    from sphinxsys_gb300 import cases
    from sphinxsys_gb300.dambreak import MixedPrecisionDamBreak
    case = cases.dambreak_3d(args.mp_dp)
    mp = MixedPrecisionDamBreak(case, device=local)
    ref = mp.fp64  # the FP64 set-up doubles as the FP64 reference run
    n = ref.water_block.n
    ext = torch.cuda.ExternalStream(mp.ctx.stream())
    steps, warm = args.mp_steps, args.warmup

    def timed(step_fn):
        for _ in range(warm):
            step_fn()
        mp.ctx.synchronize()
        with torch.cuda.stream(ext):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record()
        subs = 0
        for _ in range(steps):
            subs += step_fn()[0]
        with torch.cuda.stream(ext):
            b.record()
        mp.ctx.synchronize()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / 1e3, subs

    mp.set_profiling(True)
    l0 = mp.ctx.launch_count()
    mp_el, mp_subs = timed(mp.advection_step)
    mp_launches = mp.ctx.launch_count() - l0
    t1, t2, nsweeps = mp.kernel_times()
    sizes = mp.list_sizes()
    mp.set_profiling(False)
    fp_el, fp_subs = timed(lambda: ref.advection_step()[:2])
    # errors of mixed against FP64 after the same advection steps from the same start
    errs = {}
    for name in ("Position", "Velocity", "Density", "Pressure"):
        a = mp.fp64_view(name)
        b = ref.water_block.download(name)
        errs[name] = float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))
    p_mp = mp.observe_pressure_view()
    p_fp = ref.recorded_pressure.exec()
    vert = case.vertical_axis
    lo = [case.sys_lower[0], case.sys_lower[1], case.sys_lower[2]]
    up = [case.sys_upper[0], case.sys_upper[1], case.sys_upper[2]]
    lo[0], up[0] = case.inner_center[0] + case.inner_halfsize[0] - 0.2, case.inner_center[0] + case.inner_halfsize[0]
    h_mp = mp.upper_front(vert, lo, up)
    from sphinxsys_gb300 import sph as S
    h_fp = S.UpperFrontInAxisDirection(ref.water_block, lo, up, vert).exec()
    hbm = _hbm_peak()[0]
    n_wall_active = int(np.unique(ref.water_wall_contact.neighbors()["j"]).size)
    alg = algorithmic_bytes_mp_second(n, n_wall_active, sizes["nnz_inner"] + sizes["nnz_wall"])
    achieved = alg / (t2 / 1e3) / 1e9
    return {
        "workload": case.name, "n_fluid": n, "steps": steps, "dtype": "f32 pairs + f64 integration",
        "value": n * mp_subs / mp_el, "ms_per_step": 1e3 * mp_el / steps, "acoustic_substeps": mp_subs,
        "fp64_value_same_case": n * fp_subs / fp_el, "fp64_ms_per_step": 1e3 * fp_el / steps,
        "speedup_vs_fp64": (n * mp_subs / mp_el) / (n * fp_subs / fp_el), "gpu_launches": int(mp_launches),
        "roofline": {"bound": "hbm", "kernel": "k_mp_second<3,true>", "achieved": achieved, "peak": hbm,
                     "unit": "GB/s", "frac": achieved / hbm, "algorithmic_bytes": alg, "kernel_ms": t2,
                     "first_half_ms": t1, "sweeps_timed": nsweeps},
        "errors_vs_fp64": {"fields_max_rel": errs, "probe_pressure": [float(x) for x in p_mp],
                           "probe_pressure_fp64": [float(x) for x in p_fp],
                           "free_surface_height": h_mp, "free_surface_height_fp64": h_fp,
                           "free_surface_rel_err": abs(h_mp - h_fp) / abs(h_fp)},
        "lists": sizes,
    }


def _hbm_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
        return float(peaks["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


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
    from sphinxsys_gb300 import cases
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    case = cases.dambreak_3d(args.dp)
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
        "config": {"workload": case.name, "n_fluid": n, "dp": args.dp, "precision": "fp64"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{args.steps} advection steps ({subs} acoustic sub-steps) of {case.name}"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--dp", type=float, default=0.0075)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-threads", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--mp-dp", type=float, default=0.006)
    ap.add_argument("--mp-steps", type=int, default=5)
    ap.add_argument("--no-mixed", action="store_true")
    args = ap.parse_args()
    rank, world, local = dist_info()

    if args.impl == "reference":
        reference_arm(args, rank, world)
        return

    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)

    from sphinxsys_gb300 import cases
    from sphinxsys_gb300.dambreak import DamBreak

    case = cases.dambreak_3d(args.dp)
    sim = DamBreak(case, device=local)
    n_fluid = sim.water_block.n
    ext = torch.cuda.ExternalStream(sim.ctx.stream())

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    for _ in range(args.warmup):
        sim.advection_step()
    # active wall particles and stored neighbour indices for the roofline bytes
    wn = sim.water_wall_contact.neighbors()
    n_wall_active = int(np.unique(wn["j"]).size)
    nnz = int(sim.water_block_inner.neighbors()["counts"].sum()) + int(wn["counts"].sum())

    # per-launch events around the 2nd half (dominant sweep) inside the timed region
    k_events = []
    orig_exec = sim.fluid_density_relaxation.exec

    def timed_exec(dt=0.0):
        with torch.cuda.stream(ext):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record()
            orig_exec(dt)
            b.record()
        k_events.append((a, b))

    sim.fluid_density_relaxation.exec = timed_exec

    sampler = ClockSampler(local)
    barrier()
    sim.ctx.synchronize()
    torch.cuda.synchronize()
    launches0 = sim.ctx.launch_count()
    sampler.start()
    with torch.cuda.stream(ext):
        t_start = torch.cuda.Event(enable_timing=True)
        t_end = torch.cuda.Event(enable_timing=True)
        t_start.record()
    subs = 0
    for _ in range(args.steps):
        s, _, _, _ = sim.advection_step()
        subs += s
    with torch.cuda.stream(ext):
        t_end.record()
    sim.ctx.synchronize()
    torch.cuda.synchronize()
    barrier()
    clocks = sampler.stop()
    launches = sim.ctx.launch_count() - launches0
    elapsed = t_start.elapsed_time(t_end) / 1e3
    sim.fluid_density_relaxation.exec = orig_exec
    k_ms = [a.elapsed_time(b) for a, b in k_events]
    k_avg = sum(k_ms) / len(k_ms) / 1e3 if k_ms else float("nan")

    # aggregate over ranks: total particle-steps over the slowest rank's time
    ps = float(n_fluid * subs)
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ps, elapsed], dtype=torch.float64, device="cuda")
        tot = t.clone()
        dist.all_reduce(tot[:1], op=dist.ReduceOp.SUM)
        mx = t[1:].clone()
        dist.all_reduce(mx, op=dist.ReduceOp.MAX)
        ps, elapsed = float(tot[0]), float(mx[0])
    value = ps / elapsed

    # end to end through the public API: host state in, step, host state out
    e2e = None
    if args.e2e_steps > 0:
        names = [("Position", 3), ("Velocity", 3), ("Force", 3), ("ForcePrior", 3), ("Density", 1),
                 ("DensityChangeRate", 1), ("Mass", 1), ("VolumetricMeasure", 1)]
        host = {nm: sim.water_block.download(nm) for nm, _ in names}
        h2d = sum(a.nbytes for a in host.values())
        d2h = 0
        sim.ctx.synchronize()
        t0 = time.perf_counter()
        esubs = 0
        for _ in range(args.e2e_steps):
            for nm, _ in names:
                sim.water_block.upload(nm, host[nm])
            s, _, _, _ = sim.advection_step()
            esubs += s
            d2h = 0
            for nm in ("Position", "Velocity", "Density", "Pressure"):
                arr = sim.water_block.download(nm)
                d2h += arr.nbytes
                if nm in host:
                    host[nm] = arr
        e_el = time.perf_counter() - t0
        e2e = {"value": n_fluid * esubs / e_el * world, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h)}

    hbm, peak_source = _hbm_peak()
    alg = algorithmic_bytes_2nd_half(n_fluid, n_wall_active, nnz)
    achieved = alg / k_avg / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                "traffic": None, "kernel": "k_interact_2nd<3>", "algorithmic_bytes": alg,
                "kernel_ms": k_avg * 1e3, "peak_source": peak_source}
    prof = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(prof):
        try:
            with open(prof) as f:
                tr = json.load(f).get(f"dambreak3d_dp{args.dp}")
            if tr:
                roofline["traffic"] = tr
        except (OSError, ValueError):
            pass

    n_wall = sim.wall_boundary.n
    del sim
    mixed = None
    if not args.no_mixed:
        mixed = mixed_precision_leg(args, torch, local)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = args.cpu_threads or (os.cpu_count() or 1)
        v, sub, dt = run_cpu_sample(case, threads)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"1 advection step ({sub} acoustic sub-steps, {dt:.1f} s) of {case.name}"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic dam-break lattice",
            "config": {"workload": case.name, "n_fluid": n_fluid, "n_wall": n_wall, "dp": args.dp,
                       "precision": "fp64", "acoustic_substeps": subs, "l2": "inputs larger than L2",
                       "parallelism": f"replicas{world}"},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches),
            "clocks": clocks, "mixed_precision": mixed,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
