"""Bounds-checked build (-DSPHX_CHECK).

The checked library tests every neighbour-list entry, cell-list range and cell index the
kernels read through (counting and skipping a failed one).  The same workload runs in a
child process on each library: every solver form (FP64 drop-in with observer, mixed
precision with all seven neighbour strategies in 2D and 3D, periodic Taylor-Green, the
batch, the CK numerics).  The checked run must record no failed test and give the same
results bit for bit (the tests add branches, never arithmetic)."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

WORKLOAD = r"""
import hashlib, json
import numpy as np
from sphinxsys_gb300 import cases, native
from sphinxsys_gb300.batch import BatchDamBreak
from sphinxsys_gb300.dambreak import DamBreak, DamBreakCK, MixedPrecisionDamBreak
from sphinxsys_gb300.taylor_green import MixedPrecisionTaylorGreen

digest = hashlib.sha256()
def add(*arrays):
    for a in arrays:
        digest.update(np.ascontiguousarray(a).tobytes())

sim = DamBreak(cases.dambreak_2d())
for _ in range(3):
    sim.advection_step()
add(sim.water_block.download("Position"), sim.recorded_pressure.exec())
for case in (cases.dambreak_2d(), cases.dambreak_3d(0.04)):
    for strategy in range(7):
        mp = MixedPrecisionDamBreak(case, strategy=strategy)
        for _ in range(3):
            mp.advection_step()
        mp.sync_fp64()
        add(mp.fp64.water_block.download("Position"), mp.observe_pressure())
tg = MixedPrecisionTaylorGreen(cases.TaylorGreenCase("taylor_green3d_16", 3, 2.0 * np.pi, 2.0 * np.pi / 16, 1))
for _ in range(3):
    tg.advection_step()
tg.download()
add(tg.water_block.download("Position"))
insts = [c for c in cases.batch_instances(12, seed=1, n_min=1500, n_max=6000) if c.dim == 3][:3]
bt = BatchDamBreak(insts)
for _ in range(3):
    bt.advection_step()
for q in range(len(insts)):
    add(*bt.download(q))
ck = DamBreakCK(cases.dambreak_2d())
for _ in range(40):
    ck.acoustic_step()
add(ck.water_block.download("Position"))
count, site, value = native.check_violations()
print(json.dumps({"checked": native.load().sphx_checked_build(), "violations": count, "site": site,
                  "value": value, "digest": digest.hexdigest()}))
"""


def run_workload(checked: bool) -> dict:
    env = dict(os.environ, SPHX_CHECKED_BUILD="1" if checked else "0", PYTHONPATH=ROOT)
    r = subprocess.run([sys.executable, "-c", WORKLOAD], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_checked_build_finds_no_bad_index_and_matches_the_unchecked_build():
    from sphinxsys_gb300 import build
    build.build(checked=True)
    checked = run_workload(True)
    plain = run_workload(False)
    print(checked, plain)
    assert checked["checked"] == 1 and plain["checked"] == 0
    assert checked["violations"] == 0, checked
    assert plain["violations"] == 0
    assert checked["digest"] == plain["digest"]
