"""Dam-break case descriptions (the driver-level parameters of the reference examples).

Each case states the system bounds, particle spacing, the water block and the tank wall
as boxes (centre + half size, the ``Transform(translation)`` + ``halfsize`` pairs the
reference drivers pass to ``GeometricShapeBox``), the material and gravity, and the
observer points.

* ``dambreak_2d`` follows tests/2d_examples/test_2d_dambreak/Dambreak.cpp:13-47,56-73.
* ``dambreak_3d_reference`` follows tests/3d_examples/test_3d_dambreak/dambreak.cpp:11-61
  (y vertical, dp = 0.05; used for the regression-series check).
* ``dambreak_3d`` is the benchmark tank: 3.2 x 1.0 x 1.8 (x, y, z) with a 1.2 x 1.0 x 0.6
  water block at x = 0, z vertical, rho0 = 1, g = 1, U_ref = 2 sqrt(g H), c0 = 10 U_ref,
  4 wall layers.  dp = 0.0075 gives 1,702,400 fluid particles, dp = 0.006 gives 3,340,000.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Sequence, Tuple

Vec = Tuple[float, float, float]


@dataclass
class DamBreakCase:
    name: str
    dim: int
    sys_lower: Vec
    sys_upper: Vec
    dp: float
    water_center: Vec
    water_halfsize: Vec
    outer_center: Vec
    outer_halfsize: Vec
    inner_center: Vec
    inner_halfsize: Vec
    rho0: float
    c0: float
    U_ref: float
    gravity: Vec
    observers: List[Vec] = field(default_factory=list)
    h_ratio: float = 1.3
    # driver loop: 0 = Dambreak.cpp (acoustic dt before the relaxation),
    # 1 = 3D dambreak.cpp (acoustic dt after the relaxation, starting from 0)
    loop_style: int = 0
    vertical_axis: int = 1

    @property
    def h(self) -> float:
        return self.h_ratio * self.dp

    @property
    def gravity_g(self) -> float:
        return math.sqrt(sum(g * g for g in self.gravity))


def _pad(v: Sequence[float]) -> Vec:
    v = list(v) + [0.0] * (3 - len(v))
    return (float(v[0]), float(v[1]), float(v[2]))


def dambreak_2d(dp: float = 0.025) -> DamBreakCase:
    """Dambreak.cpp:13-47: tank 5.366 x 5.366, water 2 x 1, 4 wall layers, probe (DL, 0.2)."""
    DL, DH, LL, LH = 5.366, 5.366, 2.0, 1.0
    BW = dp * 4
    rho0, g = 1.0, 1.0
    U_ref = 2.0 * math.sqrt(g * LH)
    c0 = 10.0 * U_ref
    water_hs = (0.5 * LL, 0.5 * LH)
    outer_hs = (0.5 * DL + BW, 0.5 * DH + BW)
    outer_c = (-BW + outer_hs[0], -BW + outer_hs[1])
    inner_hs = (0.5 * DL, 0.5 * DH)
    return DamBreakCase(
        name=f"dambreak2d_dp{dp}", dim=2,
        sys_lower=_pad((-BW, -BW)), sys_upper=_pad((DL + BW, DH + BW)), dp=dp,
        water_center=_pad(water_hs), water_halfsize=_pad(water_hs),
        outer_center=_pad(outer_c), outer_halfsize=_pad(outer_hs),
        inner_center=_pad(inner_hs), inner_halfsize=_pad(inner_hs),
        rho0=rho0, c0=c0, U_ref=U_ref, gravity=_pad((0.0, -g)),
        observers=[_pad((DL, 0.2))], loop_style=0, vertical_axis=1)


def dambreak_3d_reference(dp: float = 0.05) -> DamBreakCase:
    """test_3d_dambreak/dambreak.cpp:11-61: tank 5.366 x 2 x 0.5 (y up), six wall probes."""
    DL, DH, DW, LL, LH, LW = 5.366, 2.0, 0.5, 2.0, 1.0, 0.5
    BW = dp * 4
    rho0, g = 1.0, 1.0
    U_ref = 2.0 * math.sqrt(g * LH)
    c0 = 10.0 * U_ref
    water_hs = (0.5 * LL, 0.5 * LH, 0.5 * LW)
    outer_hs = (0.5 * DL + BW, 0.5 * DH + BW, 0.5 * DW + BW)
    inner_hs = (0.5 * DL, 0.5 * DH, 0.5 * DW)
    obs = [(DL, y, 0.5 * DW) for y in (0.01, 0.1, 0.2, 0.24, 0.252, 0.266)]
    return DamBreakCase(
        name=f"dambreak3d_ref_dp{dp}", dim=3,
        sys_lower=(-BW, -BW, -BW), sys_upper=(DL + BW, DH + BW, DW + BW), dp=dp,
        water_center=water_hs, water_halfsize=water_hs,
        outer_center=inner_hs, outer_halfsize=outer_hs,
        inner_center=inner_hs, inner_halfsize=inner_hs,
        rho0=rho0, c0=c0, U_ref=U_ref, gravity=(0.0, -g, 0.0),
        observers=obs, loop_style=1, vertical_axis=1)


def dambreak_3d(dp: float = 0.0075) -> DamBreakCase:
    """Benchmark tank 3.2 x 1.0 x 1.8 (z up), water 1.2 x 1.0 x 0.6 at x = 0, 4 wall layers.

    The probe sits on the far wall at (DL, 0.5, 0.2).
    """
    DL, DW, DH = 3.2, 1.0, 1.8
    LL, LW, LH = 1.2, 1.0, 0.6
    BW = dp * 4
    rho0, g = 1.0, 1.0
    U_ref = 2.0 * math.sqrt(g * LH)
    c0 = 10.0 * U_ref
    water_hs = (0.5 * LL, 0.5 * LW, 0.5 * LH)
    inner_hs = (0.5 * DL, 0.5 * DW, 0.5 * DH)
    outer_hs = (0.5 * DL + BW, 0.5 * DW + BW, 0.5 * DH + BW)
    return DamBreakCase(
        name=f"dambreak3d_dp{dp}", dim=3,
        sys_lower=(-BW, -BW, -BW), sys_upper=(DL + BW, DW + BW, DH + BW), dp=dp,
        water_center=water_hs, water_halfsize=water_hs,
        outer_center=inner_hs, outer_halfsize=outer_hs,
        inner_center=inner_hs, inner_halfsize=inner_hs,
        rho0=rho0, c0=c0, U_ref=U_ref, gravity=(0.0, 0.0, -g),
        observers=[(DL, 0.5, 0.2)], loop_style=0, vertical_axis=2)
