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

    Two wall-pressure probes at z = 0.2: on the far wall at (DL, 0.5, 0.2), where the water
    arrives at impact (t ~ 1.3), and on the near wall at (0, 0.5, 0.2), inside the initial
    column, wetted from t = 0.
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
        observers=[(DL, 0.5, 0.2), (0.0, 0.5, 0.2)], loop_style=0, vertical_axis=2)


class MT19937_64:
    """64-bit Mersenne Twister (Matsumoto & Nishimura, 2000) as std::mt19937_64 defines it,
    so batch draws follow the stated seed exactly."""

    N, M = 312, 156
    MATRIX_A = 0xB5026F5AA96619E9
    UPPER, LOWER = 0xFFFFFFFF80000000, 0x7FFFFFFF
    MASK = (1 << 64) - 1

    def __init__(self, seed: int = 5489):
        self.mt = [0] * self.N
        self.mt[0] = seed & self.MASK
        for i in range(1, self.N):
            prev = self.mt[i - 1]
            self.mt[i] = (6364136223846793005 * (prev ^ (prev >> 62)) + i) & self.MASK
        self.idx = self.N

    def _twist(self):
        mt = self.mt
        for i in range(self.N):
            x = (mt[i] & self.UPPER) | (mt[(i + 1) % self.N] & self.LOWER)
            xa = x >> 1
            if x & 1:
                xa ^= self.MATRIX_A
            mt[i] = mt[(i + self.M) % self.N] ^ xa
        self.idx = 0

    def __call__(self) -> int:
        if self.idx >= self.N:
            self._twist()
        y = self.mt[self.idx]
        self.idx += 1
        y ^= (y >> 29) & 0x5555555555555555
        y ^= (y << 17) & 0x71D67FFFEDA60000
        y ^= (y << 37) & 0xFFF7EEE000000000
        y ^= y >> 43
        return y & self.MASK

    def uniform(self) -> float:
        """std::generate_canonical<double, 53> over one 64-bit draw (libstdc++)."""
        return self() / 18446744073709551616.0


def batch_instances(count: int = 64, seed: int = 0, n_min: float = 2e4, n_max: float = 5e5):
    """Independent dam breaks for the batched solver: per instance, fluid particle count
    N log-uniform in [n_min, n_max], column aspect H/L uniform in [0.25, 1], and the
    dimension (2D if the draw is below 0.5) from one std::mt19937_64(seed) stream.

    Geometry per instance: water column H = 1 (as Dambreak.cpp), L = H / aspect (and width
    W = L / 2 in 3D); dp from N and the column volume; tank DL = 2.683 L, DH = 5.366 H (the
    Dambreak.cpp tank-to-column ratios), DW = W in 3D; U_ref = 2 sqrt(g H), c0 = 10 U_ref."""
    rng = MT19937_64(seed)
    out = []
    for k in range(count):
        n = round(math.exp(math.log(n_min) + rng.uniform() * (math.log(n_max) - math.log(n_min))))
        aspect = 0.25 + 0.75 * rng.uniform()
        dim = 2 if rng.uniform() < 0.5 else 3
        H = 1.0
        L = H / aspect
        if dim == 2:
            dp = math.sqrt(L * H / n)
            case = _column_case(f"batch{k}_2d", 2, L, H, 0.0, dp)
        else:
            W = 0.5 * L
            dp = (L * H * W / n) ** (1.0 / 3.0)
            case = _column_case(f"batch{k}_3d", 3, L, H, W, dp)
        out.append(case)
    return out


def _column_case(name: str, dim: int, L: float, H: float, W: float, dp: float) -> DamBreakCase:
    DL, DH = 2.683 * L, 5.366 * H
    BW = 4 * dp
    g = 1.0
    U_ref = 2.0 * math.sqrt(g * H)
    c0 = 10.0 * U_ref
    if dim == 2:
        water_hs = (0.5 * L, 0.5 * H)
        outer_hs = (0.5 * DL + BW, 0.5 * DH + BW)
        inner_hs = (0.5 * DL, 0.5 * DH)
        return DamBreakCase(
            name=name, dim=2, sys_lower=_pad((-BW, -BW)), sys_upper=_pad((DL + BW, DH + BW)), dp=dp,
            water_center=_pad(water_hs), water_halfsize=_pad(water_hs),
            outer_center=_pad(inner_hs), outer_halfsize=_pad(outer_hs),
            inner_center=_pad(inner_hs), inner_halfsize=_pad(inner_hs),
            rho0=1.0, c0=c0, U_ref=U_ref, gravity=_pad((0.0, -g)), observers=[_pad((DL, 0.2 * H))],
            loop_style=0, vertical_axis=1)
    DW = W
    water_hs = (0.5 * L, 0.5 * W, 0.5 * H)
    inner_hs = (0.5 * DL, 0.5 * DW, 0.5 * DH)
    outer_hs = (0.5 * DL + BW, 0.5 * DW + BW, 0.5 * DH + BW)
    return DamBreakCase(
        name=name, dim=3, sys_lower=(-BW, -BW, -BW), sys_upper=(DL + BW, DW + BW, DH + BW), dp=dp,
        water_center=water_hs, water_halfsize=water_hs, outer_center=inner_hs, outer_halfsize=outer_hs,
        inner_center=inner_hs, inner_halfsize=inner_hs, rho0=1.0, c0=c0, U_ref=U_ref, gravity=(0.0, 0.0, -g),
        observers=[(DL, 0.5 * DW, 0.2 * H)], loop_style=0, vertical_axis=2)


@dataclass
class TaylorGreenCase:
    """A periodic Taylor-Green vortex: lattice particles in [0, L]^dim at rest density.

    velocity_kind 0 is tests/2d_examples/test_2d_taylor_green/taylor_green.cpp:13-45
    (L = 1, u = -cos 2pi x sin 2pi y, v = sin 2pi x cos 2pi y, U = 1, c0 = 10, Re = 100);
    kind 1 the 3D vortex u = sin x cos y cos z, v = -cos x sin y cos z, w = 0 on
    [0, 2 pi]^3 (rho0 = 1, c0 = 10, Re = 100)."""
    name: str
    dim: int
    L: float
    dp: float
    velocity_kind: int = 0
    h_ratio: float = 1.3
    rho0: float = 1.0
    U: float = 1.0
    c0: float = 10.0
    Re: float = 100.0

    @property
    def h(self) -> float:
        return self.h_ratio * self.dp

    @property
    def mu(self) -> float:
        return self.rho0 * self.U * self.L / self.Re


def taylor_green_2d(resolution: int = 100) -> TaylorGreenCase:
    return TaylorGreenCase(f"taylor_green2d_{resolution}", 2, 1.0, 1.0 / resolution, 0)


def taylor_green_3d(resolution: int = 256) -> TaylorGreenCase:
    return TaylorGreenCase(f"taylor_green3d_{resolution}", 3, 2.0 * math.pi, 2.0 * math.pi / resolution, 1)
