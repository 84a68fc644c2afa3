"""Seeded synthetic workloads of many hydro runs: the mixed batch (Sod,
Sedov and advection instances of uneven sizes) and the Poisson request
stream of the serving loop.

Randomness comes from std::mt19937_64 (restated here in pure Python and
checked against the C++ standard's known answer: the 10000th output of a
default-seeded engine is 9981545732273789042).  A uniform draw on [a, b) is
a + (b - a) * (x >> 11) * 2**-53 for the next engine output x; a log-uniform
size is round(exp(U[ln lo, ln hi])).

Instance kinds (all VNR, order-2 remap, no PenteBorne):
  Sod       SodCaseX/Y (one material) or BiSodCaseX/Y (two or more), the
            reference initialisation, on [0,1]^2
  Sedov     SedovTestCase for VNR (an extension: rho 1, p 1e-6, energy
            0.244816 in the cell at the origin, Eucclhyd Sedov boundary
            conditions) on [0,1.2]^2, the |e| > 5 abort disabled
  Advection BiAdvectionX with init_variant 2 (an extension: density step
            1 -> 0.1 at x = 0.5 over two materials, velocity (1, 0)), no
            Lagrange phase, dt = 0.25 dx
"""
from __future__ import annotations

import math
from dataclasses import dataclass

MASK64 = (1 << 64) - 1


class MT19937_64:
    """std::mt19937_64."""

    def __init__(self, seed: int = 5489):
        self.mt = [0] * 312
        self.mt[0] = seed & MASK64
        for i in range(1, 312):
            self.mt[i] = (6364136223846793005 * (self.mt[i - 1] ^ (self.mt[i - 1] >> 62)) + i) & MASK64
        self.idx = 312

    def _twist(self) -> None:
        mt = self.mt
        for i in range(312):
            x = (mt[i] & 0xFFFFFFFF80000000) | (mt[(i + 1) % 312] & 0x7FFFFFFF)
            xa = x >> 1
            if x & 1:
                xa ^= 0xB5026F5AA96619E9
            mt[i] = mt[(i + 156) % 312] ^ xa
        self.idx = 0

    def __call__(self) -> int:
        if self.idx >= 312:
            self._twist()
        y = self.mt[self.idx]
        self.idx += 1
        y ^= (y >> 29) & 0x5555555555555555
        y ^= (y << 17) & 0x71D67FFFEDA60000
        y ^= (y << 37) & 0xFFF7EEE000000000
        y ^= y >> 43
        return y & MASK64

    def uniform(self, a: float = 0.0, b: float = 1.0) -> float:
        return a + (b - a) * ((self() >> 11) * (1.0 / 9007199254740992.0))

    def log_uniform_int(self, lo: int, hi: int) -> int:
        return int(round(math.exp(self.uniform(math.log(lo), math.log(hi)))))


SOD, SEDOV, ADVECTION = "sod", "sedov", "advection"


@dataclass
class Instance:
    kind: str
    nx: int
    ny: int
    nbmat: int
    limiter: str
    cycles: int
    sod_axis: str = "X"

    @property
    def cells(self) -> int:
        return self.nx * self.ny

    def spec(self, M):
        """HydroSpec of this instance (M is the mahyco_gb300 module)."""
        s = M.default_spec()
        s.scheme = M.SCHEME_VNR
        s.nx, s.ny = self.nx, self.ny
        L = 1.2 if self.kind == SEDOV else 1.0
        s.dx, s.dy = L / self.nx, L / self.ny
        s.nbmat = self.nbmat
        for m in range(3):
            s.eos[m] = 101
            s.gamma[m] = 1.4
        s.gamma_scalar = 1.4
        s.projection = 1
        s.projection_order = 2
        s.space_order = 2
        s.threshold = 1e-16
        s.limiter = M.LIMITERS[self.limiter]
        s.limiter_pure = M.LIMITERS[self.limiter]
        s.pb = 0
        s.pb_mixte = 0
        s.pb_complet = 0
        s.pseudo_centree = 0
        s.dual_mass_flux = 0
        s.max_cycles = self.cycles
        s.final_time = 1.0
        s.output_time = 1.0
        s.dt_min = 1e-12
        s.dt_init = 1e-4
        s.init_variant = 0
        s.sans_lagrange = 0
        s.energy_limit = 5.0
        if self.kind == SOD:
            if self.nbmat == 1:
                s.test_case = 4 if self.sod_axis == "X" else 5
            else:
                s.test_case = 15 if self.sod_axis == "X" else 16
        elif self.kind == SEDOV:
            s.test_case = 1
            s.energy_limit = 0.0
        else:
            s.test_case = 18
            s.init_variant = 2
            s.sans_lagrange = 1
            s.dt_init = 0.25 * s.dx
        return s


def batch_mix(n: int = 512, seed: int = 20261203, cycles: int = 100,
              nx_range=(64, 1024), ny_range=(64, 256)) -> list[Instance]:
    """The mixed batch: per instance, draws nx then ny (log-uniform); kind
    cycles Sod, Sedov, advection; a Sod instance then draws its axis (X if
    < 0.5) and material count (1 if < 0.5, else 2); every instance then
    draws its limiter (minmod if < 0.5, else superBee)."""
    g = MT19937_64(seed)
    out = []
    for i in range(n):
        nx = g.log_uniform_int(*nx_range)
        ny = g.log_uniform_int(*ny_range)
        kind = (SOD, SEDOV, ADVECTION)[i % 3]
        axis, nbmat = "X", 1
        if kind == SOD:
            axis = "X" if g.uniform() < 0.5 else "Y"
            nbmat = 1 if g.uniform() < 0.5 else 2
        elif kind == ADVECTION:
            nbmat = 2
        lim = "minmod" if g.uniform() < 0.5 else "superBee"
        out.append(Instance(kind, nx, ny, nbmat, lim, cycles, axis))
    return out


@dataclass
class Request:
    arrival: float  # seconds after the stream starts
    inst: Instance


def request_stream(rate: float, n: int, seed: int | None = None,
                   size_range=(32, 2048), cycle_range=(50, 500)) -> list[Request]:
    """Poisson arrivals at `rate` req/s (seed 7 + rate by default).  Per
    request, in order: the exponential gap, nx, ny (log-uniform), the
    material count (1, 2 or 3), the cycle count (uniform integer), then the
    kind-specific draws of batch_mix (Sod axis) and the limiter; kinds cycle
    Sod, Sedov, advection.  Advection runs carry at least two materials."""
    g = MT19937_64(int(7 + rate) if seed is None else seed)
    out, t = [], 0.0
    lo, hi = cycle_range
    for i in range(n):
        t += -math.log(1.0 - g.uniform()) / rate
        nx = g.log_uniform_int(*size_range)
        ny = g.log_uniform_int(*size_range)
        nbmat = 1 + min(2, int(g.uniform() * 3))
        cycles = lo + min(hi - lo, int(g.uniform() * (hi - lo + 1)))
        kind = (SOD, SEDOV, ADVECTION)[i % 3]
        axis = "X"
        if kind == SOD:
            axis = "X" if g.uniform() < 0.5 else "Y"
        if kind == ADVECTION:
            nbmat = max(nbmat, 2)
        lim = "minmod" if g.uniform() < 0.5 else "superBee"
        out.append(Request(t, Instance(kind, nx, ny, nbmat, lim, cycles, axis)))
    return out


def state_bytes(inst: Instance) -> int:
    """Persistent state of one VNR run (cell, per-material and node fields
    read and written each cycle): (80 + 56 m) bytes per cell."""
    return (80 + 56 * inst.nbmat) * inst.cells
