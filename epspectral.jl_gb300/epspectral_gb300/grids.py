"""FrequencyGrid and its constructors, the host side of the grid type the API passes across the
ABI as (origin, unit, offsets).

Mirrors src/frequency_grids.jl: `FrequencyGrid(ω_origin, dω_unit, offsets)` (:119-141),
`FrequencyGrid(ωs::AbstractVector; atol)` (:143-171) and `graded_frequency_grid(windows)`
(:261-294), with the same arguments, results and ArgumentError conditions.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


class ArgumentError(ValueError):
    """The reference's ArgumentError: an argument out of range."""


@dataclass(frozen=True)
class FrequencyGrid:
    """Nodes origin + offsets[j] * unit with strictly increasing integer offsets (at least two)."""

    origin: float
    unit: float
    offsets: tuple

    def __init__(self, origin, unit, offsets):
        origin, unit = float(origin), float(unit)
        if not (math.isfinite(origin) and math.isfinite(unit) and unit > 0):
            raise ArgumentError(
                f"ω_origin must be finite and dω_unit finite and positive, got {origin}, {unit}")
        off = np.asarray(offsets, dtype=np.int64).ravel()
        if len(off) < 2:
            raise ArgumentError("a FrequencyGrid needs at least two nodes")
        gaps = np.diff(off)
        if not np.all(gaps > 0):
            k = int(np.argmax(gaps <= 0))
            raise ArgumentError(f"offsets must be strictly increasing, got offsets[{k + 1}] >= offsets[{k + 2}]")
        object.__setattr__(self, "origin", origin)
        object.__setattr__(self, "unit", unit)
        object.__setattr__(self, "offsets", tuple(int(o) for o in off))

    @property
    def dw_min(self) -> float:
        """Smallest distance between neighbouring nodes (:131)."""
        return self.unit * float(np.min(np.diff(np.asarray(self.offsets))))

    def nodes(self) -> np.ndarray:
        """ωs[j] = origin + offsets[j] * unit, evaluated as the reference's getindex (:140-141)."""
        return self.origin + np.asarray(self.offsets, dtype=np.float64) * self.unit

    def __len__(self):
        return len(self.offsets)

    @staticmethod
    def from_nodes(ws, atol: float = 1e-8) -> "FrequencyGrid":
        """`FrequencyGrid(ωs::AbstractVector; atol)`: the largest commensurate step
        min(diff(ωs)) / k, k <= 64, with every node within atol steps of the grid (:143-171)."""
        ws = np.asarray(ws, dtype=np.float64)
        if len(ws) < 2:
            raise ArgumentError("ωs must have at least two points")
        gaps = np.diff(ws)
        jmin = int(np.argmin(gaps)) if np.all(np.isfinite(gaps)) else int(np.nanargmin(np.where(np.isnan(gaps), -np.inf, gaps)))
        dw_min = gaps[jmin]
        span = ws[-1] - ws[0]
        if not (dw_min > 1e-8 * span):
            raise ArgumentError(
                f"ωs must be finite and strictly increasing with spacings above 1e-8 of its span; "
                f"ωs[{jmin + 1}] = {ws[jmin]} and ωs[{jmin + 2}] = {ws[jmin + 1]} are {dw_min} apart")
        best = (math.inf, 0, dw_min)
        for k in range(1, 65):
            unit = span / round(span / (dw_min / k))
            p = (ws - ws[0]) / unit
            dev = np.abs(p - np.round(p))
            j = int(np.argmax(dev))
            if dev[j] <= atol:
                return FrequencyGrid(ws[0], unit, np.round(p).astype(np.int64))
            if dev[j] < best[0]:
                best = (dev[j], j, unit)
        raise ArgumentError(
            f"ωs is not commensurate: no step minimum(diff(ωs)) / k with k <= 64 puts every node "
            f"within {atol} steps of ωs[1] + dω_unit ℤ; at the closest, dω_unit = {best[2]}, the node "
            f"ωs[{best[1] + 1}] = {ws[best[1]]} is {best[0]} steps off. Build the grid with "
            f"`graded_frequency_grid`, or move the node onto the grid.")

    @staticmethod
    def uniform(start: float, stop: float, step: float) -> "FrequencyGrid":
        """`FrequencyGrid(first, step, 0:n-1)` with n = length(range(start, stop; step)), the default
        spectral grid of run_scgd0 (src/scgd0.jl:89-92)."""
        n = int(math.floor((stop - start) / step * (1 + 1e-12) + 1e-9)) + 1
        return FrequencyGrid(start, step, np.arange(n))


def graded_frequency_grid(windows) -> FrequencyGrid:
    """Nested windows [(wmin, wmax, dw), ...], finest first (src/frequency_grids.jl:261-294)."""
    if len(windows) == 0:
        raise ArgumentError("windows must not be empty")
    wmins = np.array([float(w[0]) for w in windows])
    wmaxs = np.array([float(w[1]) for w in windows])
    dws = np.array([float(w[2]) for w in windows])
    if not (np.all(dws > 0) and np.all(wmins < wmaxs)):
        raise ArgumentError(f"every window needs dw > 0 and wmin < wmax, got {windows}")
    if not (np.all(np.diff(wmins) <= 0) and np.all(np.diff(wmaxs) >= 0)):
        raise ArgumentError(
            "windows must be nested from the smallest to the largest (wmin non-increasing, wmax "
            f"non-decreasing), got {windows}")
    origin, dw1 = (wmins[0] + wmaxs[0]) / 2, dws[0]
    tol = 1e-8
    u = (wmins - origin) / dw1
    v = (wmaxs - origin) / dw1
    ps: list[int] = []
    for l in range(len(windows)):
        ratio = dws[l] / dw1
        if abs(ratio - round(ratio)) > tol:
            raise ArgumentError(f"dw[{l + 1}] = {dws[l]} is not an integer multiple of dw[1] = {dw1} (ratio {ratio})")
        r = int(round(ratio))
        if l == 0:
            ps.extend(range(math.ceil(u[0] - tol), math.floor(v[0] + tol) + 1))
            if len(ps) < 2:
                raise ArgumentError(
                    f"the finest window must hold at least two nodes, got {len(ps)} for {windows[0]}")
        else:
            p_lo, p_hi = min(ps), max(ps)
            ps.extend(range(p_hi + r, math.floor(v[l] + tol) + 1, r))
            ps.extend(range(p_lo - r, math.ceil(u[l] - tol) - 1, -r))
    return FrequencyGrid(origin, dw1, sorted(ps))
