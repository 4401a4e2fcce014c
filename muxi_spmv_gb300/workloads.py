"""Named synthetic workloads (seeded stand-ins for the benchmark matrices).

poisson16k        16,384^2, row lengths Poisson(12) clamped to [1,64], columns
                  uniform without replacement per row (sorted), values and x
                  U[-1,1], seed 0.
powerlaw8m        8,388,608^2, row lengths Zipf(1.8) on [1,65,536], 70% of
                  columns within +-4,096 of the diagonal (reflected at the
                  edges) and 30% uniform, sorted; values N(0,1); x U[-1,1].
                  The support [1,65,536] makes the mean row length 22.06
                  (about 185M nonzeros).
powerlaw8m_c1024  the same law on [1,1,024] (mean 8.3, about 69.5M nonzeros).
stencil2d_4096    5-point Laplacian on a 4096x4096 grid: 16,777,216 rows,
                  83,869,696 nonzeros, values 4 / -1.
stencil3d_256     27-point stencil on 256^3: 16,777,216 rows, 449,455,096
                  nonzeros, values N(0,1).
`scaled(name, rows)` gives the same law on fewer rows for tests.
"""
from __future__ import annotations

from .api import (GEN_POISSON_UNIFORM, GEN_POWERLAW, GEN_STENCIL2D, GEN_STENCIL3D, GEN_BANDED, GEN_BLOCKDIAG,
                  GEN_ZIPF_UNIFORM, GEN_DIAGONAL, GenSpec)

X_SEED_OFFSET = 0x5eed


def spec(name: str, seed: int = 0) -> GenSpec:
    if name == "poisson16k":
        return GenSpec(GEN_POISSON_UNIFORM, 16384, 16384, 12.0, 1, 64, 0, seed)
    if name == "powerlaw8m":
        return GenSpec(GEN_POWERLAW, 8388608, 8388608, 1.8, 65536, 4096, 0.7, seed)
    if name == "powerlaw8m_c1024":
        return GenSpec(GEN_POWERLAW, 8388608, 8388608, 1.8, 1024, 4096, 0.7, seed)
    if name == "stencil2d_4096":
        return GenSpec(GEN_STENCIL2D, 4096 * 4096, 4096 * 4096, 4096, 4096, 0, 0, seed)
    if name == "stencil3d_256":
        n = 256
        return GenSpec(GEN_STENCIL3D, n ** 3, n ** 3, n, n, n, 0, seed)
    raise KeyError(name)


def scaled(name: str, rows: int, seed: int = 0) -> GenSpec:
    """Same law as `name` on about `rows` rows (square)."""
    s = spec(name, seed)
    if s.kind == GEN_STENCIL2D:
        n = max(2, int(round(rows ** 0.5)))
        return GenSpec(GEN_STENCIL2D, n * n, n * n, n, n, 0, 0, seed)
    if s.kind == GEN_STENCIL3D:
        n = max(2, int(round(rows ** (1 / 3))))
        return GenSpec(GEN_STENCIL3D, n ** 3, n ** 3, n, n, n, 0, seed)
    if s.kind == GEN_POWERLAW:
        band = min(s.p2, max(1, rows // 8))
        return GenSpec(s.kind, rows, rows, s.p0, min(s.p1, rows), band, s.p3, seed)
    return GenSpec(s.kind, rows, rows, s.p0, s.p1, min(s.p2, rows), s.p3, seed)


def x_seed(seed: int) -> int:
    return seed + X_SEED_OFFSET


ALL = ["poisson16k", "powerlaw8m", "powerlaw8m_c1024", "stencil2d_4096", "stencil3d_256"]
__all__ = ["spec", "scaled", "x_seed", "ALL", "GenSpec", "GEN_POISSON_UNIFORM", "GEN_POWERLAW", "GEN_STENCIL2D",
           "GEN_STENCIL3D", "GEN_BANDED", "GEN_BLOCKDIAG", "GEN_ZIPF_UNIFORM", "GEN_DIAGONAL"]
