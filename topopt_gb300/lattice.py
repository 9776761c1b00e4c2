"""Unit-cell generators for the periodic homogenization workload.

Restates the lattice generators of the reference's homogenization harness
(core/tests/harness/lattice_homog_probe.cpp:78-229): a voxel is solid when its
centre lies inside the structure -- the gyroid sheet |sin x cos y + sin y cos z +
sin z cos x| < level, the Schwarz-D sheet, or the octet truss (struts from each
face centre to the four corners of that face, radius r).  ``calibrate`` bisects
the level (or strut radius) 28 times so the cell's solid fraction approaches a
target relative density, as calibrate_level / calibrate_octet_r do.
"""
from __future__ import annotations

import numpy as np

KINDS = ("gyroid", "schwarzD", "octet")


def _centres(vpc: int):
    c = (np.arange(vpc) + 0.5) / vpc  # cell of period L = 1
    z, y, x = np.meshgrid(c, c, c, indexing="ij")
    return x, y, z


def _octet_struts():
    corners = [(x, y, z) for z in (0, 1) for y in (0, 1) for x in (0, 1)]
    faces = [(0.5, 0.5, 0.0), (0.5, 0.5, 1.0), (0.5, 0.0, 0.5), (0.5, 1.0, 0.5),
             (0.0, 0.5, 0.5), (1.0, 0.5, 0.5)]
    segs = []
    for f in faces:
        for c in corners:
            d2 = sum((c[k] - f[k]) ** 2 for k in range(3) if f[k] in (0.0, 1.0))
            if d2 < 1e-9:
                segs.append((np.array(f), np.array(c, dtype=float)))
    return segs


def _field(kind: str, vpc: int):
    """The scalar whose sub-level set is the solid: |g| for the sheets, the
    squared distance to the nearest strut for the octet."""
    x, y, z = _centres(vpc)
    a = 2.0 * np.pi
    if kind == "gyroid":
        g = np.sin(a * x) * np.cos(a * y) + np.sin(a * y) * np.cos(a * z) + \
            np.sin(a * z) * np.cos(a * x)
        return np.abs(g)
    if kind == "schwarzD":
        g = (np.sin(a * x) * np.sin(a * y) * np.sin(a * z) +
             np.sin(a * x) * np.cos(a * y) * np.cos(a * z) +
             np.cos(a * x) * np.sin(a * y) * np.cos(a * z) +
             np.cos(a * x) * np.cos(a * y) * np.sin(a * z))
        return np.abs(g)
    if kind == "octet":
        p = np.stack([x, y, z], axis=-1)
        best = np.full(x.shape, 1e30)
        for s0, s1 in _octet_struts():
            ab = s1 - s0
            t = np.clip(((p - s0) @ ab) / (ab @ ab), 0.0, 1.0)
            c = s0 + t[..., None] * ab
            best = np.minimum(best, ((p - c) ** 2).sum(-1))
        return best
    raise ValueError(f"unknown lattice kind {kind!r}; one of {KINDS}")


def cell(kind: str, vpc: int, level: float) -> np.ndarray:
    """A (vpc, vpc, vpc) uint8 cell: 1 solid, 0 void.  ``level`` is the sheet
    half-thickness for gyroid/schwarzD and the strut radius for octet."""
    f = _field(kind, vpc)
    thr = level * level if kind == "octet" else level
    return (f < thr).astype(np.uint8)


def calibrate(kind: str, vpc: int, target: float) -> float:
    """Bisect the level to a target solid fraction (28 steps)."""
    lo, hi = (0.0005, 0.30) if kind == "octet" else (0.001, 1.6)
    f = _field(kind, vpc)
    for _ in range(28):
        mid = 0.5 * (lo + hi)
        thr = mid * mid if kind == "octet" else mid
        if (f < thr).mean() < target:
            lo = mid
        else:
            hi = mid
    return 0.5 * (lo + hi)


def batch(n: int, vpc: int = 32, seed: int = 0, kinds=("gyroid", "octet"),
          density=(0.1, 0.4)) -> tuple[np.ndarray, list]:
    """n cells of random kind and relative density ~ U[density]; returns the
    (n, vpc, vpc, vpc) tags and the (kind, target, achieved) of each cell."""
    rng = np.random.default_rng(seed)
    out = np.zeros((n, vpc, vpc, vpc), np.uint8)
    meta = []
    fields = {k: _field(k, vpc) for k in kinds}
    for i in range(n):
        kind = kinds[int(rng.integers(len(kinds)))]
        target = float(rng.uniform(*density))
        f = fields[kind]
        lo, hi = (0.0005, 0.30) if kind == "octet" else (0.001, 1.6)
        for _ in range(28):
            mid = 0.5 * (lo + hi)
            thr = mid * mid if kind == "octet" else mid
            if (f < thr).mean() < target:
                lo = mid
            else:
                hi = mid
        lev = 0.5 * (lo + hi)
        thr = lev * lev if kind == "octet" else lev
        out[i] = (f < thr).astype(np.uint8)
        meta.append((kind, target, float(out[i].mean())))
    return out, meta
