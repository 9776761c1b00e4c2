"""Seeded synthetic voxel problems for the batched and serving workloads.

* ``design(seed)`` -- one design of the batched workload: a solid grid with nx
  in [32, 128], ny, nz in [16, 64] (even), volume fraction U[0.15, 0.5], filter
  radius U[1.2, 2.5], penalty 3, one clamped face chosen at random and 1-3 unit
  loads (a point load, or an edge load spread over the nodes of an edge) on
  random nodes of the opposite face.  The reference's simp_optimize takes one
  load set, so the 1-3 loads act together as one load case.
* ``stream(seed, rate, duration)`` -- an open-loop Poisson arrival stream of such
  jobs whose grids are log-uniform in element count between 24^3 and
  192 x 96 x 96 (aspect 2:1:1).
"""
from __future__ import annotations

import numpy as np

from ._capi import Problem, SimpOptions, SimpParams, SolveOptions


def _even(v):
    return max(2, int(round(v / 2.0)) * 2)


def _problem(rng, nx, ny, nz):
    pb = Problem(nx, ny, nz)
    dims = (nx, ny, nz)
    axis = int(rng.integers(3))
    side = int(rng.integers(2))
    fixed = 0 if side == 0 else dims[axis]
    far = dims[axis] - fixed

    def face_nodes(pos):
        out = []
        rngs = [range(d + 1) for d in dims]
        rngs[axis] = [pos]
        for c in rngs[2]:
            for b in rngs[1]:
                for a in rngs[0]:
                    out.append(pb.node(a, b, c))
        return out

    bcs = [(n, k, 0.0) for n in face_nodes(fixed) for k in range(3)]
    loads = []
    for _ in range(int(rng.integers(1, 4))):
        comp = int(rng.integers(3))
        sign = -1.0 if rng.random() < 0.5 else 1.0
        coord = [int(rng.integers(d + 1)) for d in dims]
        coord[axis] = far
        if rng.random() < 0.5:  # point load
            loads.append((pb.node(*coord), comp, sign))
        else:  # edge load: total 1 over a line of the far face
            free = [a for a in range(3) if a != axis]
            along = free[int(rng.integers(2))]
            nodes = []
            for t in range(dims[along] + 1):
                cc = list(coord)
                cc[along] = t
                nodes.append(pb.node(*cc))
            loads += [(n, comp, sign / len(nodes)) for n in nodes]
    return Problem(nx, ny, nz, 1.0, None, bcs, loads)


def design(seed: int, precision: int = 1, iterations: int = 40, sizes=None):
    """(Problem, SimpParams, SimpOptions) of one seeded design."""
    rng = np.random.default_rng(seed)
    if sizes is None:
        nx = _even(rng.integers(32, 129))
        ny = _even(rng.integers(16, 65))
        nz = _even(rng.integers(16, 65))
    else:
        nx, ny, nz = sizes
    pb = _problem(rng, nx, ny, nz)
    opt = SimpOptions(volume_fraction=float(rng.uniform(0.15, 0.5)),
                      filter_radius=float(rng.uniform(1.2, 2.5)), move=0.2, change_tol=0.0,
                      cg_tolerance=1e-8, max_iterations=iterations,
                      solve=SolveOptions(precision=precision))
    return pb, SimpParams(), opt


def stream_sizes(rng, lo=24 ** 3, hi=192 * 96 * 96):
    n_el = float(np.exp(rng.uniform(np.log(lo), np.log(hi))))
    nx = _even((4.0 * n_el) ** (1.0 / 3.0))
    return nx, max(2, _even(nx / 2)), max(2, _even(nx / 2))


def stream(seed: int, rate: float, duration: float, precision: int = 1, iterations: int = 40):
    """[(arrival_s, Problem, SimpParams, SimpOptions)] of a Poisson stream."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += float(rng.exponential(1.0 / rate))
        if t >= duration:
            return out
        sizes = stream_sizes(rng)
        pb, prm, opt = design(int(rng.integers(1 << 31)), precision, iterations, sizes)
        out.append((t, pb, prm, opt))


def cantilever_seeded_load(nx, ny, nz, seed=0):
    """The benchmark cantilever's boundary conditions: the x = 0 face clamped,
    a unit -z load at a seeded uniform point (numpy default_rng(seed)) of the
    x = nx end face, spread bilinearly to the four surrounding nodes.  Returns
    (bcs, loads) as (node, component, value) triples."""
    rng = np.random.default_rng(seed)
    yy, zz = rng.uniform(0.0, ny), rng.uniform(0.0, nz)
    b0, c0 = min(int(yy), ny - 1), min(int(zz), nz - 1)
    ty, tz = yy - b0, zz - c0

    def node(a, b, c):
        return (c * (ny + 1) + b) * (nx + 1) + a

    bcs = [(node(0, b, c), k, 0.0) for c in range(nz + 1) for b in range(ny + 1) for k in range(3)]
    loads = []
    for db, wb in ((0, 1.0 - ty), (1, ty)):
        for dc, wc in ((0, 1.0 - tz), (1, tz)):
            if wb * wc > 0.0:
                loads.append((node(nx, b0 + db, c0 + dc), 2, -1.0 * wb * wc))
    return bcs, loads
