"""The oracle's C restatement against the reference's own compiled code, run
live on seeded problems beyond the golden vectors: odd grids, void pockets,
prescribed non-zero displacements, point loads at random end-face nodes, graded
moduli, three filter radii, and short plain, masked, MMA and Heaviside-projected
optimisation runs.  Every comparison is bit for bit.

CPU only.  Skipped where the reference build (oracle/_ref, compiled from the
reference tree by oracle/build_ref.sh) is absent; the golden vectors carry the
pin there."""
import os

import numpy as np
import pytest

from oracle.oracle import REF_SO, OracleLib, Problem

pytestmark = pytest.mark.skipif(not os.path.exists(REF_SO), reason="reference build absent")

SEEDS = range(6)


@pytest.fixture(scope="module")
def ref():
    return OracleLib("reference")


def random_problem(seed, tags=False):
    """A seeded cantilever-like problem: x = 0 face clamped (a few of its DOFs
    prescribed non-zero), 1-4 point loads on the x = nx face, ~10 % void voxels
    away from both end layers.  With tags=True the voxels carry raw tags (Empty,
    Interior, a Fixture slab at x = 0, a Load slab at x = nx - 1)."""
    rng = np.random.default_rng(1000 + seed)
    nx, ny, nz = int(rng.integers(5, 18)), int(rng.integers(3, 10)), int(rng.integers(3, 9))
    solid = np.ones((nz, ny, nx), np.uint8)
    inner = rng.random((nz, ny, nx)) < 0.10
    inner[:, :, 0] = inner[:, :, nx - 1] = False
    solid[inner] = 0
    if tags:
        solid[:, :, 0] = 5
        solid[:, :, nx - 1] = np.where(rng.random((nz, ny)) < 0.5, 4, 1)
    pb = Problem(nx, ny, nz, 1.0, solid.ravel())
    bcs = []
    for c in range(nz + 1):
        for b in range(ny + 1):
            for comp in range(3):
                v = float(rng.uniform(-0.01, 0.01)) if rng.random() < 0.05 else 0.0
                bcs.append((pb.node(0, b, c), comp, v))
    loads = []
    for _ in range(int(rng.integers(1, 5))):
        b, c = int(rng.integers(0, ny + 1)), int(rng.integers(0, nz + 1))
        loads.append((pb.node(nx, b, c), int(rng.integers(0, 3)), float(rng.uniform(-1, 1))))
    return Problem(nx, ny, nz, 1.0, solid.ravel(), bcs, loads), rng


@pytest.mark.parametrize("seed", SEEDS)
def test_operator_reduced_system_and_solve(port, ref, seed):
    pb, rng = random_problem(seed)
    fac = rng.random(pb.nv) * 0.99 + 0.01
    u = rng.standard_normal(pb.ndof)
    assert np.array_equal(port.apply(pb, u, fac), ref.apply(pb, u, fac))
    a, b = port.build_reduced(pb, fac), ref.build_reduced(pb, fac)
    for k in ("kept", "rhs", "invdiag", "up"):
        assert np.array_equal(a[k], b[k]), k
    assert a["ng"] == b["ng"]
    ua, ia, ra = port.solve_cg(pb, fac, tol=1e-10)
    ub, ib, rb = ref.solve_cg(pb, fac, tol=1e-10)
    assert ia == ib and ra == rb and np.array_equal(ua, ub)


@pytest.mark.parametrize("seed", SEEDS)
def test_compliance_filter_and_oc(port, ref, seed):
    pb, rng = random_problem(seed)
    rho = rng.uniform(0.05, 1.0, pb.nv)
    a = port.simp_compliance(pb, rho, tol=1e-10)
    b = ref.simp_compliance(pb, rho, tol=1e-10)
    assert a["compliance"] == b["compliance"] and a["iterations"] == b["iterations"]
    assert np.array_equal(a["u"], b["u"]) and np.array_equal(a["dc"], b["dc"])
    x = rng.random(pb.nv)
    for r in (1.2, 1.7, 2.5):
        for adj in (False, True):
            assert np.array_equal(port.filter(pb, x, r, adj), ref.filter(pb, x, r, adj)), (r, adj)
    vf = float(rng.uniform(0.2, 0.5))
    assert np.array_equal(port.oc_update(pb, rho, a["dc"], vf, 1.7, 0.2),
                          ref.oc_update(pb, rho, a["dc"], vf, 1.7, 0.2))


@pytest.mark.parametrize("seed", SEEDS[:3])
def test_short_runs(port, ref, seed):
    """Five design iterations, plain and masked (FrozenSolid and FrozenVoid
    islands on a tagged grid): the whole trajectory is identical."""
    pb, rng = random_problem(seed)
    a = port.simp_optimize(pb, volfrac=0.35, radius=1.5, move=0.2, max_it=5, change_tol=0.0,
                           cg_tol=1e-10)
    b = ref.simp_optimize(pb, volfrac=0.35, radius=1.5, move=0.2, max_it=5, change_tol=0.0,
                          cg_tol=1e-10)
    assert np.array_equal(a["hist_c"], b["hist_c"]) and np.array_equal(a["design"], b["design"])
    pt, rng = random_problem(seed, tags=True)
    mask = np.zeros(pt.nv, np.uint8)
    rr = rng.random(pt.nv)
    mask[rr < 0.08] = 1
    mask[(rr >= 0.08) & (rr < 0.14)] = 2
    assert np.array_equal(port.effective_design_mask(pt, mask), ref.effective_design_mask(pt, mask))
    x = rng.random(pt.nv)
    for adj in (False, True):
        assert np.array_equal(port.filter_masked(pt, mask, x, 1.5, adj),
                              ref.filter_masked(pt, mask, x, 1.5, adj))
    a = port.simp_optimize_masked(pt, mask, volfrac=0.35, radius=1.5, move=0.2, max_it=5,
                                  change_tol=0.0, cg_tol=1e-10)
    b = ref.simp_optimize_masked(pt, mask, volfrac=0.35, radius=1.5, move=0.2, max_it=5,
                                 change_tol=0.0, cg_tol=1e-10)
    for k in ("hist_c", "hist_change", "hist_vf", "design", "phys"):
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("seed", SEEDS[3:])
def test_short_mma_and_projected_runs(port, ref, seed):
    """Eight MMA design iterations and a two-stage Heaviside-projected run
    (beta 1 then 2): identical trajectories."""
    pb, rng = random_problem(seed)
    a = port.simp_optimize_mma(pb, volfrac=0.35, radius=1.5, move=0.2, max_it=8, change_tol=0.0,
                               cg_tol=1e-10)
    b = ref.simp_optimize_mma(pb, volfrac=0.35, radius=1.5, move=0.2, max_it=8, change_tol=0.0,
                              cg_tol=1e-10)
    assert a["iterations"] == b["iterations"]
    for k in ("hist_c", "hist_change", "hist_vf", "design", "phys"):
        assert np.array_equal(a[k], b[k]), k
    stages = [(1.0, 0.2, 3), (2.0, 0.2, 3)]
    a = port.simp_optimize(pb, volfrac=0.35, radius=2.0, change_tol=0.0, cg_tol=1e-10,
                           stages=stages)
    b = ref.simp_optimize(pb, volfrac=0.35, radius=2.0, change_tol=0.0, cg_tol=1e-10,
                          stages=stages)
    assert a["iterations"] == b["iterations"] == 6
    for k in ("hist_c", "hist_vf", "design", "phys"):
        assert np.array_equal(a[k], b[k]), k
