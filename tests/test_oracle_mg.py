"""The CPU restatement of the reference's geometric-multigrid PCG
(oracle/oracle_mg.c), the timed CPU baseline of the benchmark.  CPU only.

It is a restatement (Galerkin coarse operators kept as node stencils, a banded
Cholesky at the coarsest level), so it is pinned at the solution level: the
same displacement as the exact Jacobi-PCG restatement (itself bit-identical to
the reference's compiled code), and its design-iteration driver follows the
oracle's own simp_optimize trajectory."""
import numpy as np
import pytest

from oracle.oracle import cantilever


def smooth_modulus(nx, ny, nz, seed=2):
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    rng = np.random.default_rng(seed)
    rho = np.full(i.shape, 0.3)
    for _ in range(4):
        fx, fy, fz, ph = rng.uniform(0.5, 3.0, 3).tolist() + [rng.uniform(0, 6.3)]
        rho += 0.15 * np.sin(fx * np.pi * i / nx + fy * np.pi * j / ny + fz * np.pi * k / nz + ph)
    return np.clip(rho, 1e-3, 1.0).ravel() ** 3


@pytest.mark.parametrize("dims,voids", [((16, 8, 8), False), ((24, 12, 10), False),
                                        ((33, 17, 9), False), ((40, 16, 16), True)])
def test_mg_solution_matches_exact_cg(port, dims, voids):
    nx, ny, nz = dims
    solid = None
    if voids:  # a void pocket away from the supports and the load
        s = np.ones((nz, ny, nx), np.uint8)
        s[4:10, 4:10, 10:20] = 0
        solid = s.ravel()
    o = cantilever(nx, ny, nz, solid=solid)
    f = smooth_modulus(nx, ny, nz)
    ue, _, _ = port.solve_cg(o, f, tol=1e-12)
    um, it, res, lev = port.mg_solve(o, f, tol=1e-10)
    assert res <= 1e-10 and lev >= 2
    assert np.abs(um - ue).max() <= 1e-8 * np.abs(ue).max()


def test_mg_depth_rule(port):
    """Coarsening stops at the first level with <= 6000 active DOFs (the
    reference's coarse_dof_cap): 60x20x20 gives 3 levels, 64x32x32 gives 3."""
    for dims, want in [((60, 20, 20), 3), ((64, 32, 32), 3)]:
        o = cantilever(*dims)
        f = smooth_modulus(*dims)
        _, it, _, lev = port.mg_solve(o, f, tol=1e-8)
        assert lev == want, (dims, lev)
        assert it < 60


def test_design_iterations_follow_the_oracle_trajectory(port):
    """Three OC design iterations of the 60x20x20 configuration with the MG-PCG
    restatement: compliances and the design track the oracle's simp_optimize
    (exact Jacobi-PCG) run to the solve tolerance."""
    o = cantilever(60, 20, 20)
    ref = port.simp_optimize(o, volfrac=0.3, radius=1.5, move=0.2, max_it=3, change_tol=0.0,
                             cg_tol=1e-10)
    x0 = np.full(o.nv, 0.3)
    r = port.design_iterations_mg(o, x0, 3, cg_tol=1e-10)
    assert np.abs(r["compliance"] - ref["hist_c"]).max() <= 1e-8 * ref["hist_c"][0]
    assert np.abs(r["x"] - ref["design"]).max() <= 1e-6
    assert (r["cg"] > 0).all() and r["seconds"].shape == (3, 5)


def test_mg_independent_of_thread_count(port):
    """The restatement gives the same bits on 1 and 3 threads: its element apply
    runs colour by colour, every other parallel loop writes one output each,
    and its dot products sum fixed blocks in a fixed order."""
    o = cantilever(24, 12, 10)
    f = smooth_modulus(24, 12, 10)
    old = port.threads()
    try:
        out = []
        for t in (1, 3):
            port.set_threads(t)
            u, it, res, lev = port.mg_solve(o, f, tol=1e-10)
            r = port.design_iterations_mg(o, np.full(o.nv, 0.3), 2, cg_tol=1e-8)
            out.append((u, it, res, r["x"], r["compliance"], r["cg"]))
    finally:
        port.set_threads(old)
    (u1, i1, r1, x1, c1, g1), (u3, i3, r3, x3, c3, g3) = out
    assert i1 == i3 and r1 == r3 and np.array_equal(u1, u3)
    assert np.array_equal(x1, x3) and np.array_equal(c1, c3) and np.array_equal(g1, g3)
