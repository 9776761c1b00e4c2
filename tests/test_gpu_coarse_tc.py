"""The level-1 Galerkin operator of the mixed V-cycle on the tensor cores
(tcgen05 MMA into TMEM, TF32 splits to FP32 accuracy) against the assembled
FP32 stencil of the same operator, and the mixed solve with it against the FP64
solve.  GPU only.

Cases: the clamped cantilever (Dirichlet DOFs put the first coarse layer off the
fast path), odd extents (the aligned half elements), voids and a Fixture/Load
mask, and the 256x128x128 benchmark grid."""
import numpy as np
import pytest

from oracle.oracle import cantilever

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _job(tg, pb, iters=2):
    opt = tg.SimpOptions(volume_fraction=0.3, filter_radius=1.5, move=0.2, change_tol=0.0,
                         cg_tolerance=1e-8, max_iterations=iters + 2,
                         solve=tg.SolveOptions(precision=tg.PREC_MIXED))
    job = tg.SimpJob(pb, tg.SimpParams(), opt)
    for _ in range(iters):
        job.step()
    return job


@pytest.mark.parametrize("dims,voids", [((48, 24, 24), False), ((47, 21, 19), False),
                                        ((40, 24, 16), True)])
def test_level1_tc_matches_stencil(tg, dims, voids):
    nx, ny, nz = dims
    solid = None
    if voids:
        rng = np.random.default_rng(3)
        solid = (rng.random(nx * ny * nz) > 0.08).astype(np.uint8)
        solid.reshape(nz, ny, nx)[:, :, :2] = 1
        solid.reshape(nz, ny, nx)[nz // 2 - 1:nz // 2 + 1, :, -1] = 1
    o = cantilever(nx, ny, nz, solid=solid)
    pb = tg.Problem(nx, ny, nz, 1.0, solid, list(zip(o.bc_node, o.bc_comp, o.bc_val)),
                    list(zip(o.ld_node, o.ld_comp, o.ld_val)))
    job = _job(tg, pb)
    assert job.check_level1() < 2e-6
    job.close()


def test_level1_tc_at_scale(tg):
    from topopt_gb300.workloads import cantilever_seeded_load
    bcs, loads = cantilever_seeded_load(256, 128, 128)
    pb = tg.Problem(256, 128, 128, 1.0, None, bcs, loads)
    job = _job(tg, pb, iters=1)
    assert job.check_level1() < 2e-6
    job.close()


def test_mixed_solve_with_level1_tc(tg):
    """The mixed solve with the tensor-core level 1 and with the stencil level 1
    both reach the FP64 solution; the inner iteration counts stay close."""
    from test_gpu_parity import smooth_modulus
    o = cantilever(64, 32, 32)
    pb = tg.Problem(64, 32, 32, 1.0, None, list(zip(o.bc_node, o.bc_comp, o.bc_val)),
                    list(zip(o.ld_node, o.ld_comp, o.ld_val)))
    E = smooth_modulus(pb)
    u64, _ = tg.fea_solve_mgcg_matfree(pb, E, tolerance=1e-10, max_iterations=600)
    its = {}
    try:
        for on in (True, False):
            tg.set_level1_tc(on)
            u, info = tg.fea_solve_mgcg_matfree(pb, E, tolerance=1e-10, max_iterations=600,
                                                options=tg.SolveOptions(precision=tg.PREC_MIXED))
            assert info.converged and not info.mixed_fallback, (on, info)
            assert rel(u, u64) < 1e-8
            its[on] = info.iterations
    finally:
        tg.set_level1_tc(True)
    assert abs(its[True] - its[False]) <= max(2, its[False] // 10), its
