"""The small levels of the mixed V-cycle (from the first of at most 4096 nodes
to the coarsest) in one thread-block-cluster launch, against the same V-cycle as
a launch per step: the same arithmetic in the same order, so the solves agree
bit for bit, and the fused form launches fewer kernels.  Both coarse smoothers
(damped Jacobi below 200K elements, Chebyshev above); the fused part starts at
level 2 on 64x32x32, level 3 on 96x48x48 and level 4 on 192x96x96.  GPU only."""
import numpy as np
import pytest

from oracle.oracle import cantilever

pytestmark = pytest.mark.gpu


def _pb(tg, nx, ny, nz):
    o = cantilever(nx, ny, nz)
    return tg.Problem(nx, ny, nz, 1.0, None, list(zip(o.bc_node, o.bc_comp, o.bc_val)),
                      list(zip(o.ld_node, o.ld_comp, o.ld_val)))


@pytest.mark.parametrize("dims", [(64, 32, 32), (96, 48, 48), (192, 96, 96)])
def test_fused_coarse_vcycle_bit_identical(tg, dims):
    from test_gpu_parity import smooth_modulus
    pb = _pb(tg, *dims)
    E = smooth_modulus(pb)
    out = {}
    try:
        for on in (True, False):
            tg.set_coarse_fused(on)
            k0 = tg.kernel_launches()
            u, info = tg.fea_solve_mgcg_matfree(pb, E, tolerance=1e-10, max_iterations=600,
                                                options=tg.SolveOptions(precision=tg.PREC_MIXED))
            assert info.converged and not info.mixed_fallback, (on, info)
            out[on] = (u, info.iterations, tg.kernel_launches() - k0)
    finally:
        tg.set_coarse_fused(False)
    assert out[True][1] == out[False][1]
    assert out[True][2] < out[False][2], (out[True][2], out[False][2])
    assert np.array_equal(out[True][0], out[False][0])


def test_fused_coarse_vcycle_design_run(tg):
    pb = _pb(tg, 128, 64, 64)
    hist = {}
    try:
        for on in (True, False):
            tg.set_coarse_fused(on)
            s = tg.simp_optimize(pb, tg.SimpParams(), tg.SimpOptions(
                volume_fraction=0.3, filter_radius=1.5, change_tol=0.0, max_iterations=6,
                cg_tolerance=1e-8, solve=tg.SolveOptions(precision=tg.PREC_MIXED)))
            hist[on] = [h["compliance"] for h in s["history"]]
    finally:
        tg.set_coarse_fused(False)
    assert hist[True] == hist[False]
