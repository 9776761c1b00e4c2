"""Level 1's Galerkin matrices on the tensor-core fast path formed by the
bandwidth-bound kernel against the general kernel for every element: the
matrices are bit-identical, so whole mixed solves are.  An even grid and an odd
one with boundary-aligned coarsening (whose half elements stay on the general
kernel).  GPU only."""
import numpy as np
import pytest

from oracle.oracle import cantilever

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dims", [(128, 64, 64), (127, 63, 65)])
def test_level1_galerkin_fast_path_bit_identical(tg, dims):
    nx, ny, nz = dims
    o = cantilever(nx, ny, nz)
    pb = tg.Problem(nx, ny, nz, 1.0, None, list(zip(o.bc_node, o.bc_comp, o.bc_val)),
                    list(zip(o.ld_node, o.ld_comp, o.ld_val)))
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    rho = 0.5 + 0.45 * np.sin(2 * np.pi * x / nx) * np.cos(2 * np.pi * y / ny) * np.cos(np.pi * z / nz)
    E = (1e-3 + rho ** 3).ravel()
    out = {}
    try:
        for on in (True, False):
            tg.set_level1_galerkin_fast(on)
            u, info = tg.fea_solve_mgcg_matfree(pb, E, tolerance=1e-8, max_iterations=600,
                                                options=tg.SolveOptions(precision=tg.PREC_MIXED))
            assert info.converged and not info.mixed_fallback, (on, info)
            out[on] = (u, info.iterations)
    finally:
        tg.set_level1_galerkin_fast(True)
    assert out[True][1] == out[False][1]
    assert np.array_equal(out[True][0], out[False][0])
