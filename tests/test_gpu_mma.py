"""The MMA updater on the GPU (SimpUpdater::MMA: mma_update, mma_update_masked,
mma_update_joint, the objective-plateau stop) against the reference's own runs
(the golden file) and the oracle.  GPU only.

Tolerances.  The per-voxel subproblem (asymptotes, coefficients, move box,
candidate) rounds exactly like the reference; the dual's constraint sums are
fixed-order device sums, so a bisection branch on a near-tie may go the other
way and the multiplier differ in its last bits.  Trajectories are held to 1e-6
relative in compliance, designs to 1e-4, and the plateau stop to the same
iteration.
"""
import numpy as np
import pytest

from oracle.oracle import cantilever

pytestmark = pytest.mark.gpu


def _tg_problem(tg, o, tags=None):
    return tg.Problem(o.nx, o.ny, o.nz, o.h, tags, list(zip(o.bc_node, o.bc_comp, o.bc_val)),
                      list(zip(o.ld_node, o.ld_comp, o.ld_val)))


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("prec", [0, 1])
def test_mma_plateau_run_matches_reference(tg, golden, prec):
    o = cantilever(12, 4, 4)
    s = tg.simp_optimize(_tg_problem(tg, o), tg.SimpParams(), tg.SimpOptions(
        volume_fraction=0.3, filter_radius=1.5, move=0.2, max_iterations=200,
        cg_tolerance=1e-10, updater=tg.UPDATER_MMA, solve=tg.SolveOptions(precision=prec)))
    assert [s["iterations"], int(s["converged"])] == golden["mma_out"].tolist()
    hc = np.array([h["compliance"] for h in s["history"]])
    assert rel(hc, golden["mma_hist_c"]) < 1e-6
    assert rel(s["design"], golden["mma_design"]) < 1e-4
    assert abs(s["compliance"] - float(golden["mma_compliance"])) <= 1e-6 * s["compliance"]


def test_mma_masked_matches_reference(tg, golden):
    nx, ny, nz = (int(v) for v in golden["mask_dims"])
    tags, mask = golden["mask_tags"], golden["mask_mask"]
    o = cantilever(nx, ny, nz, solid=tags)
    s = tg.simp_optimize(_tg_problem(tg, o, tags), tg.SimpParams(), tg.SimpOptions(
        volume_fraction=0.35, filter_radius=1.5, move=0.2, max_iterations=40,
        cg_tolerance=1e-10, updater=tg.UPDATER_MMA), mask=mask)
    hc = np.array([h["compliance"] for h in s["history"]])
    assert s["iterations"] == len(golden["mmam_hist_c"])
    assert rel(hc, golden["mmam_hist_c"]) < 1e-6
    assert rel(s["physical_density"], golden["mmam_phys"]) < 1e-4
    eff = golden["mask_eff"]
    assert np.all(s["physical_density"][eff == 1] == 1.0)
    assert np.all(s["design"][eff != 0] == 0.0)  # mma_update_joint leaves non-dof at 0


def test_mma_matches_oracle_mid_grid(tg, port):
    """A 40x16x12 cantilever (multi-pass dual evaluation) against the oracle."""
    o = cantilever(40, 16, 12)
    want = port.simp_optimize_mma(o, max_it=15, cg_tol=1e-10, plateau_window=0,
                                  change_tol=0.0)
    s = tg.simp_optimize(_tg_problem(tg, o), tg.SimpParams(), tg.SimpOptions(
        volume_fraction=0.3, filter_radius=1.5, move=0.2, max_iterations=15, change_tol=0.0,
        cg_tolerance=1e-10, updater=tg.UPDATER_MMA, mma_plateau_window=0))
    hc = np.array([h["compliance"] for h in s["history"]])
    assert rel(hc, want["hist_c"]) < 1e-6
    assert rel(s["design"], want["design"]) < 1e-5


def test_mma_rejects_projection(tg):
    o = cantilever(6, 3, 3)
    with pytest.raises(ValueError, match="MMA updater does not support"):
        tg.simp_optimize(_tg_problem(tg, o), tg.SimpParams(), tg.SimpOptions(
            updater=tg.UPDATER_MMA, projection=[(1.0, 0.2, 2)]))
