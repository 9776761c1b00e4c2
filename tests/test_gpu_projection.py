"""Heaviside projection and beta continuation on the GPU (simp.cpp:352-374,
:1638-1726, the stage loop :2158-2517) against the reference's values, the
oracle, and the Gate V2 known-answer fixtures (benchmarks.json through the
golden file).  GPU only.

Tolerances.  The projection's tanh / cosh of beta (rt - eta) are the device's,
within a few units in the last place of the host library's: the projected value
is held to 1e-14 relative (1e-15 absolute near 0) and the derivative to 1e-13
relative.  Everything downstream (a bisection branch on a near-tie can go the
other way) is held to tolerances: projected OC updates within 1e-6 of the
oracle's, trajectories within 1e-6 relative while the design is smooth, and the
Gate V2 gates -- stage-end compliances at beta 1 and 8 within 1 %, the final
compliance band or 5 %, projected volume within 0.01, one 6-connected component
at 0.5, y-symmetry within 1e-6, discreteness M_nd under the gate.
"""
import numpy as np
import pytest

from oracle.oracle import CONTINUATION, GATE_V2, cantilever, gate_v2_metrics, gate_v2_problem

pytestmark = pytest.mark.gpu


def _tg_problem(tg, o, solid=None):
    return tg.Problem(o.nx, o.ny, o.nz, 1.0, solid, list(zip(o.bc_node, o.bc_comp, o.bc_val)),
                      list(zip(o.ld_node, o.ld_comp, o.ld_val)))


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_projection_kernel_matches_reference(tg, golden):
    rt = golden["proj_rt"]
    for i, beta in enumerate(golden["proj_beta"]):
        v, d = tg.heaviside_project(rt, beta, 0.5)
        want_v, want_d = golden["proj_value"][i], golden["proj_deriv"][i]
        assert np.all(np.abs(v - want_v) <= 1e-14 * np.abs(want_v) + 1e-15)
        assert np.all(np.abs(d - want_d) <= 1e-13 * np.abs(want_d))
        # The 15 analytic spot values (rt 0, .3, .5, .7, 1 at beta 1, 8, 32)
        # at the fixture's rel 1e-12 (test_gate_v2.cpp:371-392).
        if beta in (1.0, 8.0, 32.0):
            assert np.all(np.abs(v[:5] - want_v[:5]) <= 1e-12 * np.abs(want_v[:5]) + 1e-15)
            assert np.all(np.abs(d[:5] - want_d[:5]) <= 1e-12 * np.abs(want_d[:5]))


def test_projection_argument_errors(tg):
    with pytest.raises(ValueError, match="beta must be finite"):
        tg.heaviside_project(np.zeros(3), 0.0)
    with pytest.raises(ValueError, match="eta must be in"):
        tg.heaviside_project(np.zeros(3), 1.0, 1.0)
    sched = tg.heaviside_continuation_schedule()
    assert sched == [tuple(s) for s in CONTINUATION]


@pytest.mark.parametrize("beta", [1.0, 8.0, 32.0])
def test_oc_update_projected_matches_oracle(tg, port, beta):
    """oc_update_projected on a grid with voids: the device update is the
    oracle's up to the last bits of the projection."""
    rng = np.random.default_rng(int(beta))
    nx, ny, nz = 18, 9, 7
    solid = (rng.random(nx * ny * nz) > 0.12).astype(np.uint8)
    o = cantilever(nx, ny, nz, solid=solid)
    x = np.where(solid > 0, 0.05 + 0.9 * rng.random(o.nv), 0.0)
    xt = port.filter(o, x, 1.5)
    dc = -np.where(solid > 0, rng.random(o.nv) * 3.0, 0.0)
    want = port.oc_update_projected(o, x, xt, dc, beta, 0.3)
    pb = tg.Problem(nx, ny, nz, 1.0, solid)
    got = tg.oc_update_projected(pb, 1.5, x, xt, dc, beta, 0.5, 0.3)
    assert np.abs(got - want).max() <= 1e-6
    assert np.all(got[solid == 0] == 0.0)


@pytest.mark.parametrize("prec", [0, 1])
def test_projected_loop_matches_reference(tg, golden, prec):
    """A three-stage continuation (beta 1, 4, 16) on the 12x4x4 cantilever,
    against the reference's own run."""
    o = cantilever(12, 4, 4)
    stages = [(float(b), float(m), int(it)) for b, m, it in golden["psimp_stages"].tolist()]
    s = tg.simp_optimize(_tg_problem(tg, o), tg.SimpParams(), tg.SimpOptions(
        volume_fraction=0.3, filter_radius=1.5, change_tol=0.0, cg_tolerance=1e-10,
        projection=stages, solve=tg.SolveOptions(precision=prec)))
    assert s["iterations"] == int(golden["psimp_iterations"]) == 22
    hc = np.array([h["compliance"] for h in s["history"]])
    betas = [h["beta"] for h in s["history"]]
    assert betas == [1.0] * 8 + [4.0] * 8 + [16.0] * 6
    assert rel(hc, golden["psimp_hist_c"]) < 1e-6
    assert rel(s["design"], golden["psimp_design"]) < 1e-4
    assert rel(s["physical_density"], golden["psimp_phys"]) < 1e-4
    assert abs(s["volume_fraction"] - float(golden["psimp_volume_fraction"])) < 1e-6
    assert abs(s["compliance"] - float(golden["psimp_compliance"])) <= 1e-5 * s["compliance"]


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("name", GATE_V2)
def test_gate_v2(tg, golden, name, prec):
    """Gate V2 (test_gate_v2.cpp:396-580): the locked projected formulation on
    the two benchmark problems, 6 stages x 50 iterations, held to the fixture's
    gates; the smooth beta = 1 stage also tracks the reference's own run."""
    key = "gv2c" if name.startswith("cantilever") else "gv2b"
    o = gate_v2_problem(name)
    s = tg.simp_optimize(_tg_problem(tg, o), tg.SimpParams(), tg.SimpOptions(
        volume_fraction=0.3, filter_radius=2.5, change_tol=0.0, cg_tolerance=1e-9,
        projection=tg.heaviside_continuation_schedule(), projection_eta=0.5,
        solve=tg.SolveOptions(precision=prec)))
    assert s["iterations"] == 300 and not s["converged"]
    hist = s["history"]
    hc = np.array([h["compliance"] for h in hist])
    for si, (beta, move, _) in enumerate(CONTINUATION):
        rows = hist[50 * si:50 * (si + 1)]
        assert all(r["beta"] == beta for r in rows)
        assert all(r["change"] <= move + 1e-9 for r in rows)
    # The beta = 1 stage, against the reference's trajectory.
    assert rel(hc[:50], golden[key + "_hist_c"][:50]) < 1e-6
    se = golden[key + "_fix_stage_end"]
    r1, r8 = golden[key + "_gate_rel"]
    assert abs(hc[49] - se[0]) <= r1 * se[0]
    assert abs(hc[199] - se[3]) <= r8 * se[3]
    g = golden[key + "_gate_final"]
    c = s["compliance"]
    if bool(golden[key + "_gate_final_is_band"]):
        assert g[0] <= c <= g[1]
    else:
        assert abs(c - g[0]) <= g[1] * g[0]
    assert abs(s["volume_fraction"] - float(golden[key + "_fix_vf"])) <= \
        float(golden[key + "_gate_vf_abs"])
    ncomp, mnd, ysym = gate_v2_metrics(o.nx, o.ny, o.nz, s["physical_density"])
    assert ncomp == int(golden[key + "_gate_components"])
    assert ysym <= float(golden[key + "_gate_ysym"])
    assert mnd <= float(golden[key + "_gate_mnd"])


def test_projected_masked_loop_matches_oracle(tg, port, golden):
    """The masked overload with a continuation plan (project_active,
    simp.cpp:2789, :3203): FrozenSolid / FrozenVoid pins kept, trajectory within
    tolerance of the oracle's."""
    nx, ny, nz = (int(v) for v in golden["mask_dims"])
    tags, mask = golden["mask_tags"], golden["mask_mask"]
    o = cantilever(nx, ny, nz, solid=tags)
    stages = [(1.0, 0.2, 6), (4.0, 0.2, 6)]
    want = port.simp_optimize_masked(o, mask, volfrac=0.35, radius=1.5, change_tol=0.0,
                                     cg_tol=1e-10, stages=stages)
    s = tg.simp_optimize(_tg_problem(tg, o, tags), tg.SimpParams(), tg.SimpOptions(
        volume_fraction=0.35, filter_radius=1.5, change_tol=0.0, cg_tolerance=1e-10,
        projection=stages), mask=mask)
    assert s["iterations"] == want["iterations"] == 12
    hc = np.array([h["compliance"] for h in s["history"]])
    assert rel(hc, want["hist_c"]) < 1e-6
    assert rel(s["physical_density"], want["phys"]) < 1e-4
    eff = golden["mask_eff"]
    assert np.all(s["physical_density"][eff == 1] == 1.0)
    assert np.all(s["physical_density"][eff == 2] == 0.0)


def test_job_stage_selection(tg):
    """SimpJob.set_stage: steps run at the selected stage's beta."""
    o = cantilever(12, 4, 4)
    job = tg.SimpJob(_tg_problem(tg, o), tg.SimpParams(), tg.SimpOptions(
        volume_fraction=0.3, change_tol=0.0, projection=[(1.0, 0.2, 3), (8.0, 0.1, 3)]))
    assert job.step()["beta"] == 1.0
    job.set_stage(1)
    r = job.step()
    assert r["beta"] == 8.0 and r["change"] <= 0.1 + 1e-12
    with pytest.raises(ValueError):
        job.set_stage(2)
    job.close()
