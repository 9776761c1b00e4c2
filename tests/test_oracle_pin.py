"""The CPU oracle (a C restatement of the reference) pinned against the
reference's own fixtures and against golden vectors produced by the reference's
own compiled code (tests/golden/make_golden.py).  CPU only."""
import json
import os

import numpy as np
import pytest

from oracle.oracle import Problem, cantilever, reference_path

REF_KE_JSON = reference_path("core", "tests", "fixtures", "fea", "hex_stiffness_reference.json")


@pytest.mark.skipif(not os.path.exists(REF_KE_JSON), reason="reference tree not mounted")
def test_ke_against_reference_fixture(port):
    ref = json.load(open(REF_KE_JSON))
    for key, case in ref["cases"].items():
        K = np.array(case["K"])
        got = port.hex8_stiffness(case["youngs_modulus"], case["poisson"], 1.0)
        # hex_stiffness_reference.json: entrywise <= 1e-10 * max|K|.
        assert np.abs(got - K).max() <= 1e-10 * np.abs(K).max(), key
        assert np.abs(got - got.T).max() <= 1e-12 * np.abs(got).max()
        ev = np.linalg.eigvalsh(got)
        assert (np.abs(ev) < 1e-10).sum() == 6
        assert abs(np.trace(got) - case["properties"]["trace"]) < 1e-12


def test_ke_golden_bit_exact(port, golden):
    assert np.array_equal(port.hex8_stiffness(1.0, 0.3, 1.0), golden["ke_nu30"])
    assert np.array_equal(port.hex8_stiffness(1.0, 0.4, 1.0), golden["ke_nu40"])
    assert np.array_equal(port.hex8_stiffness(2.0, 0.3, 0.5), golden["ke_h05_E2"])


def _apply_problem(golden):
    nx, ny, nz = (int(v) for v in golden["apply_dims"])
    return cantilever(nx, ny, nz, solid=golden["apply_solid"])


def test_apply_golden_bit_exact(port, golden):
    pb = _apply_problem(golden)
    y = port.apply(pb, golden["apply_u"], golden["apply_factor"])
    assert np.array_equal(y, golden["apply_y_graded"])
    y = port.apply(pb, golden["apply_u"], None, E=2.5)
    assert np.array_equal(y, golden["apply_y_uniform"])


def test_reduced_and_cg_golden(port, golden):
    pb = _apply_problem(golden)
    red = port.build_reduced(pb, golden["apply_factor"])
    assert red["ng"] == int(golden["red_ng"])
    for k in ("kept", "rhs", "invdiag"):
        assert np.array_equal(red[k], golden["red_" + k]), k
    u, it, res = port.solve_cg(pb, golden["apply_factor"], tol=1e-12)
    assert it == int(golden["cg_iters"])
    assert np.array_equal(u, golden["cg_u"])


def test_compliance_golden(port, golden):
    pb = cantilever(*(int(v) for v in golden["comp_dims"]))
    c = port.simp_compliance(pb, golden["comp_rho"], tol=1e-12)
    assert c["compliance"] == float(golden["comp_c"])
    assert np.array_equal(c["dc"], golden["comp_dc"])


def test_filter_and_oc_golden(port, golden):
    pb = _apply_problem(golden)
    for r, tag in ((1.5, "15"), (2.5, "25")):
        assert np.array_equal(port.filter(pb, golden["filt_x"], r, False), golden["filt_fwd_r" + tag])
        assert np.array_equal(port.filter(pb, golden["filt_x"], r, True), golden["filt_adj_r" + tag])
    assert np.array_equal(port.oc_update(pb, golden["oc_x"], golden["oc_dc"], 0.3, 1.5, 0.2),
                          golden["oc_xnew"])
    assert np.array_equal(port.oc_update(pb, golden["oc_x"], golden["oc_dc"], 0.4, 2.5, 0.1),
                          golden["oc_xnew_r25"])


def test_simp_loop_golden(port, golden):
    pb = cantilever(*(int(v) for v in golden["simp_dims"]))
    s = port.simp_optimize(pb, volfrac=0.3, radius=1.5, move=0.2, max_it=20, change_tol=0.01,
                           cg_tol=1e-10)
    assert s["iterations"] == int(golden["simp_iterations"])
    assert np.array_equal(s["hist_c"], golden["simp_hist_c"])
    assert np.array_equal(s["design"], golden["simp_design"])
    assert s["compliance"] == float(golden["simp_compliance"])


def _masked_problem(golden):
    mx, my, mz = (int(v) for v in golden["mask_dims"])
    return cantilever(mx, my, mz, solid=golden["mask_tags"]), golden["mask_mask"]


def test_masked_filter_golden(port, golden):
    """effective_design_mask and the mask-aware filter, bit-identical."""
    pb, mask = _masked_problem(golden)
    assert np.array_equal(port.effective_design_mask(pb, mask), golden["mask_eff"])
    x = golden["mask_x"]
    assert np.array_equal(port.filter_masked(pb, mask, x, 1.5, False), golden["mask_filt_fwd"])
    assert np.array_equal(port.filter_masked(pb, mask, x, 1.5, True), golden["mask_filt_adj"])


def test_masked_simp_loop_golden(port, golden):
    """The masked simp_optimize overload (oc_update_masked, pins, Active budget,
    FrozenVoid removed from the analysis grid), bit-identical trajectory."""
    pb, mask = _masked_problem(golden)
    s = port.simp_optimize_masked(pb, mask, volfrac=0.35, radius=1.5, move=0.2, max_it=15,
                                  change_tol=0.01, cg_tol=1e-10)
    assert s["iterations"] == int(golden["msimp_iterations"])
    assert np.array_equal(s["hist_c"], golden["msimp_hist_c"])
    assert np.array_equal(s["hist_change"], golden["msimp_hist_change"])
    assert np.array_equal(s["hist_vf"], golden["msimp_hist_vf"])
    assert np.array_equal(s["design"], golden["msimp_design"])
    assert np.array_equal(s["phys"], golden["msimp_phys"])
    assert s["compliance"] == float(golden["msimp_compliance"])
    assert s["volume_fraction"] == float(golden["msimp_volume_fraction"])
    eff = golden["mask_eff"]
    assert np.all(s["phys"][eff == 1] == 1.0) and np.all(s["phys"][eff == 2] == 0.0)
    assert np.all(s["design"][eff == 1] == 1.0) and np.all(s["design"][eff == 2] == 0.0)


def test_filter_properties(port):
    """Partition of unity and the adjoint identity (test_simp.cpp:312-386)."""
    rng = np.random.default_rng(3)
    solid = (rng.random(9 * 7 * 5) > 0.2).astype(np.uint8)
    pb = Problem(9, 7, 5, solid=solid)
    ones = solid.astype(float)
    f1 = port.filter(pb, ones, 1.5)
    assert np.allclose(f1[solid > 0], 1.0, atol=1e-15)
    a, b = rng.random(pb.nv) * solid, rng.random(pb.nv) * solid
    lhs = np.dot(port.filter(pb, a, 1.5), b)
    rhs = np.dot(a, port.filter(pb, b, 1.5, adjoint=True))
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


def test_void_gate_errors(port):
    from oracle.oracle import OracleError
    pb = cantilever(6, 3, 3, solid=np.zeros(54, np.uint8))
    with pytest.raises(OracleError) as e:
        port.build_reduced(pb)
    assert e.value.code == 2 and "singular" in str(e.value)
    solid = np.ones((3, 3, 6), np.uint8)
    solid[:, :, 5] = 0
    pb = cantilever(6, 3, 3, solid=solid.ravel())
    with pytest.raises(OracleError) as e:
        port.build_reduced(pb)
    assert e.value.code == 2 and "void DOF" in str(e.value)


def test_cant60_trajectory_prefix(port, golden):
    """The reference's CPU configuration (60x20x20 cantilever, 50 iterations in
    the golden run): the first 10 iterations of the oracle's loop match the
    reference's bit for bit."""
    pb = cantilever(60, 20, 20)
    s = port.simp_optimize(pb, volfrac=0.3, radius=1.5, move=0.2, max_it=10, change_tol=0.0,
                           cg_tol=1e-10)
    assert np.array_equal(s["hist_c"], golden["cant60_hist_c"][:10])
    assert np.array_equal(s["hist_change"], golden["cant60_hist_change"][:10])
    assert np.array_equal(s["hist_vf"], golden["cant60_hist_vf"][:10])


BENCH_JSON = reference_path("core", "tests", "fixtures", "benchmarks.json")


def test_projection_golden(port, golden):
    """heaviside_project and its derivative (simp.cpp projection helpers) on a
    grid of rho_tilde and beta, against the reference's own values."""
    for i, b in enumerate(golden["proj_beta"]):
        for j, rt in enumerate(golden["proj_rt"]):
            v, d = port.project(float(rt), float(b), 0.5)
            assert abs(v - golden["proj_value"][i, j]) <= 1e-15 * max(1.0, abs(v))
            assert abs(d - golden["proj_deriv"][i, j]) <= 1e-14 * max(1e-300, abs(d))


@pytest.mark.skipif(not os.path.exists(BENCH_JSON), reason="reference tree not mounted")
def test_projection_unit_reference_fixture(port):
    """The 15 analytic spot values of benchmarks.json at rel 1e-12
    (test_gate_v2.cpp:371-392)."""
    unit = json.load(open(BENCH_JSON))["projection_unit_reference"]
    n = 0
    for bkey, spots in unit.items():
        if not bkey.startswith("beta_"):
            continue
        b = float(bkey[5:])
        for rkey, spot in spots.items():
            v, d = port.project(float(rkey[3:]), b, 0.5)
            for got, want in ((v, spot["value"]), (d, spot["derivative"])):
                assert abs(got - want) <= 1e-12 * (abs(want) if want != 0.0 else 1.0)
            n += 1
    assert n == 15


def test_projected_simp_loop_golden(port, golden):
    """simp_optimize with a three-stage beta continuation (oc_update_projected,
    the stage loop, the final projection) bit-identical to the reference."""
    pb = cantilever(12, 4, 4)
    stages = [tuple(s) for s in golden["psimp_stages"].tolist()]
    stages = [(b, m, int(it)) for b, m, it in stages]
    s = port.simp_optimize(pb, volfrac=0.3, radius=1.5, change_tol=0.0, cg_tol=1e-10,
                           stages=stages)
    assert s["iterations"] == int(golden["psimp_iterations"]) == 22
    for k in ("hist_c", "hist_change", "hist_vf", "design", "phys"):
        assert np.array_equal(s[k], golden["psimp_" + k]), k
    assert s["compliance"] == float(golden["psimp_compliance"])
    assert s["volume_fraction"] == float(golden["psimp_volume_fraction"])


def test_gate_v2_first_stage_prefix(port, golden):
    """The Gate V2 cantilever (24x8x8, rmin 2.5, solves at 1e-9): the beta = 1
    stage of the oracle's loop equals the reference's, all 50 iterations."""
    from oracle.oracle import CONTINUATION, gate_v2_problem
    s = port.simp_optimize(gate_v2_problem("cantilever_24x8x8"), volfrac=0.3, radius=2.5,
                           change_tol=0.0, cg_tol=1e-9, stages=CONTINUATION[:1])
    assert np.array_equal(s["hist_c"], golden["gv2c_hist_c"][:50])
    assert np.array_equal(s["hist_change"], golden["gv2c_hist_change"][:50])


@pytest.mark.parametrize("key", ["gv2c", "gv2b"])
def test_gate_v2_reference_runs_pass_gates(golden, key):
    """The reference's own 300-iteration runs in the golden file satisfy the
    fixture's gates (the gates the CUDA path is held to)."""
    from oracle.oracle import gate_v2_metrics
    hc = golden[key + "_hist_c"]
    se = golden[key + "_fix_stage_end"]
    rel1, rel8 = golden[key + "_gate_rel"]
    assert hc.size == 300
    assert abs(hc[49] - se[0]) <= rel1 * se[0]
    assert abs(hc[199] - se[3]) <= rel8 * se[3]
    c = float(golden[key + "_compliance"])
    g = golden[key + "_gate_final"]
    if bool(golden[key + "_gate_final_is_band"]):
        assert g[0] <= c <= g[1]
    else:
        assert abs(c - g[0]) <= g[1] * g[0]
    assert abs(float(golden[key + "_volume_fraction"]) - float(golden[key + "_fix_vf"])) <= \
        float(golden[key + "_gate_vf_abs"])
    nx = 24 if key == "gv2c" else 48
    ncomp, mnd, ysym = gate_v2_metrics(nx, 8, 8, golden[key + "_phys"])
    assert ncomp == int(golden[key + "_gate_components"])
    assert ysym <= float(golden[key + "_gate_ysym"])
    assert mnd <= float(golden[key + "_gate_mnd"])


def test_hex8_stress_golden(port, golden):
    """hex8_stress (hex_element.cpp:242-316) bit-identical to the reference, at
    the centre and at random natural points."""
    for q in range(golden["stress_ue"].shape[0]):
        sig, vm = port.hex8_stress(*golden["stress_mat"][q], golden["stress_ue"][q],
                                   *golden["stress_pts"][q])
        assert np.array_equal(sig, golden["stress_sigma"][q])
        assert vm == golden["stress_vm"][q]


def test_stress_margin_rules(port):
    """compute_stress_margin (report.cpp:464-491): zero stress = unbounded
    margin, z_knockdown scales the interlayer term, invalid inputs refused."""
    from oracle.oracle import OracleError
    assert port.stress_margin(50.0, 0.7, 10.0, 3.0) == (5.0, 0.7 * 50.0 / 3.0, 5.0)
    assert port.stress_margin(50.0, 1.0, 0.0, 0.0) == (np.inf, np.inf, np.inf)
    assert port.stress_margin(50.0, 1.0, 0.0, 2.0)[2] == 25.0
    for bad in ((0.0, 1.0, 1.0, 1.0), (50.0, 1.5, 1.0, 1.0), (50.0, 1.0, -1.0, 1.0)):
        with pytest.raises(OracleError):
            port.stress_margin(*bad)


def _ladder_problem(golden):
    nx, ny, nz = (int(v) for v in golden["lad_dims"])
    return cantilever(nx, ny, nz, solid=golden["lad_tags"])


def test_analysis_and_load_path_golden(port, golden):
    """The fixed-design analysis (certification solve, printed-voxel stress,
    interlayer tension along a tilted build direction, margins) and the
    load-path belt, bit-identical to the reference's own pieces."""
    pb = _ladder_problem(golden)
    a, vm = port.analyze_fixed_design(pb, golden["ana_density"], yield_strength=30.0,
                                      margin_stop=25.0, build_dir=(0.3, -0.2, 0.9),
                                      cg_tol=1e-10)
    assert np.array_equal(vm, golden["ana_vm"])
    got = [a["compliance"], a["max_von_mises"], a["max_interlayer"], a["margin_in_plane"],
           a["margin_interlayer"], a["margin_worst"]]
    assert np.array_equal(np.array(got), golden["ana_d"])
    assert [a["printed_voxels"], a["load_path_ok"], a["accepted"]] == golden["ana_i"].tolist()
    d = golden["ana_density"].reshape(8, 6, 20).copy()
    assert port.load_path_connected(pb, d.ravel()) == bool(golden["lp_connected"][0])
    d[:, :, 10] = 0.0
    assert port.load_path_connected(pb, d.ravel()) == bool(golden["lp_connected"][1]) is False


@pytest.mark.parametrize("tag,margin_stop", [("a", 1.0), ("b", 25.0)])
def test_ladder_walk_golden(port, golden, tag, margin_stop):
    """The minimize_plastic ladder walk (OC, warm-start inheritance): every
    rung's trajectory, analysis and verdict, the severed rung rejected without
    stopping (a) and the margin stop (b), bit-identical to the reference."""
    pb = _ladder_problem(golden)
    L = port.ladder(pb, None, golden["lad_ladder"], max_it=25, yield_strength=30.0,
                    margin_stop=margin_stop, cg_tol=1e-9)
    rd = np.array([[r["volume_fraction"], r["compliance"], r["analysis"]["max_von_mises"],
                    r["analysis"]["max_interlayer"], r["analysis"]["margin_worst"],
                    r["analysis"]["margin_effective"]] for r in L["rungs"]])
    ri = np.array([[r["iterations"], r["trajectory_ok"], r["analysed"], r["accepted"],
                    r["analysis"]["load_path_ok"]] for r in L["rungs"]])
    assert np.array_equal(rd, golden[f"lad{tag}_rung_d"])
    assert np.array_equal(ri, golden[f"lad{tag}_rung_i"])
    assert [L["evaluated"], L["recommended"], int(L["stopped_on_margin"])] == \
        golden[f"lad{tag}_out"].tolist()
    assert np.array_equal(L["design"], golden[f"lad{tag}_design"])
    assert np.array_equal(L["phys"], golden[f"lad{tag}_phys"])


def test_mma_plateau_run_golden(port, golden):
    """simp_optimize with the MMA updater (Svanberg's asymptotes, the separable
    subproblem and its 1-D dual, mma_joint.cpp) stopped by the objective plateau
    (mma_objective_plateau, defaults 10 / 1e-3 / 0.05 / 3): bit-identical."""
    s = port.simp_optimize_mma(cantilever(12, 4, 4), max_it=200, cg_tol=1e-10)
    assert [s["iterations"], int(s["converged"])] == golden["mma_out"].tolist()
    assert s["iterations"] < 200 and s["converged"]
    for k in ("hist_c", "hist_change", "hist_vf", "design", "phys"):
        assert np.array_equal(s[k], golden["mma_" + k]), k
    assert s["compliance"] == float(golden["mma_compliance"])


def test_mma_masked_run_golden(port, golden):
    """mma_update_masked (simp.cpp:2736-2784): only Active voxels move, the rest
    of x_new is 0, pins on the physical density; bit-identical."""
    pb, mask = _masked_problem(golden)
    s = port.simp_optimize_mma(pb, mask=mask, volfrac=0.35, max_it=40, cg_tol=1e-10)
    for k in ("hist_c", "hist_change", "design", "phys"):
        assert np.array_equal(s[k], golden["mmam_" + k]), k
    assert s["compliance"] == float(golden["mmam_compliance"])
    assert s["volume_fraction"] == float(golden["mmam_volume_fraction"])


def test_active_domain_mask_golden(port, golden):
    """active_domain_mask (core + Load/Fixture pin, the x -> y -> z Chebyshev
    dilation, AND solid) at bands 0, 1, 2, 3, 64, the escape count and the auto
    band: identical to the reference's."""
    nx, ny, nz = (int(v) for v in golden["ad_dims"])
    pb = Problem(nx, ny, nz, 1.0, golden["ad_tags"])
    rho = golden["ad_rho"]
    for b, want in zip(golden["ad_bands"], golden["ad_masks"]):
        assert np.array_equal(port.active_domain_mask(pb, rho, 1e-3, int(b)), want), b
    assert port.active_domain_escape_count(pb, rho, golden["ad_prev"], 1e-3) == \
        int(golden["ad_escapes"])
    assert port.active_domain_escape_count(pb, rho, None, 1e-3) == 0
    got = [port.active_domain_auto_band(float(r)) for r in golden["ad_radii"]]
    assert got == golden["ad_auto"].tolist()


def ad_reason(golden, name):
    """The reference's latch reason.  The reference build here routes the
    matrix-free multigrid solve to its exact Jacobi-PCG (oracle/ref_shim.cpp), so
    a failed restricted solve names that function; the library itself names
    fea_solve_mgcg_matfree, as the reference's own build does."""
    r = bytes(golden[f"adr_{name}_reason"]).decode()
    return r.replace("fea_solve_cg_matfree:", "fea_solve_mgcg_matfree:")


@pytest.mark.parametrize("name", ["restricted", "masked", "escape", "failed", "latch", "mma"])
def test_active_domain_runs_golden(port, golden, name):
    """simp_optimize with active_domain_band (active_domain_solve,
    simp.cpp:1809-1896): the restricted trajectory solves, the per-iteration
    active fraction, each latch (escape, fraction, failed restricted solve) with
    its iteration and reason, and the full-domain certification: identical."""
    from oracle.oracle import active_domain_case
    pb, mask, seed, band, radius, vf, its, upd = active_domain_case(name)
    s = port.simp_optimize_active(pb, band, mask=mask, seed=seed, radius=radius, volfrac=vf,
                                  move=0.2, max_it=its, change_tol=0.0, cg_tol=1e-9,
                                  updater=upd)
    k = "adr_" + name
    assert [s["iterations"], s["band"], int(s["latched"]), s["latch_iteration"],
            s["escape_count"]] == golden[k + "_i"].tolist()
    assert np.array_equal(s["hist_af"], golden[k + "_hist_af"])
    assert np.array_equal(s["hist_c"], golden[k + "_hist_c"])
    assert np.array_equal(s["phys"], golden[k + "_phys"])
    assert [s["compliance"], s["volume_fraction"], s["fraction_mean"]] == \
        golden[k + "_d"].tolist()
    assert s["reason"] == ad_reason(golden, name)
    if name in ("restricted", "masked", "mma"):
        assert not s["latched"] and s["hist_af"].max() < 0.85
