"""Parity of the CUDA path (through the C ABI) with the oracle and the golden
vectors of the reference's own code.  GPU only.

Tolerances: compliance within 1e-9 relative and displacement within
1e-8 relative max-norm for FP64 solves (both sides solved tighter than that);
integer and index work (kept-DOF mask) bit-exact; the density filter and the OC
update bit-exact (they round exactly like the reference).  The operator is a
different (Walsh-modal) evaluation of the same Ke u, so it is compared at 1e-13
relative to its max entry in FP64, 1e-6 in FP32.
"""
import numpy as np
import pytest

from oracle.oracle import cantilever

pytestmark = pytest.mark.gpu


def _pb(tg, golden, key="apply"):
    nx, ny, nz = (int(v) for v in golden[key + "_dims"])
    o = cantilever(nx, ny, nz, solid=golden.get(key + "_solid"))
    tags = None if o.solid is None else o.solid
    bcs = list(zip(o.bc_node, o.bc_comp, o.bc_val))
    loads = list(zip(o.ld_node, o.ld_comp, o.ld_val))
    return tg.Problem(nx, ny, nz, 1.0, tags, bcs, loads), o


def smooth_modulus(pb, seed=2):
    """A SIMP-like (filtered, hence smooth) density field rho in [1e-3, 1], E = rho^3."""
    k, j, i = np.meshgrid(np.arange(pb.nz), np.arange(pb.ny), np.arange(pb.nx), indexing="ij")
    rng = np.random.default_rng(seed)
    rho = np.full(i.shape, 0.3)
    for _ in range(4):
        fx, fy, fz, ph = rng.uniform(0.5, 3.0, 3).tolist() + [rng.uniform(0, 6.3)]
        rho += 0.15 * np.sin(fx * np.pi * i / pb.nx + fy * np.pi * j / pb.ny + fz * np.pi * k / pb.nz + ph)
    return np.clip(rho, 1e-3, 1.0).ravel() ** 3


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_apply_matches_reference_golden(tg, golden):
    pb, _ = _pb(tg, golden)
    y = tg.fea_matfree_apply(pb, golden["apply_u"], youngs_per_voxel=golden["apply_factor"])
    assert rel(y, golden["apply_y_graded"]) < 1e-13
    y = tg.fea_matfree_apply(pb, golden["apply_u"], youngs_modulus=2.5)
    assert rel(y, golden["apply_y_uniform"]) < 1e-13
    yf = tg.fea_matfree_apply(pb, golden["apply_u"], youngs_per_voxel=golden["apply_factor"],
                              precision=tg.PREC_MIXED)
    assert rel(yf, golden["apply_y_graded"]) < 2e-6


@pytest.mark.parametrize("dims", [(1, 1, 1), (2, 1, 3), (17, 9, 8), (33, 17, 16), (40, 24, 9)])
def test_apply_matches_oracle_sizes(tg, port, dims):
    """Brick edges, partial bricks and one-element grids."""
    rng = np.random.default_rng(sum(dims))
    nx, ny, nz = dims
    solid = (rng.random(nx * ny * nz) > 0.1).astype(np.uint8)
    o = cantilever(nx, ny, nz, solid=solid)
    pb = tg.Problem(nx, ny, nz, 1.0, solid)
    u = rng.standard_normal(o.ndof)
    f = rng.random(o.nv) + 1e-3
    assert rel(tg.fea_matfree_apply(pb, u, youngs_per_voxel=f), port.apply(o, u, f)) < 1e-13


def test_apply_properties_at_scale(tg):
    """256x128x128 (the large benchmark grid): rigid translations are in the
    null space, the operator is symmetric (u.Kv = v.Ku) and linear."""
    nx, ny, nz = 256, 128, 128
    pb = tg.Problem(nx, ny, nz)
    rng = np.random.default_rng(7)
    f = rng.random(pb.nv) * 0.999 + 0.001
    t = np.zeros(pb.ndof)
    t[1::3] = 1.0
    y = tg.fea_matfree_apply(pb, t, youngs_per_voxel=f)
    assert np.abs(y).max() < 1e-12
    u, v = rng.standard_normal(pb.ndof), rng.standard_normal(pb.ndof)
    ku = tg.fea_matfree_apply(pb, u, youngs_per_voxel=f)
    kv = tg.fea_matfree_apply(pb, v, youngs_per_voxel=f)
    assert abs(u @ kv - v @ ku) <= 1e-12 * abs(u @ kv)
    kw = tg.fea_matfree_apply(pb, 2.0 * u - 3.0 * v, youngs_per_voxel=f)
    assert rel(kw, 2.0 * ku - 3.0 * kv) < 1e-13


def test_reduced_system_bit_exact(tg, golden):
    pb, _ = _pb(tg, golden)
    red = tg.fea_build_reduced(pb, golden["apply_factor"])
    assert red["ng"] == int(golden["red_ng"])
    assert np.array_equal(red["kept"], golden["red_kept"])
    assert np.array_equal(red["rhs"], golden["red_rhs"])
    assert rel(red["invdiag"], golden["red_invdiag"]) < 1e-14


@pytest.mark.parametrize("solver,prec,tol", [(1, 0, 1e-12), (0, 0, 1e-12), (0, 1, 1e-12)])
def test_solve_matches_reference(tg, golden, solver, prec, tol):
    pb, _ = _pb(tg, golden)
    opts = tg.SolveOptions(solver=solver, precision=prec)
    u, info = tg.fea_solve_mgcg_matfree(pb, golden["apply_factor"], tolerance=tol, options=opts)
    assert info.converged
    assert rel(u, golden["cg_u"]) < 1e-8
    if solver == 0:
        assert info.used_multigrid and info.mg_levels >= 2
    if prec == 1:  # white-noise modulus: the mixed form may hand over to FP64 MG-PCG
        assert info.matvecs_lowp > 0


def test_mixed_solve_large(tg):
    """96x48x48 cantilever with a smooth (SIMP-like) modulus field: the mixed form
    (FP32 V-cycle, FP32 coarse stencils) converges on its own, to the FP64 solution."""
    pb = tg.Problem.cantilever(96, 48, 48)
    E = smooth_modulus(pb)
    u64, i64 = tg.fea_solve_mgcg_matfree(pb, E, tolerance=1e-10)
    u32, i32 = tg.fea_solve_mgcg_matfree(pb, E, tolerance=1e-10, options=tg.SolveOptions(
        precision=tg.PREC_MIXED))
    assert not i32.mixed_fallback and i32.inner_breakdowns == 0, i32
    assert i64.used_multigrid, i64
    assert rel(u32, u64) < 1e-8


def test_compliance_and_sensitivity(tg, golden):
    nx, ny, nz = (int(v) for v in golden["comp_dims"])
    o = cantilever(nx, ny, nz)
    pb = tg.Problem(nx, ny, nz, 1.0, None, list(zip(o.bc_node, o.bc_comp, o.bc_val)),
                    list(zip(o.ld_node, o.ld_comp, o.ld_val)))
    r = tg.simp_compliance(pb, tg.SimpParams(), golden["comp_rho"], tolerance=1e-12)
    c_ref = float(golden["comp_c"])
    assert abs(r["compliance"] - c_ref) <= 1e-9 * abs(c_ref)
    assert rel(r["u"], golden["comp_u"]) < 1e-8
    assert rel(r["dcompliance"], golden["comp_dc"]) < 1e-8


def test_filter_bit_exact(tg, golden):
    pb, _ = _pb(tg, golden)
    for r, tag in ((1.5, "15"), (2.5, "25")):
        f = tg.make_density_filter(pb, r)
        assert np.array_equal(f.filter_density(golden["filt_x"]), golden["filt_fwd_r" + tag])
        assert np.array_equal(f.filter_sensitivity(golden["filt_x"]), golden["filt_adj_r" + tag])


def test_oc_update_bit_exact(tg, golden):
    pb, _ = _pb(tg, golden)
    xn = tg.oc_update(pb, tg.make_density_filter(pb, 1.5), golden["oc_x"], golden["oc_dc"], 0.3,
                      0.2, 1e-3)
    assert np.array_equal(xn, golden["oc_xnew"])
    xn = tg.oc_update(pb, tg.make_density_filter(pb, 2.5), golden["oc_x"], golden["oc_dc"], 0.4,
                      0.1, 1e-3)
    assert np.array_equal(xn, golden["oc_xnew_r25"])


def test_oc_update_bit_exact_large(tg, port):
    """A 96x48x48 OC step against the oracle, with the oracle's own dc."""
    rng = np.random.default_rng(11)
    nx, ny, nz = 96, 48, 48
    o = cantilever(nx, ny, nz)
    pb = tg.Problem(nx, ny, nz)
    x = rng.random(o.nv) * 0.8 + 0.1
    dc = -rng.random(o.nv) * 5.0
    assert np.array_equal(tg.oc_update(pb, tg.make_density_filter(pb, 1.5), x, dc, 0.3),
                          port.oc_update(o, x, dc, 0.3))


def test_simp_optimize_trajectory(tg, golden):
    nx, ny, nz = (int(v) for v in golden["simp_dims"])
    o = cantilever(nx, ny, nz)
    pb = tg.Problem(nx, ny, nz, 1.0, None, list(zip(o.bc_node, o.bc_comp, o.bc_val)),
                    list(zip(o.ld_node, o.ld_comp, o.ld_val)))
    s = tg.simp_optimize(pb, tg.SimpParams(), tg.SimpOptions(volume_fraction=0.3, max_iterations=20,
                                                              cg_tolerance=1e-10))
    hc = np.array([h["compliance"] for h in s["history"]])
    n = int(golden["simp_iterations"])
    assert s["iterations"] == n
    # Solves at 1e-10 on both sides: the first compliance to 1e-9, the
    # trajectory (fed by solver-level differences) to 1e-6.
    assert abs(hc[0] - golden["simp_hist_c"][0]) <= 1e-9 * hc[0]
    assert rel(hc, golden["simp_hist_c"]) < 1e-6
    assert rel(s["design"], golden["simp_design"]) < 1e-5
    assert abs(s["compliance"] - float(golden["simp_compliance"])) <= 1e-6 * s["compliance"]


def test_void_gate_errors(tg):
    pb = tg.Problem.cantilever(6, 3, 3, tags=np.zeros(54, np.uint8))
    with pytest.raises(RuntimeError, match="singular"):
        tg.fea_solve_mgcg_matfree(pb, np.ones(54))
    tags = np.ones((3, 3, 6), np.uint8)
    tags[:, :, 5] = 0
    pb = tg.Problem.cantilever(6, 3, 3, tags=tags.ravel())
    with pytest.raises(RuntimeError, match="void DOF"):
        tg.fea_solve_mgcg_matfree(pb, np.ones(54))


def test_nonconvergence_raises(tg):
    pb = tg.Problem.cantilever(16, 8, 8)
    with pytest.raises(tg.SolverNonConvergence) as e:
        tg.fea_solve_mgcg_matfree(pb, np.ones(pb.nv), tolerance=1e-12, max_iterations=1,
                                  options=tg.SolveOptions(solver=tg.SOLVER_JACOBI_CG))
    assert e.value.iterations >= 1


@pytest.mark.parametrize("dims", [(63, 31, 31), (45, 22, 17)])
def test_aligned_coarsening_odd_grids(tg, dims):
    """Boundary-aligned coarsening of odd axes: the same solution as the
    reference's padded hierarchy, in fewer MG-PCG iterations."""
    pb = tg.Problem.cantilever(*dims)
    E = smooth_modulus(pb)
    u_ref, i_ref = tg.fea_solve_mgcg_matfree(pb, E, tolerance=1e-10, options=tg.SolveOptions(
        coarsening=tg.COARSEN_REFERENCE))
    u_al, i_al = tg.fea_solve_mgcg_matfree(pb, E, tolerance=1e-10, options=tg.SolveOptions(
        coarsening=tg.COARSEN_ALIGNED))
    assert i_ref.used_multigrid and i_al.used_multigrid
    assert rel(u_al, u_ref) < 1e-8
    assert i_al.iterations < i_ref.iterations
    u_mx, i_mx = tg.fea_solve_mgcg_matfree(pb, E, tolerance=1e-10, options=tg.SolveOptions(
        precision=tg.PREC_MIXED))
    assert not i_mx.mixed_fallback
    assert rel(u_mx, u_ref) < 1e-8


@pytest.mark.parametrize("dims", [(48, 24, 24), (37, 19, 13)])
def test_graph_inner_loop_matches_host_loop(tg, dims):
    """The mixed inner PCG loop run as one CUDA graph (device-side loop
    condition) gives bit-identical results to the host-driven loop."""
    pb = tg.Problem.cantilever(*dims)
    E = smooth_modulus(pb)
    ug, ig = tg.fea_solve_mgcg_matfree(pb, E, tolerance=1e-10, options=tg.SolveOptions(
        precision=tg.PREC_MIXED, graph_mode=tg.GRAPH_ON))
    uh, ih = tg.fea_solve_mgcg_matfree(pb, E, tolerance=1e-10, options=tg.SolveOptions(
        precision=tg.PREC_MIXED, graph_mode=tg.GRAPH_OFF))
    assert np.array_equal(ug, uh)
    assert ig.iterations == ih.iterations and ig.matvecs_lowp == ih.matvecs_lowp
    assert ig.refinements == ih.refinements


@pytest.mark.parametrize("prec", [0, 1])
def test_cant60_fifty_iterations(tg, golden, prec):
    """The reference's CPU-runnable configuration end to end: 60x20x20
    cantilever, volume fraction 0.3, rmin 1.5, move 0.2, 50 design iterations,
    solves at 1e-10 -- against the reference's own 50-iteration run."""
    o = cantilever(60, 20, 20)
    pb = tg.Problem(60, 20, 20, 1.0, None, list(zip(o.bc_node, o.bc_comp, o.bc_val)),
                    list(zip(o.ld_node, o.ld_comp, o.ld_val)))
    s = tg.simp_optimize(pb, tg.SimpParams(), tg.SimpOptions(
        volume_fraction=0.3, filter_radius=1.5, move=0.2, change_tol=0.0, max_iterations=50,
        cg_tolerance=1e-10, solve=tg.SolveOptions(precision=prec)))
    hc = np.array([h["compliance"] for h in s["history"]])
    assert s["iterations"] == 50
    assert abs(hc[0] - golden["cant60_hist_c"][0]) <= 1e-9 * hc[0]
    assert rel(hc, golden["cant60_hist_c"]) < 1e-6
    assert rel(s["design"], golden["cant60_design"]) < 1e-4
    assert abs(s["compliance"] - float(golden["cant60_compliance"])) <= 1e-6 * s["compliance"]


def test_double_float_operator_matches_fp64(tg, golden):
    """The double-float (FP32-pair) evaluation of the FP64 operator, the mixed
    form's refinement residual: within 1e-13 of the FP64 operator relative to
    its largest entry, on the reference's golden graded case and a random one."""
    pb, _ = _pb(tg, golden)
    y = tg.fea_matfree_apply(pb, golden["apply_u"], youngs_per_voxel=golden["apply_factor"],
                             precision=2)
    assert rel(y, golden["apply_y_graded"]) < 1e-13
    rng = np.random.default_rng(11)
    nx, ny, nz = 70, 33, 20
    pb2 = tg.Problem(nx, ny, nz)
    f = np.clip(rng.random(pb2.nv), 1e-3, 1.0) ** 3
    u = rng.standard_normal(pb2.ndof)
    y64 = tg.fea_matfree_apply(pb2, u, youngs_per_voxel=f)
    ydf = tg.fea_matfree_apply(pb2, u, youngs_per_voxel=f, precision=2)
    assert rel(ydf, y64) < 1e-13


@pytest.mark.parametrize("residual", [0, 1])
def test_mixed_solve_residual_forms_agree(tg, residual):
    """The mixed solve with the double-float and the FP64 refinement residual:
    both converge to the FP64 solve's solution at the tolerance."""
    nx, ny, nz = 48, 24, 24
    o = cantilever(nx, ny, nz)
    pb = tg.Problem(nx, ny, nz, 1.0, None, list(zip(o.bc_node, o.bc_comp, o.bc_val)),
                    list(zip(o.ld_node, o.ld_comp, o.ld_val)))
    E = smooth_modulus(pb)
    u64, _ = tg.fea_solve_mgcg_matfree(pb, E, tolerance=1e-10)
    um, info = tg.fea_solve_mgcg_matfree(pb, E, tolerance=1e-10, options=tg.SolveOptions(
        precision=tg.PREC_MIXED, mixed_residual=residual))
    assert info.converged and info.residual <= 1e-10
    assert rel(um, u64) < 1e-8


def test_mixed_coarse_smoothers_agree(tg):
    """The FP32 V-cycle's coarse smoother (damped Jacobi or the Chebyshev
    polynomial) changes the preconditioner, not the answer: both mixed runs track
    the FP64 run's compliance history within 1e-6.  On a seeded high-contrast
    design (a thin beam at 1, the box at the density floor, stiffness contrast
    ~1e-8) Chebyshev needs no more inner iterations than Jacobi.  Bad values are
    rejected."""
    from oracle.oracle import beam_seed
    nx, ny, nz = 96, 48, 48
    o = cantilever(nx, ny, nz)
    pb = tg.Problem(nx, ny, nz, 1.0, None, list(zip(o.bc_node, o.bc_comp, o.bc_val)),
                    list(zip(o.ld_node, o.ld_comp, o.ld_val)))
    base = dict(volume_fraction=0.05, filter_radius=1.5, change_tol=0.0, max_iterations=8,
                cg_tolerance=1e-9, initial_design=beam_seed(nx, ny, nz, half_width=3))
    ref = tg.simp_optimize(pb, tg.SimpParams(), tg.SimpOptions(**base))
    hc64 = np.array([h["compliance"] for h in ref["history"]])
    cg = {}
    for sm in (tg.SMOOTHER_JACOBI, tg.SMOOTHER_CHEBYSHEV):
        s = tg.simp_optimize(pb, tg.SimpParams(), tg.SimpOptions(
            solve=tg.SolveOptions(precision=tg.PREC_MIXED, coarse_smoother=sm), **base))
        hc = np.array([h["compliance"] for h in s["history"]])
        assert rel(hc, hc64) < 1e-6
        assert abs(s["compliance"] - ref["compliance"]) <= 1e-8 * ref["compliance"]
        cg[sm] = sum(h["cg_iterations"] for h in s["history"])
    assert cg[tg.SMOOTHER_CHEBYSHEV] <= cg[tg.SMOOTHER_JACOBI]
    # lambda_max of the Chebyshev interval comes from a power iteration: on a
    # smooth SIMP field neither smoother may make the FP32 preconditioner
    # indefinite (an inner breakdown) or hand the solve to FP64.
    E = smooth_modulus(pb)
    u64, _ = tg.fea_solve_mgcg_matfree(pb, E, tolerance=1e-10)
    for sm in (tg.SMOOTHER_JACOBI, tg.SMOOTHER_CHEBYSHEV):
        um, info = tg.fea_solve_mgcg_matfree(pb, E, tolerance=1e-10, options=tg.SolveOptions(
            precision=tg.PREC_MIXED, coarse_smoother=sm))
        assert info.converged and not info.mixed_fallback and info.inner_breakdowns == 0, info
        assert rel(um, u64) < 1e-8
    with pytest.raises(ValueError, match="coarse_smoother"):
        tg.simp_optimize(pb, tg.SimpParams(), tg.SimpOptions(
            solve=tg.SolveOptions(precision=tg.PREC_MIXED, coarse_smoother=7), **base))
