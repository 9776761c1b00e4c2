"""Stress recovery, the fixed-design analysis, warm starts and the
minimize_plastic ladder walk on the GPU, against the reference's own values (the
golden file) and the oracle.  GPU only.

Tolerances.  The element stress kernel rounds exactly like hex8_stress, so for
the same displacement it is bit-identical.  Everything downstream of a solve
carries the solve's tolerance: the analysis's compliance within 1e-9 relative,
stresses and margins within 1e-6, ladder trajectories within 1e-6 with every
verdict (trajectory, analysis, acceptance, load path, recommendation, stop)
identical.
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


def test_element_stress_bit_exact(tg, golden, port):
    """One element: the reference's hex8_stress values at the centre; a graded
    grid: the oracle's per-element stress, bit for bit."""
    for q in range(4):  # the centre cases
        E, nu, h = golden["stress_mat"][q]
        ue = golden["stress_ue"][q]
        u = np.zeros(24)
        for a in range(8):
            ox, oy, oz = (a ^ (a >> 1)) & 1, (a >> 1) & 1, a >> 2
            u[3 * (oz * 4 + oy * 2 + ox):3 * (oz * 4 + oy * 2 + ox) + 3] = ue[3 * a:3 * a + 3]
        sig, vm = tg.element_stress(tg.Problem(1, 1, 1, h), E, nu, u)
        assert np.array_equal(sig[0], golden["stress_sigma"][q])
        assert vm[0] == golden["stress_vm"][q]
    rng = np.random.default_rng(4)
    nx, ny, nz, h = 9, 7, 5, 0.7
    tags = (rng.random(nx * ny * nz) > 0.2).astype(np.uint8)
    rho = rng.random(nx * ny * nz)
    u = rng.standard_normal(3 * (nx + 1) * (ny + 1) * (nz + 1))
    sig, vm = tg.element_stress(tg.Problem(nx, ny, nz, h, tags), 2.0, 0.3, u, rho, 0.5)
    for e in range(nx * ny * nz):
        i, j, k = e % nx, (e // nx) % ny, e // (nx * ny)
        if not (tags[e] and rho[e] > 0.5):
            assert vm[e] == 0.0 and not sig[e].any()
            continue
        ue = []
        for a in range(8):
            ox, oy, oz = (a ^ (a >> 1)) & 1, (a >> 1) & 1, a >> 2
            n = ((k + oz) * (ny + 1) + j + oy) * (nx + 1) + i + ox
            ue += list(u[3 * n:3 * n + 3])
        s_want, vm_want = port.hex8_stress(2.0, 0.3, h, np.array(ue))
        assert np.array_equal(sig[e], s_want) and vm[e] == vm_want


def _ladder_problem(tg, golden):
    nx, ny, nz = (int(v) for v in golden["lad_dims"])
    tags = golden["lad_tags"]
    return _tg_problem(tg, cantilever(nx, ny, nz, solid=tags), tags)


@pytest.mark.parametrize("prec", [0, 1])
def test_analysis_matches_reference(tg, golden, prec):
    pb = _ladder_problem(tg, golden)
    a = tg.analyze_fixed_design(pb, tg.SimpParams(), golden["ana_density"],
                                tg.StrengthSpec(yield_strength=30.0, margin_stop=25.0,
                                                build_dir=(0.3, -0.2, 0.9)),
                                cg_tolerance=1e-10, solve=tg.SolveOptions(precision=prec),
                                fields=True)
    d = golden["ana_d"]
    assert [a["printed_voxels"], a["load_path_ok"], a["accepted"]] == golden["ana_i"].tolist()
    assert a["non_convergent"] == 0
    assert abs(a["compliance"] - d[0]) <= 1e-9 * d[0]
    got = np.array([a["max_von_mises"], a["max_interlayer_tension"], a["margin_in_plane"],
                    a["margin_interlayer"], a["margin_worst_case"]])
    assert np.all(np.abs(got - d[1:]) <= 1e-6 * np.abs(d[1:]))
    assert rel(a["von_mises"], golden["ana_vm"]) < 1e-6


def test_analysis_gate_and_errors(tg, golden):
    pb = _ladder_problem(tg, golden)
    rho = golden["ana_density"].reshape(8, 6, 20).copy()
    rho[:, :, 10] = 0.0  # severed: the belt rejects whatever the margin
    a = tg.analyze_fixed_design(pb, tg.SimpParams(), rho.ravel(),
                                tg.StrengthSpec(yield_strength=30.0, margin_stop=0.0),
                                cg_tolerance=1e-8)
    assert a["load_path_ok"] == 0 and a["accepted"] == 0
    with pytest.raises(ValueError, match="printed_iso"):
        tg.analyze_fixed_design(pb, tg.SimpParams(), golden["ana_density"],
                                tg.StrengthSpec(printed_iso=1.0))
    with pytest.raises(ValueError, match="build_dir"):
        tg.analyze_fixed_design(pb, tg.SimpParams(), golden["ana_density"],
                                tg.StrengthSpec(build_dir=(0.0, 0.0, 0.0)))


@pytest.mark.parametrize("masked", [False, True])
def test_warm_start_matches_oracle(tg, port, golden, masked):
    """SimpOptions::initial_design (warm_start_design, simp.cpp:324-344):
    a seeded run tracks the oracle's seeded run."""
    import ctypes as C
    from oracle.oracle import _OrSimpOptions, _OrSimpResult
    nx, ny, nz = (int(v) for v in golden["lad_dims"])
    tags = golden["lad_tags"]
    o = cantilever(nx, ny, nz, solid=tags)
    seed = golden["lada_phys"] * 1.7 + 0.05
    mask = np.zeros(o.nv, np.uint8)
    if masked:
        mask[np.random.default_rng(1).random(o.nv) < 0.1] = tg.MASK_FROZEN_VOID
    n = 12
    hc, hch, hvf = np.zeros(n), np.zeros(n), np.zeros(n)
    hcg = np.zeros(n, np.int32)
    design, phys = np.zeros(o.nv), np.zeros(o.nv)
    opt = _OrSimpOptions(0.3, 1.5, 0.2, 0.0, 1e-9, n, 0, 0, None, None, None, 0.5,
                         seed.ctypes.data_as(C.c_void_p))
    res = _OrSimpResult()
    port._check(port.lib.or_simp_optimize_masked(
        o.nx, o.ny, o.nz, o.h, port._ptr(tags), mask, 1.0, 0.3, 3.0, 1e-3, *o.bc_args(),
        C.byref(opt), hc, hch, hvf, hcg, design, phys, C.byref(res)))
    s = tg.simp_optimize(_tg_problem(tg, o, tags), tg.SimpParams(), tg.SimpOptions(
        volume_fraction=0.3, filter_radius=1.5, move=0.2, change_tol=0.0, max_iterations=n,
        cg_tolerance=1e-9, initial_design=seed), mask=mask)
    got = np.array([h["compliance"] for h in s["history"]])
    assert rel(got, hc) < 1e-6
    assert rel(s["design"], design) < 1e-5


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("tag,margin_stop", [("a", 1.0), ("b", 25.0)])
def test_ladder_matches_reference(tg, golden, tag, margin_stop, prec):
    """The ladder walk with warm-start inheritance: (a) every rung accepted but
    the severed last one, which does not stop the walk; (b) the margin stop."""
    pb = _ladder_problem(tg, golden)
    L = tg.minimize_plastic(
        pb, tg.SimpParams(),
        tg.SimpOptions(filter_radius=1.5, move=0.2, change_tol=0.01, max_iterations=25,
                       cg_tolerance=1e-9, solve=tg.SolveOptions(precision=prec)),
        golden["lad_ladder"], tg.StrengthSpec(yield_strength=30.0, margin_stop=margin_stop))
    assert [L["evaluated"], L["recommended"], L["stopped_on_margin"]] == \
        golden[f"lad{tag}_out"].tolist()
    rd, ri = golden[f"lad{tag}_rung_d"], golden[f"lad{tag}_rung_i"]
    for r, g in enumerate(L["rungs"]):
        a = g["analysis"]
        assert [g["optimization"]["iterations"], g["trajectory_ok"], g["analysed"],
                g["accepted"], a["load_path_ok"]] == ri[r].tolist()
        assert g["volume_fraction"] == rd[r][0]
        assert abs(g["optimization"]["compliance"] - rd[r][1]) <= 1e-6 * rd[r][1]
        assert abs(a["max_von_mises"] - rd[r][2]) <= 1e-5 * rd[r][2]
        assert abs(a["margin_worst_case"] - rd[r][4]) <= 1e-5 * rd[r][4]
    rec = L["recommended"]
    assert rec >= 0
    assert rel(L["physical_density"], golden[f"lad{tag}_phys"]) < 1e-4


def test_ladder_outputs_round_trip(tg, golden, tmp_path):
    """The ladder's recommended design through design.bin and fields.bin: the
    stored field re-certifies to the recorded margin bit for bit (the
    reproduction check of the reference's re-lattice path), and the fields
    container carries the analysis's von Mises and printed-node displacement."""
    pb = _ladder_problem(tg, golden)
    strength = tg.StrengthSpec(yield_strength=30.0, margin_stop=25.0)
    L = tg.minimize_plastic(
        pb, tg.SimpParams(), tg.SimpOptions(filter_radius=1.5, max_iterations=25,
                                            cg_tolerance=1e-9), golden["lad_ladder"], strength)
    rec = L["rungs"][L["recommended"]]
    a = tg.analyze_fixed_design(pb, tg.SimpParams(), L["physical_density"], strength,
                                cg_tolerance=1e-9, fields=True)
    assert a["margin_worst_case"] == rec["analysis"]["margin_worst_case"]
    dims = (pb.nx, pb.ny, pb.nz)
    tg.write_design_file(tmp_path / "design.bin", dims, [dict(
        requested_volume_fraction=rec["volume_fraction"],
        achieved_volume_fraction=rec["optimization"]["volume_fraction"],
        margin_worst_case=rec["analysis"]["margin_worst_case"],
        margin_effective=rec["analysis"]["margin_effective"],
        max_von_mises=rec["analysis"]["max_von_mises"], accepted=1,
        iterations=rec["optimization"]["iterations"], density=L["physical_density"])])
    back = tg.read_design_file(tmp_path / "design.bin")["variants"][0]
    again = tg.analyze_fixed_design(pb, tg.SimpParams(), back["density"], strength,
                                    cg_tolerance=1e-9)
    assert again["margin_worst_case"] == back["margin_worst_case"]
    tg.write_fields_file(tmp_path / "fields.bin", dims, [dict(
        requested_volume_fraction=rec["volume_fraction"], von_mises=a["von_mises"],
        displacement=a["displacement"])])
    raw = (tmp_path / "fields.bin").read_bytes()
    nv, nd = pb.nv, pb.ndof
    hdr = 1 + 3 + 12 + 24 + 8 + 8 + 8
    vm32 = np.frombuffer(raw, np.float32, nv, hdr + 8 + 8 + 8 + 24)
    assert np.array_equal(vm32, a["von_mises"].astype(np.float32))
    d32 = np.frombuffer(raw, np.float32, nd, hdr + 8 + 8 + 8 + 24 + 4 * nv)
    assert np.array_equal(d32, a["displacement"].astype(np.float32))
    assert np.any(a["displacement"] != 0.0) and np.any(a["displacement"] == 0.0)
