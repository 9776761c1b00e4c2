"""The active domain on the GPU (SimpOptions::active_domain_band; simp.cpp:449-556,
:1745-1896) against the reference's own values (the golden file).  GPU only.

Tolerances.  The mask, its count, the escape count and the auto band are
integer work: identical.  The armed runs are held to the reference's postures
exactly -- the band, the per-iteration active fraction, whether, when and why
the mask latched off, the escape count -- and their trajectories to the solve's
tolerance: compliances within 1e-6 relative, the physical density within 1e-4.
"""
import numpy as np
import pytest

from oracle.oracle import ACTIVE_DOMAIN_RUNS, Problem, active_domain_case

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _tg_problem(tg, o):
    return tg.Problem(o.nx, o.ny, o.nz, o.h, o.solid, list(zip(o.bc_node, o.bc_comp, o.bc_val)),
                      list(zip(o.ld_node, o.ld_comp, o.ld_val)))


def test_active_domain_mask_matches_reference(tg, golden):
    nx, ny, nz = (int(v) for v in golden["ad_dims"])
    pb = tg.Problem(nx, ny, nz, 1.0, golden["ad_tags"])
    rho = golden["ad_rho"]
    for b, want in zip(golden["ad_bands"], golden["ad_masks"]):
        got, n = tg.active_domain_mask(pb, rho, 1e-3, int(b))
        assert np.array_equal(got, want), b
        assert n == int(want.sum())
    assert tg.active_domain_escape_count(pb, rho, golden["ad_prev"], 1e-3) == \
        int(golden["ad_escapes"])
    assert tg.active_domain_escape_count(pb, rho, None, 1e-3) == 0
    assert [tg.active_domain_auto_band(float(r)) for r in golden["ad_radii"]] == \
        golden["ad_auto"].tolist()


def test_active_domain_mask_large_grid(tg, port):
    """A grid with more voxels than one launch wave and a band past the shortest
    axis: the device mask equals the oracle's."""
    rng = np.random.default_rng(7)
    nx, ny, nz = 150, 37, 9
    tags = rng.choice(np.array([0, 1, 1, 1, 1, 4, 5], np.uint8), nx * ny * nz)
    rho = np.where(rng.random(tags.size) < 0.01, rng.random(tags.size), 1e-3)
    pb, o = tg.Problem(nx, ny, nz, 1.0, tags), Problem(nx, ny, nz, 1.0, tags)
    for band in (1, 4, 12):
        got, n = tg.active_domain_mask(pb, rho, 1e-3, band)
        want = port.active_domain_mask(o, rho, 1e-3, band)
        assert np.array_equal(got, want), band
        assert n == int(want.sum())


def _reason(golden, name):
    # The reference build here routes the matrix-free multigrid to its exact
    # Jacobi-PCG, whose name a failed restricted solve carries; the reference's
    # own build, like this library, names fea_solve_mgcg_matfree.
    r = bytes(golden[f"adr_{name}_reason"]).decode()
    return r.replace("fea_solve_cg_matfree:", "fea_solve_mgcg_matfree:")


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("name", list(ACTIVE_DOMAIN_RUNS))
def test_active_domain_runs_match_reference(tg, golden, name, prec):
    """Restricted trajectory solves (plain, masked, and under the MMA updater), the
    escape latch, a failed restricted solve re-solved on the full domain, and the
    fraction latch."""
    o, mask, seed, band, radius, vf, its, upd = active_domain_case(name)
    s = tg.simp_optimize(_tg_problem(tg, o), tg.SimpParams(), tg.SimpOptions(
        volume_fraction=vf, filter_radius=radius, move=0.2, change_tol=0.0, max_iterations=its,
        cg_tolerance=1e-9, initial_design=seed, active_domain_band=band, updater=upd,
        solve=tg.SolveOptions(precision=prec)), mask=mask)
    k = "adr_" + name
    ad = s["active_domain"]
    assert [s["iterations"], ad["band"], int(ad["latched"]), ad["latch_iteration"],
            ad["escape_count"]] == golden[k + "_i"].tolist()
    af = np.array([h["active_fraction"] for h in s["history"]])
    assert np.array_equal(af, golden[k + "_hist_af"])
    assert ad["fraction_mean"] == pytest.approx(float(golden[k + "_d"][2]), rel=1e-15)
    assert ad["reason"] == _reason(golden, name)
    hc = np.array([h["compliance"] for h in s["history"]])
    assert rel(hc, golden[k + "_hist_c"]) < 1e-6
    assert abs(s["compliance"] - golden[k + "_d"][0]) <= 1e-6 * golden[k + "_d"][0]
    assert rel(s["physical_density"], golden[k + "_phys"]) < 1e-4


def test_active_domain_off_is_unchanged(tg):
    """band 0 (the default) runs exactly the unarmed loop: every fraction 1, no
    record; the same run with the band armed on a compact domain latches at the
    fifth iteration and then matches it step for step."""
    o, _, _, _, radius, vf, its, _ = active_domain_case("latch")
    base = dict(volume_fraction=vf, filter_radius=radius, move=0.2, change_tol=0.0,
                max_iterations=its, cg_tolerance=1e-9)
    off = tg.simp_optimize(_tg_problem(tg, o), tg.SimpParams(), tg.SimpOptions(**base))
    on = tg.simp_optimize(_tg_problem(tg, o), tg.SimpParams(),
                          tg.SimpOptions(active_domain_band=-1, **base))
    assert off["active_domain"]["band"] == 0 and not off["active_domain"]["latched"]
    assert off["active_domain"]["fraction_mean"] == 1.0
    assert all(h["active_fraction"] == 1.0 for h in off["history"])
    assert on["active_domain"]["latched"] and on["active_domain"]["latch_iteration"] == 5
    # Band 3 covers this 12x4x4 box: the restricted system is the full one.
    assert rel(on["physical_density"], off["physical_density"]) < 1e-10
