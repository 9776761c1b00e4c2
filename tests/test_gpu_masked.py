"""The masked simp_optimize overload (passive regions) on the CUDA path, through
the C ABI: effective_design_mask and the mask-aware filter against the
reference's golden vectors (bit-exact), oc_update_masked against the oracle
(bit-exact), and the masked trajectory against the reference's golden run
(solver-level tolerances as in test_gpu_parity).  GPU only."""
import numpy as np
import pytest

from oracle.oracle import cantilever

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _masked(tg, golden):
    mx, my, mz = (int(v) for v in golden["mask_dims"])
    o = cantilever(mx, my, mz, solid=golden["mask_tags"])
    pb = tg.Problem(mx, my, mz, 1.0, golden["mask_tags"], list(zip(o.bc_node, o.bc_comp, o.bc_val)),
                    list(zip(o.ld_node, o.ld_comp, o.ld_val)))
    return pb, o, golden["mask_mask"]


def test_effective_mask_and_masked_filter(tg, golden):
    pb, _, mask = _masked(tg, golden)
    assert np.array_equal(tg.effective_design_mask(pb, mask), golden["mask_eff"])
    f = tg.make_density_filter(pb, 1.5, mask)
    assert np.array_equal(f.filter_density(golden["mask_x"]), golden["mask_filt_fwd"])
    assert np.array_equal(f.filter_sensitivity(golden["mask_x"]), golden["mask_filt_adj"])


def test_mask_rejects_bad_values(tg, golden):
    pb, _, mask = _masked(tg, golden)
    bad = mask.copy()
    bad[3] = 7
    with pytest.raises(ValueError, match="mask values"):
        tg.effective_design_mask(pb, bad)


@pytest.mark.parametrize("dims", [(14, 6, 5), (40, 20, 20)])
def test_oc_update_masked_bit_exact(tg, port, golden, dims):
    rng = np.random.default_rng(sum(dims))
    nx, ny, nz = dims
    tags = np.ones(nx * ny * nz, np.uint8)
    tags[rng.random(tags.size) < 0.05] = 0
    tags[rng.random(tags.size) < 0.03] = 4
    mask = np.zeros(tags.size, np.uint8)
    r = rng.random(tags.size)
    mask[r < 0.1] = 1
    mask[(r >= 0.1) & (r < 0.2)] = 2
    o = cantilever(nx, ny, nz, solid=tags)
    pb = tg.Problem(nx, ny, nz, 1.0, tags)
    eff = port.effective_design_mask(o, mask)
    x = np.where(eff == 0, rng.random(tags.size) * 0.8 + 0.1, np.where(eff == 1, 1.0, 0.0))
    dc = -rng.random(tags.size) * 5.0
    for vf, radius, move in ((0.3, 1.5, 0.2), (0.45, 2.5, 0.1)):
        got = tg.oc_update_masked(pb, radius, mask, x, dc, vf, move, 1e-3)
        want = port.oc_update_masked(o, mask, x, dc, vf, radius, move, 1e-3)
        assert np.array_equal(got, want)
        assert np.all(got[eff == 1] == 1.0) and np.all(got[eff == 2] == 0.0)


@pytest.mark.parametrize("prec", [0, 1])
def test_masked_simp_trajectory(tg, golden, prec):
    pb, _, mask = _masked(tg, golden)
    opt = tg.SimpOptions(volume_fraction=0.35, max_iterations=15, cg_tolerance=1e-10,
                         solve=tg.SolveOptions(precision=prec))
    s = tg.simp_optimize(pb, tg.SimpParams(), opt, mask=mask)
    hc = np.array([h["compliance"] for h in s["history"]])
    n = int(golden["msimp_iterations"])
    assert s["iterations"] == n
    assert abs(hc[0] - golden["msimp_hist_c"][0]) <= 1e-9 * hc[0]
    assert rel(hc, golden["msimp_hist_c"]) < 1e-6
    assert rel(s["design"], golden["msimp_design"]) < 1e-5
    assert rel(s["physical_density"], golden["msimp_phys"]) < 1e-5
    assert abs(s["compliance"] - float(golden["msimp_compliance"])) <= 1e-6 * s["compliance"]
    assert abs(s["volume_fraction"] - float(golden["msimp_volume_fraction"])) <= 1e-6
    eff = golden["mask_eff"]
    assert np.all(s["physical_density"][eff == 1] == 1.0)
    assert np.all(s["physical_density"][eff == 2] == 0.0)
    assert np.all(s["design"][eff == 1] == 1.0) and np.all(s["design"][eff == 2] == 0.0)


def test_masked_job_matches_one_shot(tg, golden):
    """The resident masked job reproduces simp_optimize_masked step by step."""
    pb, _, mask = _masked(tg, golden)
    opt = tg.SimpOptions(volume_fraction=0.35, max_iterations=4, cg_tolerance=1e-10,
                         change_tol=0.0)
    s = tg.simp_optimize(pb, tg.SimpParams(), opt, mask=mask)
    job = tg.SimpJob(pb, tg.SimpParams(), opt, mask=mask)
    rows = [job.step() for _ in range(4)]
    x, xp = job.read()
    job.close()
    assert [r["compliance"] for r in rows] == [h["compliance"] for h in s["history"]]
    assert np.array_equal(x, s["design"])
