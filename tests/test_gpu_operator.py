"""Schedules of the FP32 fine operator: the pencil kernel and the column-blocked
kernel in each tile shape and z-chunk length give Ke u to FP32 rounding (within
2e-6 of the FP64 result, relative to its largest entry) on brick edges, partial
tiles, voids and the 256x128x128 benchmark grid.  GPU only."""
import numpy as np
import pytest

from oracle.oracle import cantilever

pytestmark = pytest.mark.gpu

SCHEDULES = [(0, 0, 32)] + [(1, s, kz) for s in range(8) for kz in (8, 13, 32)]


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.fixture
def schedule(tg):
    yield tg.set_fp32_schedule
    tg.set_fp32_schedule(None)


@pytest.mark.parametrize("dims", [(1, 1, 1), (2, 1, 3), (33, 17, 9), (61, 20, 11), (40, 24, 9)])
def test_fp32_schedules_match_oracle(tg, port, schedule, dims):
    rng = np.random.default_rng(sum(dims) + 1)
    nx, ny, nz = dims
    solid = (rng.random(nx * ny * nz) > 0.1).astype(np.uint8)
    o = cantilever(nx, ny, nz, solid=solid)
    pb = tg.Problem(nx, ny, nz, 1.0, solid)
    u = rng.standard_normal(o.ndof)
    f = rng.random(o.nv) + 1e-3
    ref = port.apply(o, u, f)
    for kind, shape, kz in SCHEDULES:
        schedule(kind, shape, kz)
        y = tg.fea_matfree_apply(pb, u, youngs_per_voxel=f, precision=tg.PREC_MIXED)
        assert rel(y, ref) < 2e-6, (kind, shape, kz)


def test_fp32_schedules_at_scale(tg, schedule):
    """256x128x128: every schedule agrees with the FP64 operator to FP32
    rounding."""
    nx, ny, nz = 256, 128, 128
    assert tg.fp32_schedule(nx, ny, nz)[0] in (tg.SCHED_PENCIL, tg.SCHED_COLUMN)
    pb = tg.Problem(nx, ny, nz)
    rng = np.random.default_rng(7)
    f = rng.random(pb.nv) * 0.999 + 0.001
    u = rng.standard_normal(pb.ndof)
    y64 = tg.fea_matfree_apply(pb, u, youngs_per_voxel=f)
    for kind, shape, kz in [(0, 0, 32), (1, 0, 26), (1, 1, 26), (1, 2, 13), (1, 3, 32),
                            (1, 4, 26), (1, 6, 33), (1, 7, 16)]:
        schedule(kind, shape, kz)
        y = tg.fea_matfree_apply(pb, u, youngs_per_voxel=f, precision=tg.PREC_MIXED)
        assert rel(y, y64) < 2e-6, (kind, shape, kz)


def test_mixed_solve_same_answer_every_schedule(tg, schedule):
    """The mixed solve (FP32 operator in the V-cycle, the smoother and the inner
    Krylov apply) reaches the FP64 solution under every schedule."""
    from test_gpu_parity import smooth_modulus
    nx, ny, nz = 48, 24, 24
    o = cantilever(nx, ny, nz)
    pb = tg.Problem(nx, ny, nz, 1.0, None, list(zip(o.bc_node, o.bc_comp, o.bc_val)),
                    list(zip(o.ld_node, o.ld_comp, o.ld_val)))
    E = smooth_modulus(pb)
    u64, _ = tg.fea_solve_mgcg_matfree(pb, E, tolerance=1e-10)
    for kind, shape, kz in [(0, 0, 32), (1, 0, 8), (1, 2, 13), (1, 6, 11)]:
        schedule(kind, shape, kz)
        um, info = tg.fea_solve_mgcg_matfree(pb, E, tolerance=1e-10, options=tg.SolveOptions(
            precision=tg.PREC_MIXED))
        assert info.converged and not info.mixed_fallback, (kind, shape, kz, info)
        assert rel(um, u64) < 1e-8


def test_autotuned_schedule_is_recorded(tg):
    """A mixed job on a grid of >= 2^20 voxels measures the FP32 schedules on
    its first use of those dimensions and records the fastest in the table."""
    nx, ny, nz = 128, 96, 88
    o = cantilever(nx, ny, nz)
    pb = tg.Problem(nx, ny, nz, 1.0, None, list(zip(o.bc_node, o.bc_comp, o.bc_val)),
                    list(zip(o.ld_node, o.ld_comp, o.ld_val)))
    job = tg.SimpJob(pb, tg.SimpParams(), tg.SimpOptions(
        volume_fraction=0.3, filter_radius=1.5, change_tol=0.0, max_iterations=2,
        solve=tg.SolveOptions(precision=tg.PREC_MIXED)))
    kind, shape, kz = tg.fp32_schedule(nx, ny, nz)
    assert kind in (tg.SCHED_PENCIL, tg.SCHED_COLUMN)
    assert kind == tg.SCHED_PENCIL or (0 <= shape < len(tg.FP32_SHAPES) and kz >= 8)
    r = job.step()
    assert r["compliance"] > 0.0
    job.close()


def test_concurrent_jobs_share_one_measured_schedule(tg):
    """Two mixed jobs of one new grid created at the same time: one measures the
    FP32 schedules while the other waits, both then run the published schedule,
    and their results are identical."""
    import threading
    nx, ny, nz = 128, 96, 96
    o = cantilever(nx, ny, nz)
    pb = tg.Problem(nx, ny, nz, 1.0, None, list(zip(o.bc_node, o.bc_comp, o.bc_val)),
                    list(zip(o.ld_node, o.ld_comp, o.ld_val)))
    opts = tg.SimpOptions(volume_fraction=0.3, filter_radius=1.5, change_tol=0.0,
                          max_iterations=2, solve=tg.SolveOptions(precision=tg.PREC_MIXED))
    out, errs = [None, None], []

    def run(i):
        try:
            job = tg.SimpJob(pb, tg.SimpParams(), opts)
            r = job.step()
            x, _ = job.read()
            job.close()
            out[i] = (r["compliance"], x)
        except Exception as e:  # reported below
            errs.append(e)

    ts = [threading.Thread(target=run, args=(i,)) for i in range(2)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errs, errs
    assert out[0][0] == out[1][0]
    assert np.array_equal(out[0][1], out[1][1])
    assert tg.fp32_schedule(nx, ny, nz)[0] in (tg.SCHED_PENCIL, tg.SCHED_COLUMN)
