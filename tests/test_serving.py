"""The serving loop (tg_server_*): admission by HBM budget and free slots,
resident jobs on their own streams, and -- the continuous-batching property --
each job's result is the same alone and in the mix (bit-identical here: every
job owns its buffers and stream and every reduction has a fixed order)."""
import numpy as np
import pytest

from topopt_gb300 import workloads


def test_workload_generators():
    pb, prm, opt = workloads.design(7)
    assert 32 <= pb.nx <= 128 and 16 <= pb.ny <= 64 and 16 <= pb.nz <= 64
    assert pb.nx % 2 == 0 and pb.ny % 2 == 0 and pb.nz % 2 == 0
    assert 0.15 <= opt.volume_fraction <= 0.5 and 1.2 <= opt.filter_radius <= 2.5
    assert pb.nbc > 0 and pb.nloads > 0
    s = workloads.stream(3, rate=4.0, duration=5.0)
    assert len(s) > 5 and all(a < b for (a, *_), (b, *_) in zip(s, s[1:]))
    for _, p, _, _ in s:
        assert 24 ** 3 * 0.5 <= p.nv <= 192 * 96 * 96 * 1.5


def test_server_host_logic(tg):
    """Admission, rejection, tickets and shutdown are host logic and run without
    a device.  Without one, the admitted job ends with the device error (there
    is no CPU fallback); with one, it completes."""
    pb, prm, opt = workloads.design(5, iterations=1, sizes=(16, 8, 8))
    est = tg.job_estimate_bytes(pb, opt)
    srv = tg.Server(hbm_budget_bytes=est, max_active=2)
    with pytest.raises(MemoryError, match="budget"):
        srv.submit(*workloads.design(6, iterations=1, sizes=(32, 16, 16)))
    t = srv.submit(pb, prm, opt)
    try:
        assert srv.wait(t, fields=False)["iterations"] == 1
    except tg.DeviceError:
        pass
    lib = tg.lib()
    assert lib.tg_server_wait(srv._h, t, None, None, None) == 1  # released: TG_EINVAL
    assert b"unknown ticket" in lib.tg_last_error()
    st = srv.stats()
    assert (st["submitted"], st["rejected"], st["admitted"], st["completed"]) == (2, 1, 1, 1)
    assert st["active"] == 0 and st["queued"] == 0 and st["bytes_in_use"] == 0
    assert st["peak_bytes"] == est
    srv.close()
    with pytest.raises(ValueError, match="max_active"):
        tg.Server(hbm_budget_bytes=est, max_active=0)


@pytest.mark.gpu
def test_same_alone_and_in_the_mix(tg):
    jobs = [workloads.design(s, precision=p, iterations=6, sizes=sz)
            for s, p, sz in ((1, 1, (24, 12, 12)), (2, 0, (20, 10, 8)), (3, 1, (32, 16, 16)),
                             (4, 1, (16, 8, 8)))]
    alone = [tg.simp_optimize(pb, prm, opt) for pb, prm, opt in jobs]
    srv = tg.Server(hbm_budget_bytes=64 << 30, max_active=4)
    tickets = [srv.submit(pb, prm, opt) for pb, prm, opt in jobs]
    mixed = [srv.wait(t) for t in tickets]
    st = srv.stats()
    srv.close()
    assert st["completed"] == 4 and st["peak_active"] >= 2
    for a, m in zip(alone, mixed):
        assert m["iterations"] == a["iterations"]
        assert m["compliance"] == a["compliance"]
        assert np.array_equal(m["design"], a["design"])
        assert np.array_equal(m["physical_density"], a["physical_density"])


@pytest.mark.gpu
def test_budget_admission(tg):
    jobs = [workloads.design(s, iterations=2, sizes=(24, 12, 12)) for s in range(4)]
    est = max(tg.job_estimate_bytes(pb, opt) for pb, _, opt in jobs)
    srv = tg.Server(hbm_budget_bytes=int(est * 1.5), max_active=4)
    tickets = [srv.submit(pb, prm, opt) for pb, prm, opt in jobs]
    res = [srv.wait(t, fields=False) for t in tickets]
    st = srv.stats()
    assert st["peak_active"] == 1 and st["peak_bytes"] <= int(est * 1.5)
    assert all(r["iterations"] == 2 for r in res)
    big = workloads.design(9, sizes=(64, 32, 32))
    with pytest.raises(MemoryError, match="budget"):
        srv.submit(*big)
    srv.close()


@pytest.mark.gpu
def test_estimate_bounds_device_bytes(tg):
    for sz in ((24, 12, 12), (64, 32, 32), (96, 48, 48)):
        for prec in (0, 1):
            pb, prm, opt = workloads.design(5, precision=prec, iterations=1, sizes=sz)
            job = tg.SimpJob(pb, prm, opt)
            job.step()
            used = job.device_bytes
            job.close()
            assert used <= tg.job_estimate_bytes(pb, opt), (sz, prec)
