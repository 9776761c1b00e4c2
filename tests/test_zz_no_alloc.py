"""The allocation-free density filter, tg_filter_noalloc, against tg_filter.

Callers that cannot allocate device memory at the point where they filter (an
allocator-free serving loop, a host whose device memory belongs to another
runtime's arena) pass their own device buffers to tg_filter_noalloc, which keeps
its scratch in a fixed device array of the library.  Its results must equal the
allocating entry point's bit for bit (the filter is bit-exact to the reference),
call after call, with no state carried from one call to the next.  Collected
last so a stop-at-first-failure run has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _entry(tg):
    f = tg.lib().tg_filter_noalloc
    f.argtypes = [ctypes.c_int32] * 3 + [ctypes.c_void_p, ctypes.c_double, ctypes.c_int32,
                                         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def _call(tg, pb, tags_dev, radius, adjoint, xd, od):
    """One call on caller-owned device tensors; raises ValueError on a non-zero status."""
    import torch
    rc = _entry(tg)(pb.nx, pb.ny, pb.nz, None if tags_dev is None else tags_dev.data_ptr(),
                    radius, adjoint, xd.data_ptr(), od.data_ptr(), None)
    torch.cuda.synchronize()
    if rc != 0:
        raise ValueError(tg.lib().tg_last_error().decode())


def _noalloc(tg, pb, tags_dev, radius, adjoint, x):
    import torch
    xd = torch.tensor(x, dtype=torch.float64, device="cuda")
    od = torch.full_like(xd, float("nan"))
    _call(tg, pb, tags_dev, radius, adjoint, xd, od)
    return od.cpu().numpy()


def test_noalloc_filter_matches_allocating_filter_twice(tg):
    import torch
    rng = np.random.default_rng(17)
    nx, ny, nz = 40, 24, 18
    tags = (rng.random(nx * ny * nz) > 0.1).astype(np.uint8)
    pb = tg.Problem(nx, ny, nz, 1.0, tags)
    tags_dev = torch.tensor(tags, dtype=torch.uint8, device="cuda")
    for call, (radius, adjoint) in enumerate([(1.5, 0), (2.5, 1)]):
        x = rng.random(pb.nv) * tags
        ref = tg.make_density_filter(pb, radius)
        want = ref.filter_sensitivity(x) if adjoint else ref.filter_density(x)
        got = _noalloc(tg, pb, tags_dev, radius, adjoint, x)
        assert np.array_equal(got, want), f"call {call}"
    # A second round on an all-solid grid (NULL tags) after the voided one.
    pb2 = tg.Problem(nx, ny, nz)
    x = rng.random(pb2.nv)
    want = tg.make_density_filter(pb2, 1.5).filter_density(x)
    assert np.array_equal(_noalloc(tg, pb2, None, 1.5, 0, x), want)


def test_noalloc_filter_rejects_sizes_beyond_its_scratch(tg):
    pb = tg.Problem(128, 128, 65)  # 1,064,960 voxels > 1,048,576
    with pytest.raises(ValueError, match="1,048,576"):
        _noalloc(tg, pb, None, 1.5, 0, np.zeros(pb.nv))


def test_noalloc_filter_allocates_nothing(tg):
    """After one warm-up call, further calls leave the device's free memory
    unchanged: the scratch is the library's fixed array, nothing else."""
    import torch
    rng = np.random.default_rng(3)
    nx, ny, nz = 64, 48, 40
    pb = tg.Problem(nx, ny, nz)
    xd = torch.tensor(rng.random(pb.nv), dtype=torch.float64, device="cuda")
    od = torch.empty_like(xd)
    _call(tg, pb, None, 2.5, 0, xd, od)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for radius, adjoint in [(1.5, 0), (2.5, 1), (6.0, 0), (1.2, 1)]:
        _call(tg, pb, None, radius, adjoint, xd, od)
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_filter_adjoint_without_tags(tg):
    rng = np.random.default_rng(5)
    pb = tg.Problem(30, 20, 12)
    x = rng.random(pb.nv)
    want = tg.make_density_filter(pb, 2.5).filter_sensitivity(x)
    assert np.array_equal(_noalloc(tg, pb, None, 2.5, 1, x), want)


def test_noalloc_filter_rejects_radius_beyond_its_stencil(tg):
    pb = tg.Problem(16, 8, 8)
    with pytest.raises(ValueError, match="radius above 6"):
        _noalloc(tg, pb, None, 6.5, 0, np.zeros(pb.nv))
