"""The C-ABI library builds for sm_103a, loads, and exports every entry point
include/topopt_gb300.h declares.  No compute calls: CPU only."""
import ctypes
import os
import re

import pytest

from tests.conftest import ROOT

HEADER = os.path.join(ROOT, "include", "topopt_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(tg_\w+)\s*\(", text, flags=re.M)
    return sorted(set(n for n in names if not n.endswith("_fn")))


def test_header_declares_the_boundary():
    names = declared_functions()
    for n in ("tg_hex8_stiffness", "tg_matfree_apply", "tg_solve", "tg_simp_compliance",
              "tg_filter", "tg_oc_update", "tg_simp_optimize", "tg_job_create", "tg_job_step"):
        assert n in names


def test_library_exports_every_declared_symbol(tg):
    lib = ctypes.CDLL(tg.library_path())
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_errors_without_device_are_reported_not_fallen_back(tg):
    """Argument validation runs before any device work and uses the reference's
    exception classes; hex8_stiffness is host-only and matches the oracle."""
    import numpy as np
    from oracle.oracle import OracleLib
    with pytest.raises(ValueError, match="poisson"):
        tg.hex8_stiffness(1.0, 0.5, 1.0)
    with pytest.raises(ValueError, match="element_size"):
        tg.hex8_stiffness(1.0, 0.3, 0.0)
    ke = tg.hex8_stiffness(1.0, 0.3, 1.0)
    assert np.array_equal(ke, OracleLib("port").hex8_stiffness(1.0, 0.3, 1.0))


def test_page_locked_host_buffers_fail_loudly(tg):
    """tg_host_alloc returns NULL for a non-positive size and, without a device,
    for any size; host_array then raises instead of handing out pageable memory.
    With a device the buffer is a usable float64 array."""
    lib = tg.lib()
    assert not lib.tg_host_alloc(0)
    assert lib.tg_host_free(None) == 0
    try:
        a = tg.host_array(16)
    except MemoryError:
        return
    a[:] = 1.0
    assert a.dtype.name == "float64" and a.sum() == 16.0


def test_python_face_mirrors_reference_names(tg):
    for n in ("hex8_stiffness", "fea_matfree_apply", "fea_solve_mgcg_matfree", "simp_compliance",
              "make_density_filter", "oc_update", "simp_optimize", "SimpJob",
              "SolverNonConvergence"):
        assert hasattr(tg, n)


def test_self_weight_loads_host(tg):
    """self_weight_loads (fea.hpp:215) and its masked form: each solid voxel's
    weight lumped equally to its 8 corners along the unit direction, FrozenVoid
    voxels weightless; host-only (the reference's is built on Eigen, absent
    here, so this is checked by its defining properties)."""
    import numpy as np
    nx, ny, nz, h = 5, 4, 3, 0.5
    rng = np.random.default_rng(2)
    tags = (rng.random(nx * ny * nz) > 0.3).astype(np.uint8)
    pb = tg.Problem(nx, ny, nz, h, tags)
    rho, grav = 1.25, 9.81e-3
    loads = tg.self_weight_loads(pb, rho, grav, (0.0, 0.0, -2.0))
    assert all(c == 2 for _, c, _ in loads)
    nodes = [n for n, _, _ in loads]
    assert nodes == sorted(nodes) and len(set(nodes)) == len(nodes)
    total = sum(v for _, _, v in loads)
    assert abs(total + grav * rho * h ** 3 * tags.sum()) <= 1e-12 * grav * rho * tags.sum()
    per = grav * rho * (h * h * h) / 8.0
    f = np.zeros((nz + 1) * (ny + 1) * (nx + 1))
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                if tags[(k * ny + j) * nx + i]:
                    for dk in (0, 1):
                        for dj in (0, 1):
                            for di in (0, 1):
                                f[((k + dk) * (ny + 1) + j + dj) * (nx + 1) + i + di] += 1
    for n, _, v in loads:
        assert abs(v + per * f[n]) <= 1e-15 * per * 8
    mask = np.where(rng.random(tags.size) < 0.2, tg.MASK_FROZEN_VOID, 0).astype(np.uint8)
    masked = tg.self_weight_loads(pb, rho, grav, (0.0, 0.0, -1.0), mask=mask)
    tot_m = sum(v for _, _, v in masked)
    live = int(((tags > 0) & (mask != tg.MASK_FROZEN_VOID)).sum())
    assert abs(tot_m + grav * rho * h ** 3 * live) <= 1e-12 * grav * rho * live
    tilted = tg.self_weight_loads(pb, rho, grav, (1.0, 1.0, 0.0))
    assert {c for _, c, _ in tilted} == {0, 1}
    with pytest.raises(ValueError, match="direction"):
        tg.self_weight_loads(pb, rho, grav, (0.0, 0.0, 0.0))
    with pytest.raises(ValueError, match="density"):
        tg.self_weight_loads(pb, -1.0, grav)


def test_load_path_host_matches_oracle(tg, port):
    """load_path_connected on random tagged designs: the library's host walk
    agrees with the oracle's (itself pinned to the reference)."""
    import numpy as np
    from oracle.oracle import cantilever
    rng = np.random.default_rng(9)
    nx, ny, nz = 12, 5, 6
    tags = np.ones((nz, ny, nx), np.uint8)
    tags[:, :, 0] = 5
    tags[2:4, :, nx - 1] = 4
    tags[rng.random(tags.shape) < 0.05] = 0
    tags[:, :, 0] = 5
    tags = tags.ravel()
    o = cantilever(nx, ny, nz, solid=tags)
    pb = tg.Problem(nx, ny, nz, 1.0, tags)
    seen = set()
    for t in range(40):
        d = rng.random(tags.size) * (0.5 + 0.02 * t)
        d[tags == 4] = 1.0  # an unprinted Load voxel is never reached
        if t % 3 == 0:
            d[tags == 5] = 1.0
        want = port.load_path_connected(o, d)
        assert tg.load_path_connected(pb, d) == want
        seen.add(want)
    assert seen == {True, False}
    assert tg.load_path_connected(tg.Problem(nx, ny, nz), np.zeros(tags.size))  # vacuous


def test_integration_lists_every_entry_point():
    """INTEGRATION.md's table names every entry point the header declares,
    each against the reference interface it replaces (or "no counterpart")."""
    doc = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    listed = set()
    for cell in re.findall(r"`(tg_[\w/]+)`", doc):
        head, *rest = cell.split("/")
        listed.add(head)
        stem = head.rsplit("_", 1)[0]  # tg_job_create/step -> tg_job_step
        listed.update(f"{stem}_{r}" for r in rest)
    missing = [n for n in declared_functions() if n not in listed]
    assert not missing, missing
