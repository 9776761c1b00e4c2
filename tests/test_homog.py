"""Periodic homogenization (core/tests/harness/lattice_homog_probe.cpp:290-412).

CPU: the oracle's restatement recovers the isotropic tensor of a solid cell (the
harness's H1 self-check), matches tensors built on the reference's own compiled
operator for a gyroid and an octet cell, and gives symmetric, positive definite
tensors on lattice cells.  GPU: the batched CUDA path against the oracle on the same cells
(Jacobi-PCG on both sides at tolerance 1e-10: tensors within 1e-7 relative),
the H1 check, and batch invariance (a cell's tensor does not depend on the
other cells or strain columns in the batch: bit-identical)."""
import numpy as np
import pytest

from topopt_gb300 import lattice


def iso(E=1.0, nu=0.3):
    c11 = E * (1 - nu) / ((1 + nu) * (1 - 2 * nu))
    c12 = E * nu / ((1 + nu) * (1 - 2 * nu))
    c44 = E / (2 * (1 + nu))
    C = np.zeros((6, 6))
    C[:3, :3] = c12
    np.fill_diagonal(C[:3, :3], c11)
    C[3, 3] = C[4, 4] = C[5, 5] = c44
    return C


def relerr(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def test_oracle_solid_cell_isotropic(port):
    CH, it, conv = port.homogenize(4, 4, 4, tol=1e-12)
    assert conv
    assert relerr(CH, iso()) < 1e-12
    CH, _, _ = port.homogenize(3, 4, 5, h=0.5, E=2.0, nu=0.25, tol=1e-12)
    assert relerr(CH, iso(2.0, 0.25)) < 1e-12


@pytest.mark.parametrize("kind", ["gyroid", "octet"])
def test_oracle_pinned_to_reference_operator(port, golden, kind):
    """The restatement against tensors built on the reference's own compiled
    operator (fea_matfree_apply folded onto the torus, tests/golden/make_golden.py
    _homog_reference_operator): a 12^3 gyroid at relative density 0.3 and an
    octet truss at 0.25, both solved to 1e-12."""
    cell = golden[f"homog_{kind}_cell"]
    want = golden[f"homog_{kind}_CH"]
    CH, it, conv = port.homogenize(12, 12, 12, solid=cell, tol=1e-12)
    assert conv
    assert relerr(CH, want) < 1e-10


def test_oracle_lattice_tensor_properties(port):
    cell = lattice.cell("gyroid", 12, lattice.calibrate("gyroid", 12, 0.3))
    CH, it, conv = port.homogenize(12, 12, 12, solid=cell.ravel(), tol=1e-10)
    assert conv and it > 0
    assert np.abs(CH - CH.T).max() < 1e-8 * np.abs(CH).max()
    assert np.linalg.eigvalsh(0.5 * (CH + CH.T)).min() > 0
    assert CH[0, 0] < iso()[0, 0]


@pytest.mark.gpu
def test_gpu_solid_cell_isotropic(tg):
    CH, info = tg.homogenize(np.ones((8, 8, 8), np.uint8), tolerance=1e-12)
    assert info["converged"] and info["systems"] == 6
    assert relerr(CH[0], iso()) < 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("kind,vpc,rho", [("gyroid", 16, 0.3), ("octet", 16, 0.2),
                                          ("schwarzD", 12, 0.35)])
def test_gpu_matches_oracle(tg, port, kind, vpc, rho):
    cell = lattice.cell(kind, vpc, lattice.calibrate(kind, vpc, rho))
    want, it, conv = port.homogenize(vpc, vpc, vpc, solid=cell.ravel(), tol=1e-10)
    got, info = tg.homogenize(cell, tolerance=1e-10)
    assert conv and info["converged"]
    assert relerr(got[0], want) < 1e-7
    assert abs(info["iterations_max"] - it) <= max(5, it // 10)


@pytest.mark.gpu
def test_gpu_batch_invariance(tg):
    cells, _ = lattice.batch(3, vpc=12, seed=5)
    rng = np.random.default_rng(3)
    cells[2] = (rng.random((12, 12, 12)) > 0.35).astype(np.uint8)
    full, info = tg.homogenize(cells, tolerance=1e-10)
    assert info["systems"] == 18
    for i in range(3):
        solo, _ = tg.homogenize(cells[i], tolerance=1e-10)
        assert np.array_equal(solo[0], full[i])
    sub, info = tg.homogenize(cells, cases=0b001001, tolerance=1e-10)
    assert info["systems"] == 6
    assert np.array_equal(sub[:, :, [0, 3]], full[:, :, [0, 3]])
    assert np.all(sub[:, :, [1, 2, 4, 5]] == 0.0)


@pytest.mark.gpu
def test_gpu_homogenize_errors(tg):
    with pytest.raises(ValueError, match="cases_mask"):
        tg.homogenize(np.ones((4, 4, 4), np.uint8), cases=0)
    with pytest.raises(ValueError, match="cases_mask"):
        tg.homogenize(np.ones((4, 4, 4), np.uint8), cases=0x40)
    with pytest.raises(tg.SolverNonConvergence):
        tg.homogenize(np.ones((6, 6, 6), np.uint8), tolerance=1e-14, max_iterations=2)


@pytest.mark.gpu
def test_gpu_mixed_matches_fp64(tg):
    """Mixed precision (FP32 inner Jacobi-PCG, FP64 refinement on the FP64
    residual) reaches the same tolerance: tensors agree with the FP64 form."""
    cells, _ = lattice.batch(4, vpc=16, seed=9)
    c64, i64 = tg.homogenize(cells, tolerance=1e-10)
    c32, i32 = tg.homogenize(cells, tolerance=1e-10, precision=tg.PREC_MIXED)
    assert i64["converged"] and i32["converged"] and i32["refinements"] >= 2
    for a, b in zip(c32, c64):
        assert relerr(a, b) < 1e-8
    solo, _ = tg.homogenize(cells[1], tolerance=1e-10, precision=tg.PREC_MIXED)
    assert np.array_equal(solo[0], c32[1])


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["gyroid", "octet"])
@pytest.mark.parametrize("prec", [0, 1])
def test_gpu_matches_reference_operator_tensors(tg, golden, kind, prec):
    """The batched CUDA path (FP64 and mixed) against the tensors built on the
    reference's own compiled operator."""
    cell = golden[f"homog_{kind}_cell"].reshape(12, 12, 12)
    got, info = tg.homogenize(cell, tolerance=1e-10, precision=prec)
    assert info["converged"]
    assert relerr(got[0], golden[f"homog_{kind}_CH"]) < 1e-7
