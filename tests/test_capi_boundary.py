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


def test_python_face_mirrors_reference_names(tg):
    for n in ("hex8_stiffness", "fea_matfree_apply", "fea_solve_mgcg_matfree", "simp_compliance",
              "make_density_filter", "oc_update", "simp_optimize", "SimpJob",
              "SolverNonConvergence"):
        assert hasattr(tg, n)
