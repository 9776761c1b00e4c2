"""ctypes binding of libtopopt_gb300.so (include/topopt_gb300.h).

Names follow the reference library (core/include/topopt/fea.hpp, simp.hpp):
``hex8_stiffness``, ``fea_matfree_apply``, ``fea_solve_mgcg_matfree``,
``simp_compliance``, ``make_density_filter`` (+ ``filter_density`` /
``filter_sensitivity``), ``oc_update``, ``simp_optimize``.  Errors map the
reference's exception classes: ``ValueError`` for std::invalid_argument,
``RuntimeError`` for std::runtime_error (void-gate rejections),
``SolverNonConvergence`` (iterations, residual) for the solver's own exception.
"""
from __future__ import annotations

import ctypes as C
import weakref
import time
import os
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(HERE, "libtopopt_gb300.so")

TG_OK, TG_EINVAL, TG_ESINGULAR, TG_ENONCONV, TG_EDEADLINE, TG_EDEVICE, TG_ENOMEM, TG_ECANCELLED = range(8)
SOLVER_MGCG, SOLVER_JACOBI_CG = 0, 1
PREC_FP64, PREC_MIXED = 0, 1
UPDATER_OC, UPDATER_MMA = 0, 1
RESIDUAL_DF, RESIDUAL_FP64 = 0, 1
SMOOTHER_AUTO, SMOOTHER_JACOBI, SMOOTHER_CHEBYSHEV = 0, 1, 2


class LibraryMissing(RuntimeError):
    """The CUDA library has not been built (run topopt_gb300.build.build())."""


class DeviceError(RuntimeError):
    """A CUDA error inside the library."""


class SolverNonConvergence(RuntimeError):
    """The solve did not reach its tolerance (fea.hpp:418-426)."""

    def __init__(self, msg, iterations=0, residual=0.0):
        super().__init__(msg)
        self.iterations = iterations
        self.residual = residual


# ----------------------------------------------------------------- structs
class _Grid(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
                ("spacing", C.c_double), ("tags", C.c_void_p)]


class _Bc(C.Structure):
    _fields_ = [("node", C.c_int32), ("component", C.c_int32), ("value", C.c_double)]


class _Params(C.Structure):
    _fields_ = [("youngs_modulus", C.c_double), ("poisson", C.c_double), ("penalty", C.c_double),
                ("density_min", C.c_double), ("material_law", C.c_int32), ("e_min", C.c_double)]


class _SolveOpt(C.Structure):
    _fields_ = [("solver", C.c_int32), ("precision", C.c_int32), ("mg_levels", C.c_int32),
                ("mg_iter_budget", C.c_int32), ("omega", C.c_double),
                ("inner_tolerance", C.c_double), ("max_refinements", C.c_int32),
                ("coarsening", C.c_int32), ("graph_mode", C.c_int32),
                ("smooth_sweeps", C.c_int32), ("mixed_residual", C.c_int32),
                ("coarse_smoother", C.c_int32)]


class _CgInfo(C.Structure):
    _fields_ = [("converged", C.c_int32), ("iterations", C.c_int32), ("residual", C.c_double),
                ("used_multigrid", C.c_int32), ("mg_levels", C.c_int32),
                ("hier_built", C.c_int32), ("mg_cycles_attempted", C.c_int32),
                ("matvecs", C.c_int64), ("matvecs_lowp", C.c_int64),
                ("refinements", C.c_int32), ("ng", C.c_int32), ("mixed_fallback", C.c_int32),
                ("inner_breakdowns", C.c_int32), ("t_build_ms", C.c_double),
                ("t_mg_build_ms", C.c_double), ("t_solve_ms", C.c_double),
                ("t_total_ms", C.c_double)]


class _ProjStage(C.Structure):
    _fields_ = [("beta", C.c_double), ("move", C.c_double), ("iterations", C.c_int32)]


class _SimpOpt(C.Structure):
    _fields_ = [("volume_fraction", C.c_double), ("filter_radius", C.c_double),
                ("move", C.c_double), ("change_tol", C.c_double), ("cg_tolerance", C.c_double),
                ("max_iterations", C.c_int32), ("cg_max_iterations", C.c_int32),
                ("solve", _SolveOpt), ("projection", C.POINTER(_ProjStage)),
                ("projection_stages", C.c_int32), ("projection_eta", C.c_double),
                ("initial_design", C.c_void_p), ("updater", C.c_int32),
                ("mma_plateau_window", C.c_int32), ("mma_plateau_tol", C.c_double),
                ("mma_plateau_min_drop", C.c_double), ("mma_plateau_flat_windows", C.c_int32),
                ("active_domain_band", C.c_int32)]


class _Iter(C.Structure):
    _fields_ = [("iteration", C.c_int32), ("compliance", C.c_double), ("change", C.c_double),
                ("volume_fraction", C.c_double), ("cg_iterations", C.c_int32),
                ("mg_levels", C.c_int32), ("used_multigrid", C.c_int32),
                ("oc_volume_evals", C.c_int32), ("t_filter_ms", C.c_double),
                ("t_solve_ms", C.c_double), ("t_sensitivity_ms", C.c_double),
                ("t_update_ms", C.c_double), ("t_total_ms", C.c_double),
                ("t_device_ms", C.c_double), ("fine_matvecs", C.c_int64),
                ("fine_matvecs_lowp", C.c_int64), ("oc_volume_passes", C.c_int32),
                ("beta", C.c_double), ("hier_built", C.c_int32),
                ("mg_cycles_attempted", C.c_int32), ("oc_exact_evals", C.c_int32),
                ("oc_host_fallbacks", C.c_int32), ("active_fraction", C.c_double)]


class _Result(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("converged", C.c_int32), ("cancelled", C.c_int32),
                ("infeasible", C.c_int32), ("non_convergent", C.c_int32),
                ("compliance", C.c_double), ("initial_compliance", C.c_double),
                ("volume_fraction", C.c_double), ("active_domain_band", C.c_int32),
                ("active_domain_latched", C.c_int32),
                ("active_domain_latch_iteration", C.c_int32),
                ("active_domain_escape_count", C.c_int64),
                ("active_fraction_mean", C.c_double),
                ("active_domain_latch_reason", C.c_char * 256)]


_PROGRESS = C.CFUNCTYPE(None, C.c_void_p, C.c_int32, C.c_double, C.c_double)

# ------------------------------------------------------------------ loading
_lib = None


def library_path() -> str:
    return _LIB_PATH


def lib():
    """Load (once) and return the CUDA library; raises LibraryMissing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH):
        raise LibraryMissing(f"{_LIB_PATH} is not built; run topopt_gb300.build.build()")
    L = C.CDLL(_LIB_PATH)
    vp, i32, dbl = C.c_void_p, C.c_int32, C.c_double
    sig = {
        "tg_last_error": ([], C.c_char_p),
        "tg_set_device": ([i32], C.c_int),
        "tg_version": ([], C.c_char_p),
        "tg_hex8_stiffness": ([dbl, dbl, dbl, vp], C.c_int),
        "tg_matfree_apply": ([vp, dbl, dbl, vp, i32, vp, vp], C.c_int),
        "tg_build_reduced": ([vp, vp, dbl, vp, i32, vp, i32, vp, vp, vp, vp], C.c_int),
        "tg_solve": ([vp, vp, dbl, vp, i32, vp, i32, dbl, i32, vp, vp, vp, vp, vp], C.c_int),
        "tg_simp_compliance": ([vp, vp, vp, vp, i32, vp, i32, dbl, i32, vp, vp, vp, vp, vp],
                               C.c_int),
        "tg_filter": ([vp, dbl, i32, vp, vp], C.c_int),
        "tg_oc_update": ([vp, dbl, vp, vp, dbl, dbl, dbl, vp], C.c_int),
        "tg_simp_optimize": ([vp, vp, vp, i32, vp, i32, vp, _PROGRESS, vp, vp, vp, vp, vp, vp],
                             C.c_int),
        "tg_effective_design_mask": ([vp, vp, vp], C.c_int),
        "tg_active_domain_auto_band": ([dbl], C.c_int32),
        "tg_active_domain_mask": ([vp, vp, dbl, i32, vp, vp], C.c_int),
        "tg_active_domain_escape_count": ([vp, vp, vp, dbl, vp], C.c_int),
        "tg_filter_masked": ([vp, vp, dbl, i32, vp, vp], C.c_int),
        "tg_oc_update_masked": ([vp, vp, dbl, vp, vp, dbl, dbl, dbl, vp], C.c_int),
        "tg_simp_optimize_masked": ([vp, vp, vp, i32, vp, i32, vp, vp, _PROGRESS, vp, vp, vp, vp,
                                     vp, vp], C.c_int),
        "tg_homogenize": ([i32, i32, i32, i32, dbl, dbl, dbl, vp, i32, dbl, i32, i32, vp, vp],
                          C.c_int),
        "tg_set_sync_mode": ([i32], C.c_int),
        "tg_heaviside_project": ([C.c_int64, vp, dbl, dbl, vp, vp], C.c_int),
        "tg_heaviside_continuation_schedule": ([vp, i32], C.c_int32),
        "tg_oc_update_projected": ([vp, dbl, vp, vp, vp, dbl, dbl, dbl, dbl, dbl, vp], C.c_int),
        "tg_job_set_stage": ([vp, i32], C.c_int),
        "tg_design_fingerprint": ([vp, C.c_int64], C.c_uint64),
        "tg_write_design_file": ([C.c_char_p, vp, vp, i32], C.c_int32),
        "tg_read_design_file": ([C.c_char_p, vp, vp, vp, i32, vp], C.c_int),
        "tg_write_fields_file": ([C.c_char_p, vp, vp, i32], C.c_int32),
        "tg_iteration_csv_header": ([], C.c_char_p),
        "tg_iteration_record_from": ([vp, i32, vp], None),
        "tg_iteration_csv_row": ([C.c_int64, vp, C.c_int64, vp, C.c_int64], C.c_int64),
        "tg_element_stress": ([vp, dbl, dbl, vp, vp, dbl, vp, vp], C.c_int),
        "tg_load_path_connected": ([vp, vp, dbl, vp], C.c_int),
        "tg_analyze_fixed_design": ([vp, vp, vp, vp, i32, vp, i32, vp, dbl, i32, vp, vp, vp,
                                     vp, vp], C.c_int),
        "tg_self_weight_loads": ([vp, vp, dbl, dbl, vp, vp, C.c_int64], C.c_int64),
        "tg_minimize_plastic": ([vp, vp, vp, i32, vp, i32, vp, vp, vp, _PROGRESS, vp, vp, vp,
                                 vp, vp, vp], C.c_int),
        "tg_server_create": ([vp, vp], C.c_int),
        "tg_server_submit": ([vp, vp, vp, vp, i32, vp, i32, vp, vp, vp], C.c_int),
        "tg_server_wait": ([vp, C.c_int64, vp, vp, vp], C.c_int),
        "tg_server_stats": ([vp, vp], C.c_int),
        "tg_server_destroy": ([vp], None),
        "tg_job_create": ([vp, vp, vp, i32, vp, i32, vp, vp], C.c_int),
        "tg_job_create_masked": ([vp, vp, vp, i32, vp, i32, vp, vp, vp], C.c_int),
        "tg_job_step": ([vp, vp], C.c_int),
        "tg_job_read": ([vp, vp, vp], C.c_int),
        "tg_job_write_design": ([vp, vp], C.c_int),
        "tg_job_read_displacement": ([vp, vp], C.c_int),
        "tg_job_device_bytes": ([vp], C.c_int64),
        "tg_job_estimate_bytes": ([vp, vp], C.c_int64),
        "tg_job_destroy": ([vp], None),
        "tg_job_time_operator": ([vp, i32, i32, vp], C.c_int),
        "tg_host_alloc": ([C.c_int64], C.c_void_p),
        "tg_host_free": ([C.c_void_p], C.c_int),
        "tg_kernel_launches": ([], C.c_int64),
        "tg_device_fma_peaks": ([vp, vp], C.c_int),
        "tg_set_fp32_schedule": ([i32, i32, i32], C.c_int),
        "tg_set_level1_tc": ([i32], C.c_int),
        "tg_set_level1_galerkin_fast": ([i32], C.c_int),
        "tg_set_coarse_fused": ([i32], C.c_int),
        "tg_job_check_level1": ([vp, vp], C.c_int),
        "tg_fp32_schedule": ([i32, i32, i32, vp, vp, vp], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def _check(rc, info: "_CgInfo | None" = None):
    if rc == TG_OK:
        return
    msg = lib().tg_last_error().decode()
    if rc == TG_EINVAL:
        raise ValueError(msg)
    if rc == TG_ESINGULAR:
        raise RuntimeError(msg)
    if rc == TG_ENONCONV:
        it = info.iterations if info is not None else 0
        res = info.residual if info is not None else 0.0
        raise SolverNonConvergence(msg, it, res)
    if rc == TG_ENOMEM:
        raise MemoryError(msg)
    raise DeviceError(f"[{rc}] {msg}")


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f64(a, n=None):
    a = np.ascontiguousarray(a, dtype=np.float64).ravel()
    if n is not None and a.size != n:
        raise ValueError(f"array size {a.size} != expected {n}")
    return a


# ------------------------------------------------------------------- types
class Problem:
    """VoxelGrid + Dirichlet BCs + nodal loads, in the reference's indexing
    (voxel (k*ny+j)*nx+i, node (c*(ny+1)+b)*(nx+1)+a, DOF 3*node+comp)."""

    def __init__(self, nx, ny, nz, spacing=1.0, tags=None, bcs=(), loads=()):
        self.nx, self.ny, self.nz, self.spacing = int(nx), int(ny), int(nz), float(spacing)
        self.nv = self.nx * self.ny * self.nz
        self.nnodes = (self.nx + 1) * (self.ny + 1) * (self.nz + 1)
        self.ndof = 3 * self.nnodes
        self.tags = None if tags is None else np.ascontiguousarray(tags, dtype=np.uint8).ravel()
        if self.tags is not None and self.tags.size != self.nv:
            raise ValueError("tags size != voxel_count")
        bcs, loads = list(bcs), list(loads)
        self._bcs = (_Bc * max(1, len(bcs)))(*[_Bc(int(n), int(c), float(v)) for n, c, v in bcs])
        self._loads = (_Bc * max(1, len(loads)))(*[_Bc(int(n), int(c), float(v)) for n, c, v in loads])
        self.nbc, self.nloads = len(bcs), len(loads)
        self.bcs, self.loads = bcs, loads
        self._grid = _Grid(self.nx, self.ny, self.nz, self.spacing, _p(self.tags))

    def node(self, a, b, c):
        return (c * (self.ny + 1) + b) * (self.nx + 1) + a

    def _args(self):
        return (C.byref(self._grid), C.cast(self._bcs, C.c_void_p), self.nbc,
                C.cast(self._loads, C.c_void_p), self.nloads)

    @classmethod
    def cantilever(cls, nx, ny, nz, total_load=-1.0, spacing=1.0, tags=None):
        """The benchmark cantilever: every DOF of the x = 0 face clamped; a total
        -z load spread equally over the x = nx edge nodes at mid-height."""
        pb = cls(nx, ny, nz, spacing, tags)
        bcs = [(pb.node(0, b, c), k, 0.0) for c in range(nz + 1) for b in range(ny + 1)
               for k in range(3)]
        nodes = [pb.node(nx, b, nz // 2) for b in range(ny + 1)]
        loads = [(n, 2, total_load / len(nodes)) for n in nodes]
        return cls(nx, ny, nz, spacing, tags, bcs, loads)


@dataclass
class SolveOptions:
    solver: int = SOLVER_MGCG
    precision: int = PREC_FP64
    mg_levels: int = 0
    mg_iter_budget: int = 0
    omega: float = 0.0
    inner_tolerance: float = 0.0
    max_refinements: int = 0
    coarsening: int = 0  # COARSEN_DEFAULT / COARSEN_REFERENCE / COARSEN_ALIGNED
    graph_mode: int = 0  # GRAPH_ON / GRAPH_OFF
    smooth_sweeps: int = 0  # Jacobi sweeps per side of the coarse correction (0 = 1)
    mixed_residual: int = 0  # RESIDUAL_DF (double-float, default) / RESIDUAL_FP64
    coarse_smoother: int = 0  # SMOOTHER_AUTO / SMOOTHER_JACOBI / SMOOTHER_CHEBYSHEV (mixed)

    def _c(self):
        return _SolveOpt(self.solver, self.precision, self.mg_levels, self.mg_iter_budget,
                         self.omega, self.inner_tolerance, self.max_refinements,
                         self.coarsening, self.graph_mode, self.smooth_sweeps,
                         self.mixed_residual, self.coarse_smoother)


@dataclass
class SimpParams:
    youngs_modulus: float = 1.0
    poisson: float = 0.3
    penalty: float = 3.0
    density_min: float = 1e-3
    material_law: int = 0
    e_min: float = 0.0

    def _c(self):
        return _Params(self.youngs_modulus, self.poisson, self.penalty, self.density_min,
                       self.material_law, self.e_min)


@dataclass
class SimpOptions:
    volume_fraction: float = 0.5
    filter_radius: float = 1.5
    move: float = 0.2
    change_tol: float = 0.01
    cg_tolerance: float = 1e-8
    max_iterations: int = 200
    cg_max_iterations: int = 0
    solve: SolveOptions = field(default_factory=SolveOptions)
    # Heaviside projection + beta continuation (simp.hpp:1426-1444): a list of
    # (beta, move, iterations) stages; empty = the unprojected loop.
    projection: list = field(default_factory=list)
    projection_eta: float = 0.5
    # Warm start (simp.hpp:1557-1575): a raw seed density per voxel, or None.
    initial_design: object = None
    # The updater (simp.hpp:1119): UPDATER_OC or UPDATER_MMA, and MMA's plateau
    # stop (simp.hpp:1241-1277 defaults).
    updater: int = 0
    mma_plateau_window: int = 10
    mma_plateau_tol: float = 1e-3
    mma_plateau_min_drop: float = 0.05
    mma_plateau_flat_windows: int = 3
    # The active domain (simp.hpp:1185-1227): 0 off, > 0 the band half-width in
    # voxels, < 0 the auto band ceil(filter_radius) + 1.
    active_domain_band: int = 0

    def total_iterations(self) -> int:
        if self.projection:
            return int(sum(int(s[2]) for s in self.projection))
        return int(self.max_iterations)

    def _c(self):
        o = _SimpOpt(self.volume_fraction, self.filter_radius, self.move, self.change_tol,
                     self.cg_tolerance, self.max_iterations, self.cg_max_iterations,
                     self.solve._c())
        if self.projection:
            arr = (_ProjStage * len(self.projection))(
                *[_ProjStage(float(b), float(m), int(it)) for b, m, it in self.projection])
            o.projection = C.cast(arr, C.POINTER(_ProjStage))  # kept alive by o._objects
            o._stages = arr
            o.projection_stages = len(self.projection)
        o.projection_eta = self.projection_eta
        o.updater = self.updater
        o.mma_plateau_window = self.mma_plateau_window
        o.mma_plateau_tol = self.mma_plateau_tol
        o.mma_plateau_min_drop = self.mma_plateau_min_drop
        o.mma_plateau_flat_windows = self.mma_plateau_flat_windows
        o.active_domain_band = self.active_domain_band
        if self.initial_design is not None:
            seed = np.ascontiguousarray(self.initial_design, dtype=np.float64).ravel()
            o._seed = seed  # kept alive with the struct
            o.initial_design = seed.ctypes.data_as(C.c_void_p)
        return o


def heaviside_continuation_schedule():
    """heaviside_continuation_schedule (simp.hpp:530): [(beta, move, iterations)]."""
    buf = (_ProjStage * 8)()
    n = lib().tg_heaviside_continuation_schedule(C.cast(buf, C.c_void_p), 8)
    return [(buf[i].beta, buf[i].move, buf[i].iterations) for i in range(n)]


@dataclass
class CgInfo:
    converged: bool
    iterations: int
    residual: float
    used_multigrid: bool
    mg_levels: int
    hier_built: bool
    mg_cycles_attempted: int
    matvecs: int
    matvecs_lowp: int
    refinements: int
    ng: int
    mixed_fallback: bool
    inner_breakdowns: int
    t_build_ms: float
    t_mg_build_ms: float
    t_solve_ms: float
    t_total_ms: float

    @classmethod
    def _from(cls, c: _CgInfo):
        return cls(bool(c.converged), c.iterations, c.residual, bool(c.used_multigrid),
                   c.mg_levels, bool(c.hier_built), c.mg_cycles_attempted, c.matvecs,
                   c.matvecs_lowp, c.refinements, c.ng, bool(c.mixed_fallback),
                   c.inner_breakdowns, c.t_build_ms, c.t_mg_build_ms,
                   c.t_solve_ms, c.t_total_ms)


# --------------------------------------------------------------- functions
def hex8_stiffness(youngs_modulus, poisson, element_size):
    """hex_element.cpp:93-115: the 24x24 element stiffness (row-major)."""
    ke = np.zeros(576)
    _check(lib().tg_hex8_stiffness(youngs_modulus, poisson, element_size, _p(ke)))
    return ke.reshape(24, 24)


def fea_matfree_apply(pb: Problem, u, youngs_modulus=1.0, poisson=0.3, youngs_per_voxel=None,
                      precision=PREC_FP64):
    """fea.hpp:760-766: y = K u over the full grid (no BCs)."""
    u = _f64(u, pb.ndof)
    yv = None if youngs_per_voxel is None else _f64(youngs_per_voxel, pb.nv)
    y = np.zeros(pb.ndof)
    _check(lib().tg_matfree_apply(C.byref(pb._grid), youngs_modulus, poisson, _p(yv), precision,
                                  _p(u), _p(y)))
    return y


def fea_build_reduced(pb: Problem, youngs_per_voxel=None, poisson=0.3):
    """The void-DOF gate of mf_build_reduced: kept mask, reduced rhs, Jacobi
    inverse diagonal (full length)."""
    yv = None if youngs_per_voxel is None else _f64(youngs_per_voxel, pb.nv)
    kept = np.zeros(pb.ndof, np.uint8)
    rhs, inv = np.zeros(pb.ndof), np.zeros(pb.ndof)
    ng = C.c_int32(0)
    g, b, nb, l, nl = pb._args()
    _check(lib().tg_build_reduced(g, _p(yv), poisson, b, nb, l, nl, _p(kept), _p(rhs), _p(inv),
                                  C.byref(ng)))
    return dict(kept=kept, rhs=rhs, invdiag=inv, ng=ng.value)


def fea_solve_mgcg_matfree(pb: Problem, youngs_per_voxel, poisson=0.3, tolerance=1e-8,
                           max_iterations=0, options: SolveOptions | None = None,
                           active_mask=None, initial_guess=None):
    """fea.hpp:707-715 (graded overload).  Returns (u, CgInfo)."""
    yv = _f64(youngs_per_voxel, pb.nv)
    am = None if active_mask is None else np.ascontiguousarray(active_mask, np.uint8).ravel()
    ig = None if initial_guess is None else _f64(initial_guess, pb.ndof)
    u = np.zeros(pb.ndof)
    info = _CgInfo()
    opt = (options or SolveOptions())._c()
    g, b, nb, l, nl = pb._args()
    rc = lib().tg_solve(g, _p(yv), poisson, b, nb, l, nl, tolerance, max_iterations,
                        C.byref(opt), _p(am), _p(ig), _p(u), C.byref(info))
    _check(rc, info)
    return u, CgInfo._from(info)


def simp_compliance(pb: Problem, params: SimpParams, density, tolerance=1e-8, max_iterations=0,
                    options: SolveOptions | None = None):
    """simp.hpp:247-255.  Returns dict(u, dcompliance, compliance, cg)."""
    d = _f64(density, pb.nv)
    u, dc = np.zeros(pb.ndof), np.zeros(pb.nv)
    c = C.c_double(0.0)
    info = _CgInfo()
    prm = params._c()
    opt = (options or SolveOptions())._c()
    g, b, nb, l, nl = pb._args()
    rc = lib().tg_simp_compliance(g, C.byref(prm), _p(d), b, nb, l, nl, tolerance, max_iterations,
                                  C.byref(opt), _p(u), _p(dc), C.byref(c), C.byref(info))
    _check(rc, info)
    return dict(u=u, dcompliance=dc, compliance=c.value, cg=CgInfo._from(info))


COARSEN_DEFAULT, COARSEN_REFERENCE, COARSEN_ALIGNED = 0, 1, 2
GRAPH_ON, GRAPH_OFF = 0, 1

# MaskValue (voxel.hpp:42-46).
MASK_ACTIVE, MASK_FROZEN_SOLID, MASK_FROZEN_VOID = 0, 1, 2


def _mask(pb: Problem, mask):
    m = np.ascontiguousarray(mask, dtype=np.uint8).ravel()
    if m.size != pb.nv:
        raise ValueError("mask size != voxel_count")
    return m


class DensityFilter:
    """make_density_filter(grid, radius[, mask]) (simp.cpp:834-896): over the
    solid voxels, or with a mask over the solid Active voxels."""

    def __init__(self, pb: Problem, radius: float, mask=None):
        self.pb, self.radius = pb, float(radius)
        self.mask = None if mask is None else _mask(pb, mask)

    def _run(self, v, adjoint):
        v = _f64(v, self.pb.nv)
        out = np.zeros(self.pb.nv)
        if self.mask is None:
            _check(lib().tg_filter(C.byref(self.pb._grid), self.radius, adjoint, _p(v), _p(out)))
        else:
            _check(lib().tg_filter_masked(C.byref(self.pb._grid), _p(self.mask), self.radius,
                                          adjoint, _p(v), _p(out)))
        return out

    def filter_density(self, x):
        return self._run(x, 0)

    def filter_sensitivity(self, s):
        return self._run(s, 1)


def make_density_filter(pb: Problem, radius: float, mask=None) -> DensityFilter:
    if not (radius > 0.0):
        raise ValueError("make_density_filter: radius must be > 0")
    return DensityFilter(pb, radius, mask)


def active_domain_auto_band(filter_radius):
    """active_domain_auto_band (simp.hpp:314): ceil(filter_radius) + 1, at least 1."""
    return int(lib().tg_active_domain_auto_band(float(filter_radius)))


def active_domain_mask(pb: Problem, density, density_min, band):
    """active_domain_mask (simp.hpp:298-300) on the device: (mask uint8[nv], ones)."""
    d = _f64(density, pb.nv)
    out = np.zeros(pb.nv, np.uint8)
    n = C.c_int64(0)
    _check(lib().tg_active_domain_mask(C.byref(pb._grid), _p(d), float(density_min), int(band),
                                       _p(out), C.byref(n)))
    return out, int(n.value)


def active_domain_escape_count(pb: Problem, density, prev_mask, density_min):
    """active_domain_escape_count (simp.hpp:336-339) on the device; prev_mask None
    (the first armed iteration) counts 0."""
    d = _f64(density, pb.nv)
    pm = None if prev_mask is None else np.ascontiguousarray(prev_mask, dtype=np.uint8).ravel()
    if pm is not None and pm.size != pb.nv:
        raise ValueError("prev_mask size != voxel_count")
    n = C.c_int64(0)
    _check(lib().tg_active_domain_escape_count(C.byref(pb._grid), _p(d),
                                               None if pm is None else _p(pm),
                                               float(density_min), C.byref(n)))
    return int(n.value)


def effective_design_mask(pb: Problem, mask):
    """simp.cpp:2610-2633: Empty -> FrozenVoid, Load/Fixture -> FrozenSolid."""
    m = _mask(pb, mask)
    out = np.zeros(pb.nv, np.uint8)
    _check(lib().tg_effective_design_mask(C.byref(pb._grid), _p(m), _p(out)))
    return out


def oc_update(pb: Problem, filt: DensityFilter, density, dcompliance, volume_fraction, move=0.2,
              density_min=1e-3):
    """oc_update (simp.hpp:481-485): bit-identical to the reference."""
    d, dc = _f64(density, pb.nv), _f64(dcompliance, pb.nv)
    out = np.zeros(pb.nv)
    _check(lib().tg_oc_update(C.byref(pb._grid), filt.radius, _p(d), _p(dc), volume_fraction, move,
                              density_min, _p(out)))
    return out


def oc_update_masked(pb: Problem, radius, mask, density, dcompliance, volume_fraction, move=0.2,
                     density_min=1e-3):
    """oc_update_masked (simp.cpp:2662-2720) under effective_design_mask(mask) and
    its Active-only filter: bit-identical to the reference."""
    m = _mask(pb, mask)
    d, dc = _f64(density, pb.nv), _f64(dcompliance, pb.nv)
    out = np.zeros(pb.nv)
    _check(lib().tg_oc_update_masked(C.byref(pb._grid), _p(m), float(radius), _p(d), _p(dc),
                                     volume_fraction, move, density_min, _p(out)))
    return out


def heaviside_project(rho_tilde, beta, eta=0.5):
    """heaviside_project and its derivative (simp.hpp:506-514) of an array, on
    the device: returns (value, derivative)."""
    rt = _f64(rho_tilde)
    v, d = np.zeros(rt.size), np.zeros(rt.size)
    _check(lib().tg_heaviside_project(rt.size, _p(rt), float(beta), float(eta), _p(v), _p(d)))
    return v, d


def oc_update_projected(pb: Problem, radius, density, xtilde, dcompliance, beta, eta,
                        volume_fraction, move=0.2, density_min=1e-3):
    """oc_update_projected (simp.cpp:1665-1726) on the solid voxels of ``pb``."""
    d, xt, dc = _f64(density, pb.nv), _f64(xtilde, pb.nv), _f64(dcompliance, pb.nv)
    out = np.zeros(pb.nv)
    _check(lib().tg_oc_update_projected(C.byref(pb._grid), float(radius), _p(d), _p(xt), _p(dc),
                                        float(beta), float(eta), volume_fraction, move,
                                        density_min, _p(out)))
    return out


# ------------------------------------------------- stress and the ladder
@dataclass
class StrengthSpec:
    """Material strength and the acceptance gate of analyze_fixed_design
    (analyze.cpp:145-440, solid posture)."""
    yield_strength: float = 50.0
    z_knockdown: float = 1.0
    build_dir: tuple = (0.0, 0.0, 1.0)
    printed_iso: float = 0.5
    infill_knockdown: float = 1.0
    margin_stop: float = 1.5

    def _c(self):
        return _Strength(self.yield_strength, self.z_knockdown,
                         (C.c_double * 3)(*[float(v) for v in self.build_dir]), self.printed_iso,
                         self.infill_knockdown, self.margin_stop)


class _Strength(C.Structure):
    _fields_ = [("yield_strength", C.c_double), ("z_knockdown", C.c_double),
                ("build_dir", C.c_double * 3), ("printed_iso", C.c_double),
                ("infill_knockdown", C.c_double), ("margin_stop", C.c_double)]


class _Analysis(C.Structure):
    _fields_ = [("non_convergent", C.c_int32), ("cg_iterations", C.c_int32),
                ("load_path_ok", C.c_int32), ("accepted", C.c_int32),
                ("printed_voxels", C.c_int64), ("compliance", C.c_double),
                ("max_von_mises", C.c_double), ("max_interlayer_tension", C.c_double),
                ("margin_in_plane", C.c_double), ("margin_interlayer", C.c_double),
                ("margin_worst_case", C.c_double), ("margin_effective", C.c_double)]


class _LadderOpt(C.Structure):
    _fields_ = [("volume_fractions", C.c_void_p), ("rungs", C.c_int32),
                ("warm_start_inherit", C.c_int32), ("strength", _Strength)]


class _LadderRung(C.Structure):
    _fields_ = [("volume_fraction", C.c_double), ("trajectory_ok", C.c_int32),
                ("analysed", C.c_int32), ("accepted", C.c_int32), ("optimization", _Result),
                ("analysis", _Analysis)]


class _LadderResult(C.Structure):
    _fields_ = [("evaluated", C.c_int32), ("recommended", C.c_int32),
                ("stopped_on_margin", C.c_int32), ("cancelled", C.c_int32)]


def _struct_dict(st):
    out = {}
    for name, _ in st._fields_:
        v = getattr(st, name)
        out[name] = _struct_dict(v) if isinstance(v, C.Structure) else v
    return out


def element_stress(pb: Problem, youngs_modulus, poisson, u, density=None, iso=0.5):
    """hex8_stress at every voxel centre (on the device): (sigma (nv, 6), von Mises)."""
    uu = _f64(u, pb.ndof)
    d = None if density is None else _f64(density, pb.nv)
    sig, vm = np.zeros(6 * pb.nv), np.zeros(pb.nv)
    _check(lib().tg_element_stress(C.byref(pb._grid), youngs_modulus, poisson, _p(uu), _p(d), iso,
                                   _p(sig), _p(vm)))
    return sig.reshape(pb.nv, 6), vm


def load_path_connected(pb: Problem, density, iso=0.5) -> bool:
    """load_path_connected (voxel.hpp:359-361) on the problem's tags."""
    d = _f64(density, pb.nv)
    out = C.c_int32(0)
    _check(lib().tg_load_path_connected(C.byref(pb._grid), _p(d), iso, C.byref(out)))
    return bool(out.value)


def analyze_fixed_design(pb: Problem, params: SimpParams, density, strength: StrengthSpec,
                         cg_tolerance=1e-8, cg_max_iterations=0, solve: SolveOptions | None = None,
                         fields=False):
    """analyze_fixed_design (analyze.cpp:145-440), solid posture: a dict of the
    certification solve, peak stresses, margins and the verdict (+ the von Mises
    and stress fields with fields=True)."""
    d = _f64(density, pb.nv)
    prm, st = params._c(), strength._c()
    so = (solve or SolveOptions())._c()
    out = _Analysis()
    vm = np.zeros(pb.nv) if fields else None
    sig = np.zeros(6 * pb.nv) if fields else None
    disp = np.zeros(pb.ndof) if fields else None
    g, b, nb, l, nl = pb._args()
    _check(lib().tg_analyze_fixed_design(g, C.byref(prm), _p(d), b, nb, l, nl, C.byref(st),
                                         cg_tolerance, cg_max_iterations, C.byref(so),
                                         C.byref(out), _p(vm), _p(sig), _p(disp)))
    res = _struct_dict(out)
    if fields:
        res["von_mises"] = vm
        res["stress"] = sig.reshape(pb.nv, 6)
        res["displacement"] = disp
    return res


def self_weight_loads(pb: Problem, density, gravity=9.81e-3, direction=(0.0, 0.0, -1.0),
                      mask=None):
    """self_weight_loads (fea.hpp:215; masked form minimize_plastic.cpp:132-143):
    a list of (node, component, value)."""
    m = None if mask is None else _mask(pb, mask)
    dv = (C.c_double * 3)(*[float(v) for v in direction])
    n = lib().tg_self_weight_loads(C.byref(pb._grid), _p(m), float(density), float(gravity), dv,
                                   None, 0)
    if n < 0:
        raise ValueError(lib().tg_last_error().decode())
    buf = (_Bc * max(int(n), 1))()  # tg_nodal_load has the same layout
    lib().tg_self_weight_loads(C.byref(pb._grid), _p(m), float(density), float(gravity), dv,
                               C.cast(buf, C.c_void_p), int(n))
    return [(buf[i].node, buf[i].component, buf[i].value) for i in range(int(n))]


def minimize_plastic(pb: Problem, params: SimpParams, options: SimpOptions, ladder,
                     strength: StrengthSpec, mask=None, warm_start_inherit=True, progress=None,
                     cancel=None):
    """The volume-fraction ladder walk of minimize_plastic
    (minimize_plastic.cpp:1402-2742, OC): per-rung records, the recommended
    (lightest accepted) rung and its design / physical density."""
    lad = np.ascontiguousarray(ladder, dtype=np.float64)
    prm, opt = params._c(), options._c()
    lo = _LadderOpt(lad.ctypes.data_as(C.c_void_p), lad.size, int(bool(warm_start_inherit)),
                    strength._c())
    rungs = (_LadderRung * lad.size)()
    res = _LadderResult()
    design, phys = np.zeros(pb.nv), np.zeros(pb.nv)
    m = None if mask is None else _mask(pb, mask)
    cb = _PROGRESS(lambda ctx, it, c, ch: progress(it, c, ch)) if progress else _PROGRESS()
    cptr = None if cancel is None else cancel.ctypes.data_as(C.c_void_p)
    g, b, nb, l, nl = pb._args()
    _check(lib().tg_minimize_plastic(g, C.byref(prm), b, nb, l, nl, C.byref(opt), _p(m),
                                     C.byref(lo), cb, None, cptr, C.cast(rungs, C.c_void_p),
                                     C.byref(res), _p(design), _p(phys)))
    out = _struct_dict(res)
    out["rungs"] = [_struct_dict(rungs[i]) for i in range(res.evaluated)]
    if res.recommended >= 0:
        out["design"], out["physical_density"] = design, phys
    return out


# ------------------------------------------- design.bin / fields.bin / csv
class _Frame(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
                ("origin", C.c_double * 3), ("spacing", C.c_double)]


class _DesignVariant(C.Structure):
    _fields_ = [("requested_volume_fraction", C.c_double),
                ("achieved_volume_fraction", C.c_double), ("margin_worst_case", C.c_double),
                ("margin_effective", C.c_double), ("max_von_mises", C.c_double),
                ("accepted", C.c_int32), ("iterations", C.c_int32),
                ("applied_build_dir", C.c_double * 3),
                ("build_direction_auto_applied", C.c_int32), ("export_baked", C.c_int32),
                ("fingerprint", C.c_uint64), ("density", C.c_void_p)]


class _FieldsVariant(C.Structure):
    _fields_ = [("requested_volume_fraction", C.c_double), ("mass_grams", C.c_double),
                ("support_volume_voxels", C.c_int32), ("von_mises", C.c_void_p),
                ("displacement", C.c_void_p)]


class _IterRecord(C.Structure):
    _fields_ = ([("iteration", C.c_int32), ("compliance", C.c_double),
                 ("volume_fraction", C.c_double), ("plateau", C.c_int32),
                 ("cg_iterations", C.c_int32), ("cg_multigrid", C.c_int32),
                 ("beta", C.c_double), ("hier_built", C.c_int32),
                 ("mg_cycles_attempted", C.c_int32), ("infeasible", C.c_int32),
                 ("recycle_dim", C.c_int32), ("active_fraction", C.c_double)] +
                [(n, C.c_double) for n in (
                    "total_ms", "tail_prev_ms", "filter_ms", "project_ms", "solve_ms", "fea_ms",
                    "sens_ms", "update_ms", "analysis_ms", "observe_ms", "residual_ms",
                    "solver_build_ms", "mg_build_ms", "mg_ms", "cg_ms", "geneo_setup_ms",
                    "geneo_apply_ms", "recycle_ms")] +
                [("fea_solves", C.c_int64), ("matvecs", C.c_int64), ("geneo_dim", C.c_int32),
                 ("geneo_action", C.c_int32), ("geneo_burn", C.c_int32),
                 ("geneo_threshold", C.c_int32), ("rss_mb", C.c_double),
                 ("peak_rss_mb", C.c_double), ("compressed_mb", C.c_double),
                 ("available_mb", C.c_double), ("major_faults", C.c_int64),
                 ("swapins", C.c_int64)])


def _frame(dims, spacing=1.0, origin=(0.0, 0.0, 0.0)):
    nx, ny, nz = (int(v) for v in dims)
    return _Frame(nx, ny, nz, (C.c_double * 3)(*[float(v) for v in origin]), float(spacing))


def design_fingerprint(density) -> int:
    """design_fingerprint (design_store.hpp:102): FNV-1a 64 over the bytes."""
    d = _f64(density)
    return int(lib().tg_design_fingerprint(_p(d), d.size))


def write_design_file(path, dims, variants, spacing=1.0, origin=(0.0, 0.0, 0.0)) -> int:
    """design.bin v1 (design_store.hpp:40-90).  ``variants``: dicts with
    requested_volume_fraction, achieved_volume_fraction, margin_worst_case,
    margin_effective, max_von_mises, accepted, iterations, density (and
    optionally applied_build_dir, build_direction_auto_applied, export_baked)."""
    fr = _frame(dims, spacing, origin)
    nv = fr.nx * fr.ny * fr.nz
    arr = (_DesignVariant * max(len(variants), 1))()
    keep = []
    for i, v in enumerate(variants):
        d = _f64(v["density"], nv)
        keep.append(d)
        arr[i] = _DesignVariant(
            v["requested_volume_fraction"], v.get("achieved_volume_fraction", 0.0),
            v.get("margin_worst_case", 0.0), v.get("margin_effective", 0.0),
            v.get("max_von_mises", 0.0), int(bool(v.get("accepted", False))),
            int(v.get("iterations", 0)),
            (C.c_double * 3)(*v.get("applied_build_dir", (0.0, 0.0, 1.0))),
            int(bool(v.get("build_direction_auto_applied", False))),
            int(bool(v.get("export_baked", False))), 0, d.ctypes.data_as(C.c_void_p))
    n = lib().tg_write_design_file(str(path).encode(), C.byref(fr), C.cast(arr, C.c_void_p),
                                   len(variants))
    if n < 0:
        raise ValueError(lib().tg_last_error().decode())
    return int(n)


def read_design_file(path):
    """read_design_file (design_store.hpp:183): frame and variants (version,
    counts and fingerprints checked)."""
    fr, cnt = _Frame(), C.c_int32(0)
    _check(lib().tg_read_design_file(str(path).encode(), C.byref(fr), C.byref(cnt), None, 0,
                                     None))
    nv = fr.nx * fr.ny * fr.nz
    arr = (_DesignVariant * max(cnt.value, 1))()
    dens = np.zeros(max(cnt.value, 1) * nv)
    _check(lib().tg_read_design_file(str(path).encode(), C.byref(fr), C.byref(cnt),
                                     C.cast(arr, C.c_void_p), cnt.value, _p(dens)))
    out = []
    for i in range(cnt.value):
        v = {f[0]: getattr(arr[i], f[0]) for f in _DesignVariant._fields_ if f[0] != "density"}
        v["applied_build_dir"] = tuple(arr[i].applied_build_dir)
        v["density"] = dens[i * nv:(i + 1) * nv].copy()
        out.append(v)
    return dict(dims=(fr.nx, fr.ny, fr.nz), origin=tuple(fr.origin), spacing=fr.spacing,
                variants=out)


def write_fields_file(path, dims, variants, spacing=1.0, origin=(0.0, 0.0, 0.0)) -> int:
    """fields.bin v1 (fields.hpp:33-75): dicts with requested_volume_fraction,
    mass_grams, support_volume_voxels, von_mises (nv), displacement (ndof)."""
    fr = _frame(dims, spacing, origin)
    nv = fr.nx * fr.ny * fr.nz
    ndof = 3 * (fr.nx + 1) * (fr.ny + 1) * (fr.nz + 1)
    arr = (_FieldsVariant * max(len(variants), 1))()
    keep = []
    for i, v in enumerate(variants):
        vm, dp = _f64(v["von_mises"], nv), _f64(v["displacement"], ndof)
        keep += [vm, dp]
        arr[i] = _FieldsVariant(v["requested_volume_fraction"], v.get("mass_grams", 0.0),
                                int(v.get("support_volume_voxels", 0)),
                                vm.ctypes.data_as(C.c_void_p), dp.ctypes.data_as(C.c_void_p))
    n = lib().tg_write_fields_file(str(path).encode(), C.byref(fr), C.cast(arr, C.c_void_p),
                                   len(variants))
    if n < 0:
        raise ValueError(lib().tg_last_error().decode())
    return int(n)


def iteration_csv_header() -> str:
    return lib().tg_iteration_csv_header().decode()


def iteration_csv_row(rung, record, wall_ms=0) -> str:
    """One iterations.csv row: ``record`` is a dict of tg_iteration_record fields
    (missing fields at the schema's absent values) or a history row of
    simp_optimize (converted by tg_iteration_record_from)."""
    rec = _IterRecord()
    if "t_total_ms" in record:
        row = _Iter(**{f[0]: record[f[0]] for f in _Iter._fields_ if f[0] in record})
        lib().tg_iteration_record_from(C.byref(row), int(record.get("infeasible", 0)),
                                       C.byref(rec))
    else:
        rec.active_fraction = 1.0
        for k in ("rss_mb", "peak_rss_mb", "compressed_mb", "available_mb"):
            setattr(rec, k, -1.0)
        rec.major_faults = rec.swapins = -1
        for k, v in record.items():
            setattr(rec, k, v)
    buf = C.create_string_buffer(1024)
    n = lib().tg_iteration_csv_row(int(rung), C.byref(rec), int(wall_ms), buf, 1024)
    if n < 0:
        raise ValueError("iteration_csv_row: formatting failed")
    return buf.value.decode()


def write_iterations_csv(path, rows, wall_ms=None):
    """iterations.csv: the header and one row per (rung, history row)."""
    with open(path, "w") as f:
        f.write(iteration_csv_header() + "\n")
        for rung, row in rows:
            f.write(iteration_csv_row(rung, row, int(time.time() * 1000)
                                      if wall_ms is None else wall_ms))


class _HomogInfo(C.Structure):
    _fields_ = [("iterations_max", C.c_int32), ("converged", C.c_int32), ("systems", C.c_int32),
                ("iterations_total", C.c_int64), ("refinements", C.c_int32),
                ("t_setup_ms", C.c_double),
                ("t_solve_ms", C.c_double), ("t_total_ms", C.c_double)]


def homogenize(cells, spacing=1.0, youngs_modulus=1.0, poisson=0.3, cases=0x3F, tolerance=1e-9,
               max_iterations=0, precision=PREC_FP64, check=True):
    """Periodic homogenization (lattice_homog_probe.cpp:290-412) of a batch of unit
    cells: ``cells`` is a uint8 array (ncell, nz, ny, nx) or (nz, ny, nx) of voxel
    tags (0 = void).  Returns (CH of shape (ncell, 6, 6), info dict)."""
    t = np.ascontiguousarray(cells, dtype=np.uint8)
    if t.ndim == 3:
        t = t[None]
    if t.ndim != 4:
        raise ValueError("cells must be (ncell, nz, ny, nx) or (nz, ny, nx)")
    nc, nz, ny, nx = t.shape
    ch = np.zeros((nc, 6, 6))
    info = _HomogInfo()
    rc = lib().tg_homogenize(nc, nx, ny, nz, spacing, youngs_modulus, poisson, _p(t), cases,
                             tolerance, max_iterations, precision, _p(ch), C.byref(info))
    d = {f[0]: getattr(info, f[0]) for f in _HomogInfo._fields_}
    if check or rc != TG_ENONCONV:
        _check(rc)
    return ch, d


def host_array(n: int, dtype=np.float64) -> np.ndarray:
    """A numpy array of ``n`` elements in page-locked host memory (tg_host_alloc),
    freed when the array is garbage-collected: host buffers the job API copies
    to and from by direct DMA."""
    nbytes = int(n) * np.dtype(dtype).itemsize
    ptr = lib().tg_host_alloc(max(nbytes, 1))
    if not ptr:
        raise MemoryError("tg_host_alloc failed")
    buf = (C.c_char * max(nbytes, 1)).from_address(ptr)
    arr = np.frombuffer(buf, dtype=dtype, count=int(n))
    weakref.finalize(buf, lib().tg_host_free, C.c_void_p(ptr))
    return arr


def kernel_launches() -> int:
    return int(lib().tg_kernel_launches())


SCHED_PENCIL, SCHED_COLUMN = 0, 1
# (element rows per thread, warps per CTA, x/y in paired FP32 instructions)
FP32_SHAPES = [(4, 4, False), (6, 4, False), (3, 4, False), (2, 8, False),
               (4, 4, True), (6, 4, True), (3, 4, True), (2, 8, True)]


APPLY_L1_STENCIL, APPLY_L1_TC = 3, 4


def set_level1_tc(on: bool):
    """Level 1 of the mixed V-cycle on the tensor cores (True, default) or as the
    assembled FP32 stencil (False), for solvers created afterwards."""
    _check(lib().tg_set_level1_tc(int(bool(on))))


def set_level1_galerkin_fast(on: bool):
    """Level 1's fast-path Galerkin matrices from the bandwidth-bound kernel
    (True, default) or all from the general kernel (False); bit-identical."""
    _check(lib().tg_set_level1_galerkin_fast(int(bool(on))))


def set_coarse_fused(on: bool):
    """The small levels of the mixed V-cycle (from the first of at most 4096
    nodes to the coarsest) as one thread-block-cluster launch (True) or a launch
    per step (False, default), for solvers created afterwards."""
    _check(lib().tg_set_coarse_fused(int(bool(on))))


def set_fp32_schedule(kind=None, shape=0, kz=32):
    """Force the FP32 operator's schedule for every later launch (kind None
    clears the override: the per-grid table decides again)."""
    _check(lib().tg_set_fp32_schedule(-1 if kind is None else int(kind), int(shape), int(kz)))


def fp32_schedule(nx, ny, nz):
    """(kind, shape, kz) the FP32 operator uses on an nx x ny x nz grid now."""
    k, s, z = C.c_int32(0), C.c_int32(0), C.c_int32(0)
    _check(lib().tg_fp32_schedule(nx, ny, nz, C.byref(k), C.byref(s), C.byref(z)))
    return k.value, s.value, z.value


def device_fma_peaks():
    """(fp64, fp32) sustained FMA TFLOP/s from the library's microbenchmark."""
    a, b = C.c_double(0.0), C.c_double(0.0)
    _check(lib().tg_device_fma_peaks(C.byref(a), C.byref(b)))
    return a.value, b.value


def _rows(hist, n):
    keys = [f[0] for f in _Iter._fields_]
    return [{k: getattr(hist[i], k) for k in keys} for i in range(n)]


def simp_optimize(pb: Problem, params: SimpParams, options: SimpOptions, progress=None,
                  cancel=None, mask=None):
    """simp.hpp:1783-1786 (OC; projected when ``options.projection`` holds a
    stage plan); with ``mask`` the masked overload (simp.hpp:1820-1824).  ``cancel`` may be a one-element int32 numpy array
    polled once per iteration."""
    prm, opt = params._c(), options._c()
    hist = (_Iter * options.total_iterations())()
    design, phys = np.zeros(pb.nv), np.zeros(pb.nv)
    res = _Result()
    cb = _PROGRESS(lambda ctx, it, c, ch: progress(it, c, ch)) if progress else _PROGRESS()
    cptr = None if cancel is None else cancel.ctypes.data_as(C.c_void_p)
    g, b, nb, l, nl = pb._args()
    if mask is None:
        rc = lib().tg_simp_optimize(g, C.byref(prm), b, nb, l, nl, C.byref(opt), cb, None, cptr,
                                    C.cast(hist, C.c_void_p), _p(design), _p(phys),
                                    C.byref(res))
    else:
        m = _mask(pb, mask)
        rc = lib().tg_simp_optimize_masked(g, C.byref(prm), b, nb, l, nl, C.byref(opt), _p(m),
                                           cb, None, cptr, C.cast(hist, C.c_void_p), _p(design),
                                           _p(phys), C.byref(res))
    _check(rc)
    return dict(design=design, physical_density=phys, compliance=res.compliance,
                initial_compliance=res.initial_compliance, volume_fraction=res.volume_fraction,
                iterations=res.iterations, converged=bool(res.converged),
                cancelled=bool(res.cancelled), infeasible=bool(res.infeasible),
                non_convergent=bool(res.non_convergent), history=_rows(hist, res.iterations),
                active_domain=dict(band=res.active_domain_band,
                                   latched=bool(res.active_domain_latched),
                                   latch_iteration=res.active_domain_latch_iteration,
                                   escape_count=res.active_domain_escape_count,
                                   fraction_mean=res.active_fraction_mean,
                                   reason=res.active_domain_latch_reason.decode()))


class _ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_int64), ("max_active", C.c_int32), ("device", C.c_int32)]


class _ServerResult(C.Structure):
    _fields_ = [("ticket", C.c_int64), ("status", C.c_int32), ("estimate_bytes", C.c_int64),
                ("t_queue_ms", C.c_double), ("t_run_ms", C.c_double),
                ("t_latency_ms", C.c_double), ("result", _Result)]


class _ServerCounters(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("admitted", C.c_int64), ("completed", C.c_int64),
                ("rejected", C.c_int64), ("queued", C.c_int64), ("active", C.c_int32),
                ("peak_active", C.c_int32), ("bytes_in_use", C.c_int64),
                ("peak_bytes", C.c_int64), ("uptime_ms", C.c_double), ("busy_ms", C.c_double)]


class Server:
    """Continuous batching of optimisation jobs (tg_server_*): jobs are admitted
    in arrival order by HBM budget and free slots, each runs resident on its own
    stream, and their work overlaps on the GPU."""

    def __init__(self, hbm_budget_bytes: int, max_active: int = 8, device: int = 0):
        cfg = _ServerConfig(int(hbm_budget_bytes), int(max_active), int(device))
        self._h = C.c_void_p()
        _check(lib().tg_server_create(C.byref(cfg), C.byref(self._h)))
        self._nv = {}

    def submit(self, pb: Problem, params: SimpParams, options: SimpOptions, mask=None) -> int:
        prm, opt = params._c(), options._c()
        m = None if mask is None else _mask(pb, mask)
        t = C.c_int64(0)
        g, b, nb, l, nl = pb._args()
        _check(lib().tg_server_submit(self._h, g, C.byref(prm), b, nb, l, nl, C.byref(opt), _p(m),
                                      C.byref(t)))
        self._nv[t.value] = pb.nv
        return t.value

    def wait(self, ticket: int, fields=True):
        nv = self._nv.pop(ticket)
        r = _ServerResult()
        design, phys = (np.zeros(nv), np.zeros(nv)) if fields else (None, None)
        rc = lib().tg_server_wait(self._h, ticket, C.byref(r), _p(design), _p(phys))
        _check(rc)
        res = r.result
        return dict(ticket=r.ticket, estimate_bytes=r.estimate_bytes, t_queue_ms=r.t_queue_ms,
                    t_run_ms=r.t_run_ms, t_latency_ms=r.t_latency_ms, design=design,
                    physical_density=phys, compliance=res.compliance,
                    volume_fraction=res.volume_fraction, iterations=res.iterations,
                    converged=bool(res.converged), non_convergent=bool(res.non_convergent),
                    infeasible=bool(res.infeasible))

    def stats(self):
        c = _ServerCounters()
        _check(lib().tg_server_stats(self._h, C.byref(c)))
        return {f[0]: getattr(c, f[0]) for f in _ServerCounters._fields_}

    def close(self):
        if self._h:
            lib().tg_server_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def set_sync_mode(mode: int):
    """How host threads wait for the GPU: 0 default, 1 spin, 2 yield, 3 blocking."""
    _check(lib().tg_set_sync_mode(int(mode)))


def job_estimate_bytes(pb: Problem, options: SimpOptions) -> int:
    opt = options._c()
    return int(lib().tg_job_estimate_bytes(C.byref(pb._grid), C.byref(opt)))


class SimpJob:
    """A resident optimisation job: density, displacement and the multigrid
    hierarchy stay on the device between ``step()`` calls."""

    def __init__(self, pb: Problem, params: SimpParams, options: SimpOptions, mask=None):
        self.pb = pb
        self._prm, self._opt = params._c(), options._c()
        self._h = C.c_void_p()
        g, b, nb, l, nl = pb._args()
        if mask is None:
            _check(lib().tg_job_create(g, C.byref(self._prm), b, nb, l, nl, C.byref(self._opt),
                                       C.byref(self._h)))
        else:
            self._mask = _mask(pb, mask)
            _check(lib().tg_job_create_masked(g, C.byref(self._prm), b, nb, l, nl,
                                              C.byref(self._opt), _p(self._mask),
                                              C.byref(self._h)))

    def step(self):
        row = _Iter()
        _check(lib().tg_job_step(self._h, C.byref(row)))
        return {f[0]: getattr(row, f[0]) for f in _Iter._fields_}

    def set_stage(self, stage: int):
        """Run the next steps at stage ``stage`` of the options' projection plan."""
        _check(lib().tg_job_set_stage(self._h, int(stage)))

    def read(self, x=None, xp=None):
        """The design and physical density, into ``x`` / ``xp`` when given
        (float64 arrays of nv, e.g. host_array buffers) or new arrays."""
        x = np.zeros(self.pb.nv) if x is None else x
        xp = np.zeros(self.pb.nv) if xp is None else xp
        for a in (x, xp):
            if a.dtype != np.float64 or a.size != self.pb.nv or not a.flags.c_contiguous:
                raise ValueError("read buffers must be contiguous float64 arrays of nv")
        _check(lib().tg_job_read(self._h, _p(x), _p(xp)))
        return x, xp

    def check_level1(self):
        """Level-1 operator, tensor cores against the assembled FP32 stencil on a
        seeded vector: max |difference| / max |stencil result|."""
        d = C.c_double(0.0)
        _check(lib().tg_job_check_level1(self._h, C.byref(d)))
        return d.value

    def read_displacement(self):
        """The displacement of the last solve (the next step's warm start)."""
        u = np.zeros(self.pb.ndof)
        _check(lib().tg_job_read_displacement(self._h, _p(u)))
        return u

    def write_design(self, x):
        x = _f64(x, self.pb.nv)
        _check(lib().tg_job_write_design(self._h, _p(x)))

    def time_operator(self, precision=PREC_FP64, reps=20):
        """Average device ms of one fine-operator launch (CUDA events)."""
        ms = C.c_double(0.0)
        _check(lib().tg_job_time_operator(self._h, precision, reps, C.byref(ms)))
        return ms.value

    @property
    def device_bytes(self):
        return int(lib().tg_job_device_bytes(self._h))

    def close(self):
        if self._h:
            lib().tg_job_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
