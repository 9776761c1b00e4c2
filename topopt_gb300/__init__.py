"""GB300-native voxel-SIMP inner loop: Python face of the C-ABI library.

The product is ``libtopopt_gb300.so`` (hand-written sm_103a kernels behind the
``extern "C"`` boundary declared in include/topopt_gb300.h).  This module binds
it with ctypes and mirrors the reference's library API (Anarkissed/TopOpt,
core/include/topopt/fea.hpp and simp.hpp): the same function names, argument
meaning and error classes, so callers written against the reference read the
same here.

There is no CPU fallback: importing works anywhere, but every call that needs
the library raises ``LibraryMissing`` when it has not been built, and every call
fails with ``DeviceError`` when no CUDA device is usable.
"""
from __future__ import annotations

from ._capi import (  # noqa: F401
    CgInfo,
    DensityFilter,
    DeviceError,
    LibraryMissing,
    Problem,
    Server,
    SimpJob,
    SimpParams,
    SimpOptions,
    SolveOptions,
    SolverNonConvergence,
    device_fma_peaks,
    active_domain_auto_band,
    active_domain_escape_count,
    active_domain_mask,
    effective_design_mask,
    fea_build_reduced,
    kernel_launches,
    set_fp32_schedule,
    set_level1_tc,
    set_coarse_fused,
    APPLY_L1_STENCIL,
    APPLY_L1_TC,
    fp32_schedule,
    SCHED_PENCIL,
    SCHED_COLUMN,
    FP32_SHAPES,
    fea_matfree_apply,
    fea_solve_mgcg_matfree,
    hex8_stiffness,
    job_estimate_bytes,
    homogenize,
    lib,
    library_path,
    make_density_filter,
    oc_update,
    oc_update_masked,
    oc_update_projected,
    design_fingerprint,
    write_design_file,
    read_design_file,
    write_fields_file,
    iteration_csv_header,
    iteration_csv_row,
    write_iterations_csv,
    StrengthSpec,
    element_stress,
    load_path_connected,
    analyze_fixed_design,
    self_weight_loads,
    minimize_plastic,
    heaviside_project,
    heaviside_continuation_schedule,
    simp_compliance,
    simp_optimize,
    set_sync_mode,
    COARSEN_ALIGNED,
    COARSEN_DEFAULT,
    COARSEN_REFERENCE,
    GRAPH_OFF,
    GRAPH_ON,
    MASK_ACTIVE,
    MASK_FROZEN_SOLID,
    MASK_FROZEN_VOID,
    PREC_FP64,
    PREC_MIXED,
    UPDATER_MMA,
    RESIDUAL_DF,
    RESIDUAL_FP64,
    SMOOTHER_AUTO,
    SMOOTHER_CHEBYSHEV,
    SMOOTHER_JACOBI,
    UPDATER_OC,
    SOLVER_MGCG,
    SOLVER_JACOBI_CG,
)

__all__ = [n for n in dir() if not n.startswith("_")]
