"""ctypes binding of the CPU oracle (test infrastructure only).

Two CPU implementations of the reference voxel-SIMP inner loop share one Python
face here:

* ``OracleLib("port")``  -- oracle/topopt_oracle.c, the C restatement, built by
  ``build_port()`` into oracle/_build/ on any machine;
* ``OracleLib("reference")`` -- the reference's own compiled C++ (built from the
  reference tree by oracle/build_ref.sh into oracle/_ref/), present only where the
  reference tree was available at build time.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this
module.  The product library never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libtopopt_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libtopopt_ref.so")


def reference_root() -> str:
    """Root of the reference source tree: $TOPOPT_REFERENCE_ROOT, else the
    conventional mount point.  The tree is needed only to build or read the
    reference's own code and fixtures; nothing at run time depends on it."""
    return os.environ.get("TOPOPT_REFERENCE_ROOT", "/root/reference")


def reference_path(*parts: str) -> str:
    return os.path.join(reference_root(), *parts)


_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_bp = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")


def build_port(force: bool = False) -> str:
    """Compile the C restatement (gcc, -ffp-contract=off, no -march; OpenMP when
    the compiler has it -- threading never changes a result)."""
    srcs = [os.path.join(HERE, f) for f in ("topopt_oracle.c", "oracle_mg.c")]
    hdr = os.path.join(HERE, "topopt_oracle.h")
    os.makedirs(os.path.dirname(PORT_SO), exist_ok=True)
    newest = max([os.path.getmtime(f) for f in srcs] + [os.path.getmtime(hdr)])
    if force or not os.path.exists(PORT_SO) or newest > os.path.getmtime(PORT_SO):
        base = ["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-ffp-contract=off", "-o",
                PORT_SO + ".tmp"] + srcs + ["-lm"]
        try:
            subprocess.check_call(base[:2] + ["-fopenmp"] + base[2:], stderr=subprocess.DEVNULL)
        except subprocess.CalledProcessError:
            subprocess.check_call(base)
        os.replace(PORT_SO + ".tmp", PORT_SO)
    return PORT_SO


def build_reference() -> str | None:
    """Compile the reference's own code (needs the reference tree); None if absent."""
    script = os.path.join(HERE, "build_ref.sh")
    subprocess.check_call(["bash", script, reference_root()])
    return REF_SO if os.path.exists(REF_SO) else None


class OracleError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


class Problem:
    """A voxel problem in the reference's conventions (see topopt_oracle.h)."""

    def __init__(self, nx, ny, nz, spacing=1.0, solid=None, bcs=(), loads=()):
        self.nx, self.ny, self.nz, self.h = int(nx), int(ny), int(nz), float(spacing)
        self.nv = self.nx * self.ny * self.nz
        self.nnodes = (self.nx + 1) * (self.ny + 1) * (self.nz + 1)
        self.ndof = 3 * self.nnodes
        self.solid = None if solid is None else np.ascontiguousarray(solid, dtype=np.uint8).ravel()
        bcs = list(bcs)
        loads = list(loads)
        self.bc_node = np.array([b[0] for b in bcs], dtype=np.int32)
        self.bc_comp = np.array([b[1] for b in bcs], dtype=np.int32)
        self.bc_val = np.array([b[2] for b in bcs], dtype=np.float64)
        self.ld_node = np.array([l[0] for l in loads], dtype=np.int32)
        self.ld_comp = np.array([l[1] for l in loads], dtype=np.int32)
        self.ld_val = np.array([l[2] for l in loads], dtype=np.float64)

    def node(self, a, b, c):
        return (c * (self.ny + 1) + b) * (self.nx + 1) + a

    def bc_args(self):
        return (len(self.bc_node), self.bc_node, self.bc_comp, self.bc_val,
                len(self.ld_node), self.ld_node, self.ld_comp, self.ld_val)


class OracleLib:
    def __init__(self, kind: str = "port"):
        self.kind = kind
        if kind == "port":
            path = build_port()
            self.lib = C.CDLL(path)
            self._p = "or_"
        elif kind == "reference":
            if not os.path.exists(REF_SO):
                raise FileNotFoundError(REF_SO)
            self.lib = C.CDLL(REF_SO)
            self._p = "ref_"
        else:
            raise ValueError(kind)
        L, p = self.lib, self._p
        getattr(L, p + "last_error").restype = C.c_char_p
        L.__getattr__  # noqa: B018
        self._fn = {}
        sig = {
            "hex8_stiffness": [C.c_double, C.c_double, C.c_double, _dp],
            "apply": [C.c_int] * 3 + [C.c_double, C.c_void_p, C.c_void_p, C.c_double, C.c_double,
                                      _dp, _dp],
            "build_reduced": [C.c_int] * 3 + [C.c_double, C.c_void_p, C.c_void_p, C.c_double,
                                              C.c_double, C.c_int, _ip, _ip, _dp, C.c_int, _ip,
                                              _ip, _dp, _bp, _dp, _dp, _dp, C.POINTER(C.c_int)],
            "simp_compliance": [C.c_int] * 3 + [C.c_double, C.c_void_p, C.c_double, C.c_double,
                                                C.c_double, C.c_double, _dp, C.c_int, _ip, _ip,
                                                _dp, C.c_int, _ip, _ip, _dp, C.c_double, C.c_int,
                                                _dp, _dp, C.POINTER(C.c_double),
                                                C.POINTER(C.c_int), C.POINTER(C.c_double)],
        }
        for name, args in sig.items():
            f = getattr(L, p + name)
            f.argtypes = args
            f.restype = C.c_int
            self._fn[name] = f
        solve = getattr(L, p + ("solve_cg"))
        solve.argtypes = [C.c_int] * 3 + [C.c_double, C.c_void_p, C.c_void_p, C.c_double,
                                          C.c_double, C.c_int, _ip, _ip, _dp, C.c_int, _ip, _ip,
                                          _dp, C.c_double, C.c_int, C.c_void_p, _dp,
                                          C.POINTER(C.c_int), C.POINTER(C.c_double)]
        solve.restype = C.c_int
        self._fn["solve_cg"] = solve
        if kind == "port":
            L.or_filter_make.restype = C.c_void_p
            L.or_filter_make.argtypes = [C.c_int] * 3 + [C.c_void_p, C.c_void_p, C.c_double]
            L.or_filter_free.argtypes = [C.c_void_p]
            L.or_filter_nnz.argtypes = [C.c_void_p]
            L.or_filter_nnz.restype = C.c_size_t
            for n in ("or_filter_weight_sum",):
                getattr(L, n).argtypes = [C.c_void_p, _dp]
            for n in ("or_filter_density", "or_filter_sensitivity"):
                getattr(L, n).argtypes = [C.c_void_p, _dp, _dp]
            L.or_oc_update.argtypes = [C.c_int] * 3 + [C.c_void_p, C.c_void_p, _dp, _dp,
                                                       C.c_double, C.c_double, C.c_double, _dp,
                                                       C.POINTER(C.c_double), C.POINTER(C.c_int)]
            L.or_simp_optimize.argtypes = (
                [C.c_int] * 3 + [C.c_double, C.c_void_p, C.c_double, C.c_double, C.c_double,
                                 C.c_double, C.c_int, _ip, _ip, _dp, C.c_int, _ip, _ip, _dp,
                                 C.c_void_p, _dp, _dp, _dp, _ip, _dp, _dp, C.c_void_p])
            L.or_effective_design_mask.argtypes = [C.c_int] * 3 + [C.c_void_p, _bp, _bp]
            L.or_effective_design_mask.restype = None
            L.or_oc_update_masked.argtypes = [C.c_int] * 3 + [_bp, C.c_void_p, _dp, _dp,
                                                              C.c_double, C.c_double, C.c_double,
                                                              _dp, C.POINTER(C.c_double),
                                                              C.POINTER(C.c_int)]
            L.or_simp_optimize_masked.argtypes = (
                [C.c_int] * 3 + [C.c_double, C.c_void_p, _bp, C.c_double, C.c_double, C.c_double,
                                 C.c_double, C.c_int, _ip, _ip, _dp, C.c_int, _ip, _ip, _dp,
                                 C.c_void_p, _dp, _dp, _dp, _ip, _dp, _dp, C.c_void_p])
            L.or_oc_update_projected.argtypes = ([C.c_int] * 3 + [C.c_void_p, C.c_void_p] +
                                                 [_dp] * 3 + [C.c_double] * 5 + [_dp])
            L.or_heaviside_project.argtypes = [C.c_double] * 3
            L.or_heaviside_project.restype = C.c_double
            L.or_heaviside_project_derivative.argtypes = [C.c_double] * 3
            L.or_heaviside_project_derivative.restype = C.c_double
            L.or_homogenize.argtypes = [C.c_int] * 3 + [C.c_double, C.c_double, C.c_double,
                                                        C.c_void_p, C.c_int, C.c_double, C.c_int,
                                                        _dp, C.POINTER(C.c_int),
                                                        C.POINTER(C.c_int)]
            L.or_sensitivity.argtypes = [C.c_int] * 3 + [C.c_double, C.c_void_p, C.c_double,
                                                         C.c_double, C.c_double, C.c_double, _dp,
                                                         _dp, _dp, C.POINTER(C.c_double)]
        else:
            L.ref_filter.argtypes = [C.c_int] * 3 + [C.c_void_p, C.c_double, C.c_int, _dp, _dp,
                                                     C.c_void_p]
            L.ref_oc_update.argtypes = [C.c_int] * 3 + [C.c_void_p, C.c_double, _dp, _dp,
                                                        C.c_double, C.c_double, C.c_double, _dp]
            L.ref_set_threads.argtypes = [C.c_int]
            L.ref_simp_optimize_projected.argtypes = (
                [C.c_int] * 3 + [C.c_double, C.c_void_p, C.c_double, C.c_double, C.c_double,
                                 C.c_double, C.c_int, _ip, _ip, _dp, C.c_int, _ip, _ip, _dp,
                                 C.c_double, C.c_double, C.c_double, C.c_double, C.c_int,
                                 C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double,
                                 _dp, _dp, _dp, _dp, _dp, _dp, _ip])
            L.ref_project.argtypes = [C.c_double, C.c_double, C.c_double, C.POINTER(C.c_double),
                                      C.POINTER(C.c_double)]
            L.ref_effective_design_mask.argtypes = [C.c_int] * 3 + [C.c_void_p, _bp, _bp]
            L.ref_filter_masked.argtypes = [C.c_int] * 3 + [C.c_void_p, _bp, C.c_double, C.c_int,
                                                            _dp, _dp]
            L.ref_simp_optimize_masked.argtypes = (
                [C.c_int] * 3 + [C.c_double, C.c_void_p, _bp, C.c_double, C.c_double, C.c_double,
                                 C.c_double, C.c_int, _ip, _ip, _dp, C.c_int, _ip, _ip, _dp,
                                 C.c_double, C.c_double, C.c_double, C.c_int, C.c_double,
                                 C.c_double, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _ip])
            L.ref_simp_optimize.argtypes = (
                [C.c_int] * 3 + [C.c_double, C.c_void_p, C.c_double, C.c_double, C.c_double,
                                 C.c_double, C.c_int, _ip, _ip, _dp, C.c_int, _ip, _ip, _dp,
                                 C.c_double, C.c_double, C.c_double, C.c_int, C.c_double,
                                 C.c_double, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _ip])

    # ---------------------------------------------------------------- helpers
    def _check(self, st):
        if st != 0:
            msg = getattr(self.lib, self._p + "last_error")().decode()
            raise OracleError(st, msg)

    @staticmethod
    def _ptr(a):
        return None if a is None else a.ctypes.data_as(C.c_void_p)

    def threads(self):
        if self.kind == "port":
            self.lib.or_threads.restype = C.c_int
            return self.lib.or_threads()
        return 1

    def set_threads(self, n):
        if self.kind == "reference":
            self.lib.ref_set_threads(int(n))
        else:
            self.lib.or_set_threads.argtypes = [C.c_int]
            self.lib.or_set_threads(int(n))

    # ------------------------------------------------------------------- API
    def hex8_stiffness(self, E=1.0, nu=0.3, h=1.0):
        ke = np.zeros(576)
        self._check(self._fn["hex8_stiffness"](E, nu, h, ke))
        return ke.reshape(24, 24)

    def apply(self, pb: Problem, u, factor=None, E=1.0, nu=0.3):
        y = np.zeros(pb.ndof)
        f = None if factor is None else np.ascontiguousarray(factor, dtype=np.float64)
        self._check(self._fn["apply"](pb.nx, pb.ny, pb.nz, pb.h, self._ptr(pb.solid), self._ptr(f),
                                      E, nu, np.ascontiguousarray(u, dtype=np.float64), y))
        return y

    def build_reduced(self, pb: Problem, factor=None, E=1.0, nu=0.3):
        kept = np.zeros(pb.ndof, np.uint8)
        rhs, invd, up = np.zeros(pb.ndof), np.zeros(pb.ndof), np.zeros(pb.ndof)
        ng = C.c_int(0)
        f = None if factor is None else np.ascontiguousarray(factor, dtype=np.float64)
        self._check(self._fn["build_reduced"](pb.nx, pb.ny, pb.nz, pb.h, self._ptr(pb.solid),
                                              self._ptr(f), E, nu, *pb.bc_args(), kept, rhs, invd,
                                              up, C.byref(ng)))
        return dict(kept=kept, rhs=rhs, invdiag=invd, up=up, ng=ng.value)

    def solve_cg(self, pb: Problem, factor=None, E=1.0, nu=0.3, tol=1e-8, max_it=0, guess=None):
        u = np.zeros(pb.ndof)
        it, res = C.c_int(0), C.c_double(0)
        f = None if factor is None else np.ascontiguousarray(factor, dtype=np.float64)
        g = None if guess is None else np.ascontiguousarray(guess, dtype=np.float64)
        self._check(self._fn["solve_cg"](pb.nx, pb.ny, pb.nz, pb.h, self._ptr(pb.solid), self._ptr(f),
                                         E, nu, *pb.bc_args(), tol, max_it, self._ptr(g), u,
                                         C.byref(it), C.byref(res)))
        return u, it.value, res.value

    def mg_solve(self, pb: Problem, factor, nu=0.3, tol=1e-8, max_it=300, max_levels=0,
                 guess=None):
        """The MG-PCG restatement (oracle_mg.c): (u, iterations, residual, levels)."""
        assert self.kind == "port"
        f = np.ascontiguousarray(factor, dtype=np.float64)
        g = None if guess is None else np.ascontiguousarray(guess, dtype=np.float64)
        u = np.zeros(pb.ndof)
        it, res, lev = C.c_int(0), C.c_double(0), C.c_int(0)
        fn = self._sig("mg_solve", [C.c_int] * 3 + [C.c_double, C.c_void_p, _dp, C.c_double,
                                                    C.c_int, _ip, _ip, _dp, C.c_int, _ip, _ip,
                                                    _dp, C.c_double, C.c_int, C.c_int, C.c_void_p,
                                                    _dp, C.c_void_p, C.c_void_p, C.c_void_p])
        self._check(fn(pb.nx, pb.ny, pb.nz, pb.h, self._ptr(pb.solid), f, nu, *pb.bc_args(), tol,
                       max_it, max_levels, self._ptr(g), u, C.byref(it), C.byref(res),
                       C.byref(lev)))
        return u, it.value, res.value, lev.value

    def design_iterations_mg(self, pb: Problem, x, niter, u=None, E0=1.0, nu=0.3, penal=3.0,
                             rho_min=1e-3, volfrac=0.3, radius=1.5, move=0.2, cg_tol=1e-8,
                             cg_max_it=300):
        """niter OC design iterations with the MG-PCG restatement from design x.
        Returns dict(x, u, compliance[], cg[], seconds[niter][5]) where seconds
        are [filter+modulus, reduced system+hierarchy, MG-PCG, sensitivities, OC]."""
        assert self.kind == "port"
        xs = np.array(x, dtype=np.float64, copy=True)
        warm = u is not None
        us = np.zeros(pb.ndof) if u is None else np.array(u, dtype=np.float64, copy=True)
        hc = np.zeros(niter)
        hcg = np.zeros(niter, np.int32)
        ht = np.zeros((niter, 5))
        fn = self._sig("design_iterations_mg",
                       [C.c_int] * 3 + [C.c_double, C.c_void_p] + [C.c_double] * 4 +
                       [C.c_int, _ip, _ip, _dp, C.c_int, _ip, _ip, _dp] + [C.c_double] * 4 +
                       [C.c_int] * 3 + [_dp, _dp, _dp, _ip, _dp])
        self._check(fn(pb.nx, pb.ny, pb.nz, pb.h, self._ptr(pb.solid), E0, nu, penal, rho_min,
                       *pb.bc_args(), volfrac, radius, move, cg_tol, cg_max_it, niter, int(warm),
                       xs, us, hc, hcg, ht))
        return dict(x=xs, u=us, compliance=hc, cg=hcg, seconds=ht)

    def simp_compliance(self, pb: Problem, density, E0=1.0, nu=0.3, penal=3.0, rho_min=1e-3,
                        tol=1e-8, max_it=0):
        u, dc = np.zeros(pb.ndof), np.zeros(pb.nv)
        c, it, res = C.c_double(0), C.c_int(0), C.c_double(0)
        self._check(self._fn["simp_compliance"](
            pb.nx, pb.ny, pb.nz, pb.h, self._ptr(pb.solid), E0, nu, penal, rho_min,
            np.ascontiguousarray(density, dtype=np.float64), *pb.bc_args(), tol, max_it, u, dc,
            C.byref(c), C.byref(it), C.byref(res)))
        return dict(u=u, dc=dc, compliance=c.value, iterations=it.value, residual=res.value)

    def sensitivity(self, pb: Problem, density, u, E0=1.0, nu=0.3, penal=3.0, rho_min=1e-3):
        assert self.kind == "port"
        dc = np.zeros(pb.nv)
        c = C.c_double(0)
        self._check(self.lib.or_sensitivity(pb.nx, pb.ny, pb.nz, pb.h, self._ptr(pb.solid), E0, nu,
                                            penal, rho_min,
                                            np.ascontiguousarray(density, dtype=np.float64),
                                            np.ascontiguousarray(u, dtype=np.float64), dc,
                                            C.byref(c)))
        return c.value, dc

    def filter(self, pb: Problem, x, radius=1.5, adjoint=False):
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.zeros(pb.nv)
        if self.kind == "port":
            f = self.lib.or_filter_make(pb.nx, pb.ny, pb.nz, self._ptr(pb.solid), None, radius)
            if not f:
                self._check(1)
            try:
                (self.lib.or_filter_sensitivity if adjoint else self.lib.or_filter_density)(f, x, out)
            finally:
                self.lib.or_filter_free(f)
        else:
            self._check(self.lib.ref_filter(pb.nx, pb.ny, pb.nz, self._ptr(pb.solid), radius,
                                            int(adjoint), x, out, None))
        return out

    def weight_sum(self, pb: Problem, radius=1.5):
        hs = np.zeros(pb.nv)
        if self.kind == "port":
            f = self.lib.or_filter_make(pb.nx, pb.ny, pb.nz, self._ptr(pb.solid), None, radius)
            self.lib.or_filter_weight_sum(f, hs)
            self.lib.or_filter_free(f)
        else:
            tmp = np.zeros(pb.nv)
            self._check(self.lib.ref_filter(pb.nx, pb.ny, pb.nz, self._ptr(pb.solid), radius, 0,
                                            np.zeros(pb.nv), tmp, hs.ctypes.data_as(C.c_void_p)))
        return hs

    def oc_update(self, pb: Problem, density, dc, volfrac, radius=1.5, move=0.2, rho_min=1e-3):
        xn = np.zeros(pb.nv)
        d = np.ascontiguousarray(density, dtype=np.float64)
        g = np.ascontiguousarray(dc, dtype=np.float64)
        if self.kind == "port":
            f = self.lib.or_filter_make(pb.nx, pb.ny, pb.nz, self._ptr(pb.solid), None, radius)
            lam, nvol = C.c_double(0), C.c_int(0)
            try:
                self._check(self.lib.or_oc_update(pb.nx, pb.ny, pb.nz, self._ptr(pb.solid), f, d, g,
                                                  volfrac, move, rho_min, xn, C.byref(lam),
                                                  C.byref(nvol)))
            finally:
                self.lib.or_filter_free(f)
        else:
            self._check(self.lib.ref_oc_update(pb.nx, pb.ny, pb.nz, self._ptr(pb.solid), radius, d,
                                               g, volfrac, move, rho_min, xn))
        return xn

    # ---------------------------------------------------- stress and ladder
    def _sig(self, name, args, res=C.c_int):
        f = getattr(self.lib, self._p + name)
        f.argtypes = args
        f.restype = res
        return f

    def hex8_stress(self, E, nu, h, ue, xi=0.0, eta=0.0, zeta=0.0):
        """hex8_stress (hex_element.cpp:242-316): (sigma[6], von_mises)."""
        ue = np.ascontiguousarray(ue, dtype=np.float64)
        sig, vm = np.zeros(6), C.c_double(0)
        f = self._sig("hex8_stress", [C.c_double] * 3 + [_dp] + [C.c_double] * 3 +
                      [_dp, C.POINTER(C.c_double)])
        self._check(f(E, nu, h, ue, xi, eta, zeta, sig, C.byref(vm)))
        return sig, vm.value

    def stress_margin(self, yield_strength, z_knockdown, max_vm, max_il):
        """compute_stress_margin: (in_plane, interlayer, worst_case)."""
        out = np.zeros(3)
        f = self._sig("stress_margin", [C.c_double] * 4 + [_dp])
        self._check(f(yield_strength, z_knockdown, max_vm, max_il, out))
        return tuple(out)

    def load_path_connected(self, pb: Problem, density, iso=0.5):
        d = np.ascontiguousarray(density, dtype=np.float64)
        if self.kind == "port":
            f = self._sig("load_path_connected", [C.c_int] * 3 + [C.c_void_p, _dp, C.c_double])
            return bool(f(pb.nx, pb.ny, pb.nz, self._ptr(pb.solid), d, iso))
        out = C.c_int(0)
        f = self._sig("load_path_connected", [C.c_int] * 3 + [C.c_void_p, _dp, C.c_double,
                                                              C.POINTER(C.c_int)])
        self._check(f(pb.nx, pb.ny, pb.nz, self._ptr(pb.solid), d, iso, C.byref(out)))
        return bool(out.value)

    def analyze_fixed_design(self, pb: Problem, density, E0=1.0, nu=0.3, penal=3.0,
                             rho_min=1e-3, yield_strength=50.0, z_knockdown=1.0,
                             build_dir=(0.0, 0.0, 1.0), iso=0.5, infill_knockdown=1.0,
                             margin_stop=1.5, cg_tol=1e-8, cg_max_it=0):
        """The solid-posture analyze_fixed_design: dict + von Mises field."""
        d = np.ascontiguousarray(density, dtype=np.float64)
        vm = np.zeros(pb.nv)
        if self.kind == "port":
            st = _OrStrength(yield_strength, z_knockdown, (C.c_double * 3)(*build_dir), iso,
                             infill_knockdown, margin_stop)
            out = _OrAnalysis()
            f = self._sig("analyze_fixed_design",
                          [C.c_int] * 3 + [C.c_double, C.c_void_p] + [C.c_double] * 4 +
                          [_dp, C.c_int, _ip, _ip, _dp, C.c_int, _ip, _ip, _dp, C.c_void_p,
                           C.c_double, C.c_int, C.c_void_p, _dp])
            self._check(f(pb.nx, pb.ny, pb.nz, pb.h, self._ptr(pb.solid), E0, nu, penal, rho_min,
                          d, *pb.bc_args(), C.byref(st), cg_tol, cg_max_it, C.byref(out), vm))
            return _analysis_dict(out), vm
        od, oi = np.zeros(7), np.zeros(4, np.int32)
        bd = np.ascontiguousarray(build_dir, dtype=np.float64)
        f = self._sig("analyze_fixed_design",
                      [C.c_int] * 3 + [C.c_double, C.c_void_p] + [C.c_double] * 4 +
                      [_dp, C.c_int, _ip, _ip, _dp, C.c_int, _ip, _ip, _dp, C.c_double,
                       C.c_double, _dp] + [C.c_double] * 4 + [C.c_int, _dp, _ip, _dp])
        self._check(f(pb.nx, pb.ny, pb.nz, pb.h, self._ptr(pb.solid), E0, nu, penal, rho_min, d,
                      *pb.bc_args(), yield_strength, z_knockdown, bd, iso, infill_knockdown,
                      margin_stop, cg_tol, cg_max_it, od, oi, vm))
        return dict(non_convergent=int(oi[0]), printed_voxels=int(oi[1]),
                    load_path_ok=int(oi[2]), accepted=int(oi[3]), compliance=od[0],
                    max_von_mises=od[1], max_interlayer=od[2], margin_in_plane=od[3],
                    margin_interlayer=od[4], margin_worst=od[5], margin_effective=od[6]), vm

    def active_domain_auto_band(self, radius):
        """active_domain_auto_band (simp.cpp:440-447)."""
        return int(self._sig("active_domain_auto_band", [C.c_double])(radius))

    def active_domain_mask(self, pb: Problem, density, rho_min, band):
        """active_domain_mask (simp.cpp:449-528) on pb's tags (pb.solid)."""
        d = np.ascontiguousarray(density, dtype=np.float64)
        out = np.zeros(pb.nv, np.uint8)
        f = self._sig("active_domain_mask", [C.c_int] * 3 + [C.c_void_p, _dp, C.c_double,
                                                             C.c_int, C.c_void_p])
        self._check(f(pb.nx, pb.ny, pb.nz, self._ptr(pb.solid), d, rho_min, band,
                      out.ctypes.data_as(C.c_void_p)))
        return out

    def active_domain_escape_count(self, pb: Problem, density, prev, rho_min):
        """active_domain_escape_count (simp.cpp:530-556); prev None = no band yet."""
        d = np.ascontiguousarray(density, dtype=np.float64)
        pm = None if prev is None else np.ascontiguousarray(prev, dtype=np.uint8)
        if self.kind == "port":
            f = self._sig("active_domain_escape_count",
                          [C.c_int] * 3 + [C.c_void_p, _dp, C.c_void_p, C.c_double],
                          C.c_longlong)
            return int(f(pb.nx, pb.ny, pb.nz, self._ptr(pb.solid), d, self._ptr(pm), rho_min))
        out = C.c_longlong(0)
        f = self._sig("active_domain_escape_count",
                      [C.c_int] * 3 + [C.c_void_p, _dp, C.c_void_p, C.c_double,
                                       C.POINTER(C.c_longlong)])
        self._check(f(pb.nx, pb.ny, pb.nz, self._ptr(pb.solid), d, self._ptr(pm), rho_min,
                      C.byref(out)))
        return int(out.value)

    def simp_optimize_active(self, pb: Problem, band, mask=None, seed=None, E0=1.0, nu=0.3,
                             penal=3.0, rho_min=1e-3, volfrac=0.3, radius=1.5, move=0.2,
                             max_it=50, change_tol=0.01, cg_tol=1e-8, cg_max_it=0, updater=0):
        """simp_optimize (OC; plain, or masked with mask) with
        SimpOptions::active_domain_band = band and an optional warm-start seed:
        the history with each iteration's active fraction, and the run's
        active-domain record (finalize_active_domain, simp.cpp:1981-1988)."""
        m = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
        sd = None if seed is None else np.ascontiguousarray(seed, dtype=np.float64)
        hc, hch, hvf, haf = (np.zeros(max_it) for _ in range(4))
        design, phys = np.zeros(pb.nv), np.zeros(pb.nv)
        if self.kind == "reference":
            sc, ints = np.zeros(4), np.zeros(8, np.int64)
            reason = C.create_string_buffer(256)
            f = self._sig("simp_optimize_active",
                          [C.c_int] * 3 + [C.c_double, C.c_void_p, C.c_void_p] +
                          [C.c_double] * 4 + [C.c_int, _ip, _ip, _dp, C.c_int, _ip, _ip, _dp] +
                          [C.c_double] * 3 + [C.c_int, C.c_double, C.c_double, C.c_int,
                                              C.c_int, C.c_int, C.c_void_p] + [_dp] * 7 +
                          [C.c_void_p, C.c_char_p])
            self._check(f(pb.nx, pb.ny, pb.nz, pb.h, self._ptr(pb.solid), self._ptr(m), E0, nu,
                          penal, rho_min, *pb.bc_args(), volfrac, radius, move, max_it,
                          change_tol, cg_tol, cg_max_it, band, updater, self._ptr(sd), hc, hch,
                          hvf, haf,
                          design, phys, sc, ints.ctypes.data_as(C.c_void_p), reason))
            n = int(ints[0])
            return dict(compliance=sc[0], volume_fraction=sc[1], initial_compliance=sc[2],
                        iterations=n, converged=bool(ints[1]), non_convergent=bool(ints[2]),
                        infeasible=bool(ints[3]), hist_c=hc[:n], hist_change=hch[:n],
                        hist_vf=hvf[:n], hist_af=haf[:n], design=design, phys=phys,
                        band=int(ints[4]), latched=bool(ints[5]), latch_iteration=int(ints[6]),
                        escape_count=int(ints[7]), fraction_mean=sc[3],
                        reason=reason.value.decode())
        # MMA's plateau stop at the SimpOptions defaults (simp.hpp:1241-1277).
        opt = _OrSimpOptions(volfrac, radius, move, change_tol, cg_tol, max_it, cg_max_it, 0,
                             None, None, None, 0.5, self._ptr(sd), updater,
                             10 if updater == 1 else 0, 1e-3, 0.05, 3, band,
                             haf.ctypes.data_as(C.c_void_p))
        res = _OrSimpResult()
        hcg = np.zeros(max_it, np.int32)
        if m is None:
            self._check(self.lib.or_simp_optimize(
                pb.nx, pb.ny, pb.nz, pb.h, self._ptr(pb.solid), E0, nu, penal, rho_min,
                *pb.bc_args(), C.byref(opt), hc, hch, hvf, hcg, design, phys, C.byref(res)))
        else:
            self._check(self.lib.or_simp_optimize_masked(
                pb.nx, pb.ny, pb.nz, pb.h, self._ptr(pb.solid), m, E0, nu, penal, rho_min,
                *pb.bc_args(), C.byref(opt), hc, hch, hvf, hcg, design, phys, C.byref(res)))
        n = res.iterations
        return dict(compliance=res.compliance, volume_fraction=res.volume_fraction,
                    initial_compliance=res.initial_compliance, iterations=n,
                    converged=bool(res.converged), non_convergent=bool(res.non_convergent),
                    infeasible=bool(res.infeasible), hist_c=hc[:n], hist_change=hch[:n],
                    hist_vf=hvf[:n], hist_af=haf[:n], hist_cg=hcg[:n], design=design, phys=phys,
                    band=res.ad_band, latched=bool(res.ad_latched),
                    latch_iteration=res.ad_latch_iteration, escape_count=res.ad_escape_count,
                    fraction_mean=res.ad_fraction_mean, reason=res.ad_latch_reason.decode())

    def simp_optimize_mma(self, pb: Problem, mask=None, E0=1.0, nu=0.3, penal=3.0,
                          rho_min=1e-3, volfrac=0.3, radius=1.5, move=0.2, max_it=50,
                          change_tol=0.01, cg_tol=1e-8, cg_max_it=0, plateau_window=10,
                          plateau_tol=1e-3, plateau_min_drop=0.05, plateau_flat_windows=3):
        """simp_optimize with the MMA updater (plain, or masked with mask)."""
        m = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
        hc, hch, hvf = np.zeros(max_it), np.zeros(max_it), np.zeros(max_it)
        design, phys = np.zeros(pb.nv), np.zeros(pb.nv)
        if self.kind == "reference":
            sc, ints = np.zeros(3), np.zeros(4, np.int32)
            f = self._sig("simp_optimize_mma",
                          [C.c_int] * 3 + [C.c_double, C.c_void_p, C.c_void_p] +
                          [C.c_double] * 4 + [C.c_int, _ip, _ip, _dp, C.c_int, _ip, _ip, _dp,
                                              C.c_double, C.c_double, C.c_double, C.c_int,
                                              C.c_double, C.c_double, C.c_int, C.c_int,
                                              C.c_double, C.c_double, C.c_int, _dp, _dp, _dp,
                                              _dp, _dp, _dp, _ip])
            self._check(f(pb.nx, pb.ny, pb.nz, pb.h, self._ptr(pb.solid), self._ptr(m), E0, nu,
                          penal, rho_min, *pb.bc_args(), volfrac, radius, move, max_it,
                          change_tol, cg_tol, cg_max_it, plateau_window, plateau_tol,
                          plateau_min_drop, plateau_flat_windows, hc, hch, hvf, design, phys,
                          sc, ints))
            n = int(ints[0])
            return dict(compliance=sc[0], volume_fraction=sc[1], initial_compliance=sc[2],
                        iterations=n, converged=bool(ints[1]), non_convergent=bool(ints[2]),
                        infeasible=bool(ints[3]), hist_c=hc[:n], hist_change=hch[:n],
                        hist_vf=hvf[:n], design=design, phys=phys)
        opt = _OrSimpOptions(volfrac, radius, move, change_tol, cg_tol, max_it, cg_max_it, 0,
                             None, None, None, 0.5, None, 1, plateau_window, plateau_tol,
                             plateau_min_drop, plateau_flat_windows)
        res = _OrSimpResult()
        hcg = np.zeros(max_it, np.int32)
        if m is None:
            self._check(self.lib.or_simp_optimize(
                pb.nx, pb.ny, pb.nz, pb.h, self._ptr(pb.solid), E0, nu, penal, rho_min,
                *pb.bc_args(), C.byref(opt), hc, hch, hvf, hcg, design, phys, C.byref(res)))
        else:
            self._check(self.lib.or_simp_optimize_masked(
                pb.nx, pb.ny, pb.nz, pb.h, self._ptr(pb.solid), m, E0, nu, penal, rho_min,
                *pb.bc_args(), C.byref(opt), hc, hch, hvf, hcg, design, phys, C.byref(res)))
        n = res.iterations
        return dict(compliance=res.compliance, volume_fraction=res.volume_fraction,
                    initial_compliance=res.initial_compliance, iterations=n,
                    converged=bool(res.converged), non_convergent=bool(res.non_convergent),
                    infeasible=bool(res.infeasible), hist_c=hc[:n], hist_change=hch[:n],
                    hist_vf=hvf[:n], hist_cg=hcg[:n], design=design, phys=phys)

    def ladder(self, pb: Problem, mask, ladder, E0=1.0, nu=0.3, penal=3.0, rho_min=1e-3,
               radius=1.5, move=0.2, max_it=30, change_tol=0.01, cg_tol=1e-8, cg_max_it=0,
               inherit=True, yield_strength=50.0, z_knockdown=1.0, build_dir=(0.0, 0.0, 1.0),
               iso=0.5, infill_knockdown=1.0, margin_stop=1.5):
        """The ladder walk (minimize_plastic.cpp:1402-2742, OC): per-rung records,
        the recommended rung, and its design and physical density."""
        lad = np.ascontiguousarray(ladder, dtype=np.float64)
        m = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
        design, phys = np.zeros(pb.nv), np.zeros(pb.nv)
        n = lad.size
        if self.kind == "port":
            opt = _OrSimpOptions(0.5, radius, move, change_tol, cg_tol, max_it, cg_max_it, 0,
                                 None, None, None, 0.5, None)
            st = _OrStrength(yield_strength, z_knockdown, (C.c_double * 3)(*build_dir), iso,
                             infill_knockdown, margin_stop)
            rungs = (_OrRung * n)()
            ev, rec, stop = C.c_int(0), C.c_int(-1), C.c_int(0)
            f = self._sig("ladder", [C.c_int] * 3 + [C.c_double, C.c_void_p, C.c_void_p] +
                          [C.c_double] * 4 + [C.c_int, _ip, _ip, _dp, C.c_int, _ip, _ip, _dp,
                                              C.c_void_p, _dp, C.c_int, C.c_int, C.c_void_p,
                                              C.c_void_p, C.POINTER(C.c_int),
                                              C.POINTER(C.c_int), C.POINTER(C.c_int), _dp, _dp])
            self._check(f(pb.nx, pb.ny, pb.nz, pb.h, self._ptr(pb.solid), self._ptr(m), E0, nu,
                          penal, rho_min, *pb.bc_args(), C.byref(opt), lad, n, int(inherit),
                          C.byref(st), C.cast(rungs, C.c_void_p), C.byref(ev), C.byref(rec),
                          C.byref(stop), design, phys))
            out = []
            for r in range(ev.value):
                g = rungs[r]
                out.append(dict(volume_fraction=g.volume_fraction, iterations=g.iterations,
                                trajectory_ok=g.trajectory_ok, analysed=g.analysed,
                                accepted=g.accepted, compliance=g.compliance,
                                analysis=_analysis_dict(g.analysis)))
            return dict(rungs=out, evaluated=ev.value, recommended=rec.value,
                        stopped_on_margin=bool(stop.value), design=design, phys=phys)
        rd, ri, oi = np.zeros(8 * n), np.zeros(6 * n, np.int32), np.zeros(3, np.int32)
        bd = np.ascontiguousarray(build_dir, dtype=np.float64)
        f = self._sig("ladder", [C.c_int] * 3 + [C.c_double, C.c_void_p, C.c_void_p] +
                      [C.c_double] * 4 + [C.c_int, _ip, _ip, _dp, C.c_int, _ip, _ip, _dp,
                                          C.c_double, C.c_double, C.c_int, C.c_double,
                                          C.c_double, C.c_int, _dp, C.c_int, C.c_int,
                                          C.c_double, C.c_double, _dp, C.c_double, C.c_double,
                                          C.c_double, _dp, _ip, _ip, _dp, _dp])
        self._check(f(pb.nx, pb.ny, pb.nz, pb.h, self._ptr(pb.solid), self._ptr(m), E0, nu, penal,
                      rho_min, *pb.bc_args(), radius, move, max_it, change_tol, cg_tol, cg_max_it,
                      lad, n, int(inherit), yield_strength, z_knockdown, bd, iso,
                      infill_knockdown, margin_stop, rd, ri, oi, design, phys))
        out = []
        for r in range(int(oi[0])):
            d, i = rd[8 * r:8 * r + 8], ri[6 * r:6 * r + 6]
            out.append(dict(volume_fraction=d[0], iterations=int(i[0]), trajectory_ok=int(i[1]),
                            analysed=int(i[2]), accepted=int(i[3]), compliance=d[1],
                            analysis=dict(max_von_mises=d[2], max_interlayer=d[3],
                                          margin_worst=d[4], margin_effective=d[5],
                                          load_path_ok=int(i[4]), non_convergent=int(i[5]))))
        return dict(rungs=out, evaluated=int(oi[0]), recommended=int(oi[1]),
                    stopped_on_margin=bool(oi[2]), design=design, phys=phys)

    def oc_update_projected(self, pb: Problem, density, xtilde, dc, beta, volfrac, radius=1.5,
                            move=0.2, rho_min=1e-3, eta=0.5):
        """oc_update_projected (simp.cpp:1665-1726), port only."""
        if self.kind != "port":
            raise OracleError(1, "oc_update_projected: port only")
        xn = np.zeros(pb.nv)
        d, xt, g = (np.ascontiguousarray(a, dtype=np.float64) for a in (density, xtilde, dc))
        f = self.lib.or_filter_make(pb.nx, pb.ny, pb.nz, self._ptr(pb.solid), None, radius)
        try:
            self._check(self.lib.or_oc_update_projected(pb.nx, pb.ny, pb.nz, self._ptr(pb.solid),
                                                        f, d, xt, g, beta, eta, volfrac, move,
                                                        rho_min, xn))
        finally:
            self.lib.or_filter_free(f)
        return xn

    def project(self, rt, beta, eta=0.5):
        """(heaviside_project, its derivative) at rt."""
        if self.kind == "port":
            return (self.lib.or_heaviside_project(rt, beta, eta),
                    self.lib.or_heaviside_project_derivative(rt, beta, eta))
        v, d = C.c_double(0), C.c_double(0)
        self._check(self.lib.ref_project(rt, beta, eta, C.byref(v), C.byref(d)))
        return v.value, d.value

    def homogenize(self, nx, ny, nz, solid=None, h=1.0, E=1.0, nu=0.3, cases=0x3F, tol=1e-9,
                   max_it=0):
        """Periodic homogenization of one cell (port only: the reference's is a
        harness built on Eigen, absent here).  Returns (CH 6x6, iters, converged)."""
        if self.kind != "port":
            raise NotImplementedError("the reference homogenization harness needs Eigen")
        CH = np.zeros(36)
        it, conv = C.c_int(0), C.c_int(0)
        sp = None if solid is None else np.ascontiguousarray(solid, dtype=np.uint8)
        self._check(self.lib.or_homogenize(nx, ny, nz, h, E, nu, self._ptr(sp), cases, tol, max_it,
                                           CH, C.byref(it), C.byref(conv)))
        return CH.reshape(6, 6), it.value, bool(conv.value)

    # ---- design masks: pb.solid holds the raw voxel tags (0 Empty, 4 Load, 5 Fixture ...)
    def effective_design_mask(self, pb: Problem, mask):
        m = np.ascontiguousarray(mask, dtype=np.uint8)
        eff = np.zeros(pb.nv, np.uint8)
        if self.kind == "port":
            self.lib.or_effective_design_mask(pb.nx, pb.ny, pb.nz, self._ptr(pb.solid), m, eff)
        else:
            self._check(self.lib.ref_effective_design_mask(pb.nx, pb.ny, pb.nz,
                                                           self._ptr(pb.solid), m, eff))
        return eff

    def filter_masked(self, pb: Problem, mask, x, radius=1.5, adjoint=False):
        """make_density_filter(grid, radius, mask) and one pass."""
        m = np.ascontiguousarray(mask, dtype=np.uint8)
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.zeros(pb.nv)
        if self.kind == "port":
            act = (m == 0).astype(np.uint8)
            f = self.lib.or_filter_make(pb.nx, pb.ny, pb.nz, self._ptr(pb.solid),
                                        act.ctypes.data_as(C.c_void_p), radius)
            if not f:
                self._check(1)
            try:
                (self.lib.or_filter_sensitivity if adjoint else self.lib.or_filter_density)(f, x, out)
            finally:
                self.lib.or_filter_free(f)
        else:
            self._check(self.lib.ref_filter_masked(pb.nx, pb.ny, pb.nz, self._ptr(pb.solid), m,
                                                   radius, int(adjoint), x, out))
        return out

    def oc_update_masked(self, pb: Problem, mask, density, dc, volfrac, radius=1.5, move=0.2,
                         rho_min=1e-3):
        """oc_update_masked under the effective mask (port only: the reference's
        is internal to simp.cpp and is pinned through simp_optimize_masked)."""
        if self.kind != "port":
            raise NotImplementedError("oc_update_masked is internal to the reference")
        eff = self.effective_design_mask(pb, mask)
        act = (eff == 0).astype(np.uint8)
        d = np.ascontiguousarray(density, dtype=np.float64)
        g = np.ascontiguousarray(dc, dtype=np.float64)
        xn = np.zeros(pb.nv)
        f = self.lib.or_filter_make(pb.nx, pb.ny, pb.nz, self._ptr(pb.solid),
                                    act.ctypes.data_as(C.c_void_p), radius)
        lam, nvol = C.c_double(0), C.c_int(0)
        try:
            self._check(self.lib.or_oc_update_masked(pb.nx, pb.ny, pb.nz, eff, f, d, g, volfrac,
                                                     move, rho_min, xn, C.byref(lam),
                                                     C.byref(nvol)))
        finally:
            self.lib.or_filter_free(f)
        return xn

    def simp_optimize_masked(self, pb: Problem, mask, E0=1.0, nu=0.3, penal=3.0, rho_min=1e-3,
                             volfrac=0.3, radius=1.5, move=0.2, max_it=50, change_tol=0.01,
                             cg_tol=1e-8, cg_max_it=0, stages=None, eta=0.5):
        m = np.ascontiguousarray(mask, dtype=np.uint8)
        if stages:
            if self.kind != "port":
                raise OracleError(1, "simp_optimize_masked with stages: port only")
            max_it = sum(s[2] for s in stages)
        ns, sb, sm, si, keep = _stage_arrays(stages)
        hc, hch, hvf = np.zeros(max_it), np.zeros(max_it), np.zeros(max_it)
        design, phys = np.zeros(pb.nv), np.zeros(pb.nv)
        if self.kind == "reference":
            sc, ints = np.zeros(3), np.zeros(4, np.int32)
            self._check(self.lib.ref_simp_optimize_masked(
                pb.nx, pb.ny, pb.nz, pb.h, self._ptr(pb.solid), m, E0, nu, penal, rho_min,
                *pb.bc_args(), volfrac, radius, move, max_it, change_tol, cg_tol, cg_max_it, hc,
                hch, hvf, design, phys, sc, ints))
            n = int(ints[0])
            return dict(compliance=sc[0], volume_fraction=sc[1], initial_compliance=sc[2],
                        iterations=n, converged=bool(ints[1]), non_convergent=bool(ints[2]),
                        infeasible=bool(ints[3]), hist_c=hc[:n], hist_change=hch[:n],
                        hist_vf=hvf[:n], design=design, phys=phys)
        opt = _OrSimpOptions(volfrac, radius, move, change_tol, cg_tol, max_it, cg_max_it, ns,
                             self._ptr(sb), self._ptr(sm), self._ptr(si), eta)
        res = _OrSimpResult()
        hcg = np.zeros(max_it, np.int32)
        self._check(self.lib.or_simp_optimize_masked(
            pb.nx, pb.ny, pb.nz, pb.h, self._ptr(pb.solid), m, E0, nu, penal, rho_min,
            *pb.bc_args(), C.byref(opt), hc, hch, hvf, hcg, design, phys, C.byref(res)))
        del keep
        n = res.iterations
        return dict(compliance=res.compliance, volume_fraction=res.volume_fraction,
                    initial_compliance=res.initial_compliance, iterations=n,
                    converged=bool(res.converged), non_convergent=bool(res.non_convergent),
                    infeasible=bool(res.infeasible), hist_c=hc[:n], hist_change=hch[:n],
                    hist_vf=hvf[:n], hist_cg=hcg[:n], design=design, phys=phys)

    def simp_optimize(self, pb: Problem, E0=1.0, nu=0.3, penal=3.0, rho_min=1e-3, volfrac=0.3,
                      radius=1.5, move=0.2, max_it=50, change_tol=0.01, cg_tol=1e-8, cg_max_it=0,
                      stages=None, eta=0.5):
        total = sum(s[2] for s in stages) if stages else max_it
        hc, hch, hvf = np.zeros(total), np.zeros(total), np.zeros(total)
        design, phys = np.zeros(pb.nv), np.zeros(pb.nv)
        ns, sb, sm, si, keep = _stage_arrays(stages)
        if self.kind == "reference":
            sc, ints = np.zeros(3), np.zeros(4, np.int32)
            if stages:
                self._check(self.lib.ref_simp_optimize_projected(
                    pb.nx, pb.ny, pb.nz, pb.h, self._ptr(pb.solid), E0, nu, penal, rho_min,
                    *pb.bc_args(), volfrac, radius, change_tol, cg_tol, cg_max_it, ns,
                    self._ptr(sb), self._ptr(sm), self._ptr(si), eta, hc, hch, hvf, design, phys,
                    sc, ints))
            else:
                self._check(self.lib.ref_simp_optimize(
                    pb.nx, pb.ny, pb.nz, pb.h, self._ptr(pb.solid), E0, nu, penal, rho_min,
                    *pb.bc_args(), volfrac, radius, move, max_it, change_tol, cg_tol, cg_max_it,
                    hc, hch, hvf, design, phys, sc, ints))
            n = int(ints[0])
            return dict(compliance=sc[0], volume_fraction=sc[1], initial_compliance=sc[2],
                        iterations=n, converged=bool(ints[1]), non_convergent=bool(ints[2]),
                        infeasible=bool(ints[3]), hist_c=hc[:n], hist_change=hch[:n],
                        hist_vf=hvf[:n], design=design, phys=phys)
        opt = _OrSimpOptions(volfrac, radius, move, change_tol, cg_tol, max_it, cg_max_it, ns,
                             self._ptr(sb), self._ptr(sm), self._ptr(si), eta)
        res = _OrSimpResult()
        hcg = np.zeros(total, np.int32)
        self._check(self.lib.or_simp_optimize(
            pb.nx, pb.ny, pb.nz, pb.h, self._ptr(pb.solid), E0, nu, penal, rho_min, *pb.bc_args(),
            C.byref(opt), hc, hch, hvf, hcg, design, phys, C.byref(res)))
        del keep
        n = res.iterations
        return dict(compliance=res.compliance, volume_fraction=res.volume_fraction,
                    initial_compliance=res.initial_compliance, iterations=n,
                    converged=bool(res.converged), non_convergent=bool(res.non_convergent),
                    infeasible=bool(res.infeasible), hist_c=hc[:n], hist_change=hch[:n],
                    hist_vf=hvf[:n], hist_cg=hcg[:n], design=design, phys=phys)


class _OrSimpOptions(C.Structure):
    _fields_ = [("volume_fraction", C.c_double), ("filter_radius", C.c_double),
                ("move", C.c_double), ("change_tol", C.c_double), ("cg_tolerance", C.c_double),
                ("max_iterations", C.c_int), ("cg_max_iterations", C.c_int),
                ("nstages", C.c_int), ("stage_beta", C.c_void_p), ("stage_move", C.c_void_p),
                ("stage_iterations", C.c_void_p), ("eta", C.c_double),
                ("initial_design", C.c_void_p), ("updater", C.c_int),
                ("mma_plateau_window", C.c_int), ("mma_plateau_tol", C.c_double),
                ("mma_plateau_min_drop", C.c_double), ("mma_plateau_flat_windows", C.c_int),
                ("active_domain_band", C.c_int), ("hist_active_fraction", C.c_void_p)]


class _OrAnalysis(C.Structure):
    _fields_ = [("non_convergent", C.c_int), ("cg_iterations", C.c_int),
                ("load_path_ok", C.c_int), ("accepted", C.c_int),
                ("printed_voxels", C.c_longlong), ("compliance", C.c_double),
                ("max_von_mises", C.c_double), ("max_interlayer", C.c_double),
                ("margin_in_plane", C.c_double), ("margin_interlayer", C.c_double),
                ("margin_worst", C.c_double), ("margin_effective", C.c_double)]


class _OrStrength(C.Structure):
    _fields_ = [("yield_strength", C.c_double), ("z_knockdown", C.c_double),
                ("build_dir", C.c_double * 3), ("iso", C.c_double),
                ("infill_knockdown", C.c_double), ("margin_stop", C.c_double)]


class _OrRung(C.Structure):
    _fields_ = [("volume_fraction", C.c_double), ("iterations", C.c_int),
                ("trajectory_ok", C.c_int), ("analysed", C.c_int), ("accepted", C.c_int),
                ("compliance", C.c_double), ("analysis", _OrAnalysis)]


def _analysis_dict(a):
    return {f[0]: getattr(a, f[0]) for f in _OrAnalysis._fields_}


# heaviside_continuation_schedule (simp.cpp:367-373): (beta, move, iterations).
CONTINUATION = [(1.0, 0.2, 50), (2.0, 0.2, 50), (4.0, 0.2, 50), (8.0, 0.2, 50), (16.0, 0.1, 50),
                (32.0, 0.05, 50)]


def _stage_arrays(stages):
    if not stages:
        return 0, None, None, None, []
    b = np.ascontiguousarray([s[0] for s in stages], dtype=np.float64)
    m = np.ascontiguousarray([s[1] for s in stages], dtype=np.float64)
    it = np.ascontiguousarray([s[2] for s in stages], dtype=np.int32)
    return len(stages), b, m, it, [b, m, it]


class _OrSimpResult(C.Structure):
    _fields_ = [("iterations", C.c_int), ("converged", C.c_int), ("non_convergent", C.c_int),
                ("infeasible", C.c_int), ("compliance", C.c_double),
                ("volume_fraction", C.c_double), ("initial_compliance", C.c_double),
                ("ad_band", C.c_int), ("ad_latched", C.c_int), ("ad_latch_iteration", C.c_int),
                ("ad_escape_count", C.c_longlong), ("ad_fraction_mean", C.c_double),
                ("ad_latch_reason", C.c_char * 256)]


def cantilever(nx, ny, nz, total_load=-1.0, spacing=1.0, solid=None):
    """Cantilever of the benchmark configs: every DOF of the x=0 face clamped, a
    total z-load spread equally over the nodes of the x=nx edge at mid-height
    (c = nz//2), all b."""
    pb = Problem(nx, ny, nz, spacing, solid)
    bcs = [(pb.node(0, b, c), comp, 0.0) for c in range(nz + 1) for b in range(ny + 1)
           for comp in range(3)]
    cmid = nz // 2
    nodes = [pb.node(nx, b, cmid) for b in range(ny + 1)]
    loads = [(n, 2, total_load / len(nodes)) for n in nodes]
    return Problem(nx, ny, nz, spacing, solid, bcs, loads)


# The Gate V2 benchmark problems and metrics (core/tests/validation/test_gate_v2.cpp:
# 430-466 for the problems, 275-350 for the metrics).  Both run the locked
# projected formulation: filter radius 2.5, eta 0.5, CONTINUATION, change_tol 0,
# solves at 1e-9, volume fraction 0.3, E0 = 1, nu = 0.3, p = 3, rho_min = 1e-3.
GATE_V2 = ("cantilever_24x8x8", "clamped_beam_48x8x8")


def gate_v2_problem(name: str) -> Problem:
    """cantilever_24x8x8: the x = 0 face clamped, Fz = -1/81 on every node of the
    x = nx face.  clamped_beam_48x8x8: both end faces clamped, Fz = -1/9 on the
    nodes (nx/2, b, nz) of the top centre line."""
    nx = {"cantilever_24x8x8": 24, "clamped_beam_48x8x8": 48}[name]
    ny = nz = 8
    pb = Problem(nx, ny, nz)

    def clamp(a):
        return [(pb.node(a, b, c), k, 0.0) for c in range(nz + 1) for b in range(ny + 1)
                for k in range(3)]

    if name == "cantilever_24x8x8":
        bcs = clamp(0)
        fz = -1.0 / ((ny + 1) * (nz + 1))
        loads = [(pb.node(nx, b, c), 2, fz) for c in range(nz + 1) for b in range(ny + 1)]
    else:
        bcs = clamp(0) + clamp(nx)
        fz = -1.0 / (ny + 1)
        loads = [(pb.node(nx // 2, b, nz), 2, fz) for b in range(ny + 1)]
    return Problem(nx, ny, nz, 1.0, None, bcs, loads)


def gate_v2_metrics(nx, ny, nz, rho):
    """(components, M_nd, y-symmetry error) of a projected density on a solid
    grid: 6-connected components of rho > 0.5, the mean of 4 rho (1 - rho), and
    max |rho(i, j, k) - rho(i, ny-1-j, k)|."""
    from scipy import ndimage
    r = np.asarray(rho, dtype=np.float64).reshape(nz, ny, nx)
    _, ncomp = ndimage.label(r > 0.5)
    mnd = float(np.mean(4.0 * r * (1.0 - r)))
    ysym = float(np.abs(r - r[:, ::-1, :]).max())
    return int(ncomp), mnd, ysym


# Active-domain cases (SimpOptions::active_domain_band, simp.cpp:1745-1896): a
# warm-start seed with a thin beam from the clamped face to the loaded edge, so
# that most of the box sits at the density floor and the band excludes it.
def beam_seed(nx, ny, nz, half_width=2, floor=1e-3):
    """Seed density: 1 on a (2*half_width)^2 beam along x through the box centre
    and on a two-voxel plate under the loaded edge (x = nx-2..nx-1, z around the
    middle, every y), `floor` elsewhere."""
    s = np.full((nz, ny, nx), floor)
    zc, yc, w = nz // 2, ny // 2, half_width
    s[zc - w:zc + w, yc - w:yc + w, :] = 1.0
    s[zc - 1:zc + 1, :, nx - 2:] = 1.0
    return s.ravel()


# name: (nx, ny, nz, masked, seed (half_width, floor) or None, band, radius,
#        volfrac, iterations, updater 0 OC / 1 MMA) -- each run at move 0.2,
#        change_tol 0, cg 1e-9.
ACTIVE_DOMAIN_RUNS = {
    "restricted": (32, 16, 16, False, (2, 1e-3), -1, 1.5, 0.05, 20, 0),
    "masked": (32, 16, 16, True, (2, 1e-3), -1, 1.5, 0.05, 10, 0),
    "escape": (24, 12, 12, False, (1, 1e-6), 1, 2.5, 0.1, 10, 0),
    "failed": (16, 6, 6, False, "plate", 1, 1.5, 0.2, 6, 0),
    "latch": (12, 4, 4, False, None, -1, 1.5, 0.3, 12, 0),
    "mma": (32, 16, 16, False, (2, 1e-3), -1, 1.5, 0.05, 15, 1),
}


def active_domain_case(name):
    """(Problem, mask or None, seed or None, band, radius, volfrac, iterations,
    updater) of one ACTIVE_DOMAIN_RUNS entry.  The masked box has a Fixture slab at x = 0,
    Load voxels under the loaded edge, a FrozenVoid keep-out block and a
    FrozenSolid insert on the beam.  The "failed" seed puts material only near
    the clamped face, so band 1 leaves the loaded edge void and the restricted
    system fails the void-load gate."""
    nx, ny, nz, masked, sd, band, radius, vf, its, upd = ACTIVE_DOMAIN_RUNS[name]
    mask = None
    tags = None
    if masked:
        t = np.ones((nz, ny, nx), np.uint8)
        t[:, :, 0] = 5
        t[nz // 2 - 1:nz // 2 + 1, :, nx - 1] = 4
        m = np.zeros((nz, ny, nx), np.uint8)
        m[2:6, 2:6, 10:16] = 2
        m[nz // 2 - 1:nz // 2 + 1, ny // 2 - 1:ny // 2 + 1, 20:24] = 1
        tags, mask = t.ravel(), m.ravel()
    pb = cantilever(nx, ny, nz, solid=tags)
    if sd is None:
        seed = None
    elif sd == "plate":
        seed = np.full((nz, ny, nx), 1e-3)
        seed[:, :, :5] = 1.0
        seed = seed.ravel()
    else:
        seed = beam_seed(nx, ny, nz, sd[0], sd[1])
    return pb, mask, seed, band, radius, vf, its, upd
