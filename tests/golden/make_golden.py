"""Generate the golden fixtures in tests/golden/ from the reference's OWN code.

Runs the reference's compiled hot path (oracle/_ref/libtopopt_ref.so, built by
oracle/build_ref.sh from the reference tree) on small seeded problems and saves
inputs and outputs as golden.npz.  Only runs where the reference tree is
available; the committed golden.npz is what the tests read everywhere else.

    python tests/golden/make_golden.py                       # everything
    python tests/golden/make_golden.py --section cant60_steps  # one section into the existing file
    python tests/golden/make_golden.py --section homog
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..", "..")))

from oracle.oracle import (ACTIVE_DOMAIN_RUNS, CONTINUATION, GATE_V2, OracleLib,  # noqa: E402
                           Problem, active_domain_case, build_reference, cantilever,
                           gate_v2_problem, reference_path)

REF_KE_JSON = reference_path("core", "tests", "fixtures", "fea", "hex_stiffness_reference.json")
BENCH_JSON = reference_path("core", "tests", "fixtures", "benchmarks.json")


def main():
    if build_reference() is None:
        raise SystemExit("reference tree not available; nothing generated")
    R = OracleLib("reference")
    R.set_threads(int(os.environ.get("GOLDEN_THREADS", "1")))
    rng = np.random.default_rng(20261203)
    out = {}
    # Element stiffness, pinned to the reference's own JSON fixture too.
    for nu in (0.3, 0.4):
        ke = R.hex8_stiffness(1.0, nu, 1.0)
        out[f"ke_nu{int(nu * 100):02d}"] = ke
    ref = json.load(open(REF_KE_JSON))
    for key, case in ref["cases"].items():
        K = np.array(case["K"])
        nu = case["poisson"]
        got = out[f"ke_nu{int(round(nu * 100)):02d}"]
        assert np.abs(got - K).max() <= 1e-10 * np.abs(K).max(), key
    out["ke_h05_E2"] = R.hex8_stiffness(2.0, 0.3, 0.5)

    # Operator apply on a grid with voids, graded and uniform.
    nx, ny, nz = 13, 6, 5
    solid = (rng.random(nx * ny * nz) > 0.15).astype(np.uint8).reshape(nz, ny, nx)
    solid[nz // 2 - 1:nz // 2 + 1, :, nx - 1] = 1  # keep the loaded edge stiff
    solid = solid.ravel()
    pb = cantilever(nx, ny, nz, solid=solid)
    u = rng.standard_normal(pb.ndof)
    fac = rng.random(pb.nv) * 0.99 + 0.01
    out.update(apply_dims=np.array([nx, ny, nz]), apply_solid=solid, apply_u=u, apply_factor=fac,
               apply_y_graded=R.apply(pb, u, fac), apply_y_uniform=R.apply(pb, u, None, E=2.5))

    # Reduced system, void-DOF gate and the exact Jacobi-PCG solve.
    red = R.build_reduced(pb, fac)
    out.update(red_kept=red["kept"], red_rhs=red["rhs"], red_invdiag=red["invdiag"],
               red_ng=np.array(red["ng"]))
    ucg, it, res = R.solve_cg(pb, fac, tol=1e-12)
    out.update(cg_u=ucg, cg_iters=np.array(it), cg_resid=np.array(res))

    # simp_compliance on a graded density (solve at 1e-12).
    pb2 = cantilever(16, 6, 6)
    rho = rng.random(pb2.nv) * 0.95 + 0.05
    c = R.simp_compliance(pb2, rho, tol=1e-12)
    out.update(comp_dims=np.array([16, 6, 6]), comp_rho=rho, comp_u=c["u"], comp_dc=c["dc"],
               comp_c=np.array(c["compliance"]))

    # Density filter, forward and adjoint, r = 1.5 and 2.5, with voids.
    x = rng.random(pb.nv)
    for r in (1.5, 2.5):
        tag = str(r).replace(".", "")
        out[f"filt_x"] = x
        out[f"filt_fwd_r{tag}"] = R.filter(pb, x, r, False)
        out[f"filt_adj_r{tag}"] = R.filter(pb, x, r, True)

    # OC update with the reference's own dc.
    xd = np.where(solid > 0, rng.random(pb.nv) * 0.8 + 0.1, 0.0)
    dc = -np.where(solid > 0, rng.random(pb.nv) * 10.0, 0.0)
    out.update(oc_x=xd, oc_dc=dc, oc_xnew=R.oc_update(pb, xd, dc, 0.3, 1.5, 0.2, 1e-3),
               oc_xnew_r25=R.oc_update(pb, xd, dc, 0.4, 2.5, 0.1, 1e-3))

    # A short simp_optimize run (the reference loop, Jacobi-PCG solves).
    pb3 = cantilever(12, 4, 4)
    s = R.simp_optimize(pb3, volfrac=0.3, radius=1.5, move=0.2, max_it=20, change_tol=0.01,
                        cg_tol=1e-10)
    out.update(simp_dims=np.array([12, 4, 4]), simp_hist_c=s["hist_c"],
               simp_hist_change=s["hist_change"], simp_hist_vf=s["hist_vf"],
               simp_design=s["design"], simp_phys=s["phys"],
               simp_compliance=np.array(s["compliance"]), simp_iterations=np.array(s["iterations"]))

    # Design masks (the masked simp_optimize overload): raw voxel tags with Empty
    # pockets, a Fixture slab at x = 0 and a Load slab at the loaded edge; a
    # mask with FrozenSolid and FrozenVoid islands.
    mx, my, mz = 14, 6, 5
    tags = np.ones((mz, my, mx), np.uint8)
    tags[rng.random((mz, my, mx)) < 0.08] = 0
    tags[:, :, 0] = 5
    tags[mz // 2 - 1:mz // 2 + 1, :, mx - 1] = 4
    tags = tags.ravel()
    mask = np.zeros(mx * my * mz, np.uint8)
    rr = rng.random(mask.size)
    mask[rr < 0.10] = 1
    mask[(rr >= 0.10) & (rr < 0.18)] = 2
    pbm = cantilever(mx, my, mz, solid=tags)
    xm = rng.random(pbm.nv)
    out.update(mask_dims=np.array([mx, my, mz]), mask_tags=tags, mask_mask=mask,
               mask_eff=R.effective_design_mask(pbm, mask), mask_x=xm,
               mask_filt_fwd=R.filter_masked(pbm, mask, xm, 1.5, False),
               mask_filt_adj=R.filter_masked(pbm, mask, xm, 1.5, True))
    sm = R.simp_optimize_masked(pbm, mask, volfrac=0.35, radius=1.5, move=0.2, max_it=15,
                                change_tol=0.01, cg_tol=1e-10)
    out.update(msimp_hist_c=sm["hist_c"], msimp_hist_change=sm["hist_change"],
               msimp_hist_vf=sm["hist_vf"], msimp_design=sm["design"], msimp_phys=sm["phys"],
               msimp_compliance=np.array(sm["compliance"]),
               msimp_volume_fraction=np.array(sm["volume_fraction"]),
               msimp_iterations=np.array(sm["iterations"]))

    # The reference's CPU-runnable configuration: 60x20x20 cantilever, volume
    # fraction 0.3, rmin 1.5, move 0.2, 50 design iterations (change_tol 0 so all
    # 50 run), solves at 1e-10.
    pb0 = cantilever(60, 20, 20)
    s0 = R.simp_optimize(pb0, volfrac=0.3, radius=1.5, move=0.2, max_it=50, change_tol=0.0,
                         cg_tol=1e-10)
    out.update(cant60_hist_c=s0["hist_c"], cant60_hist_change=s0["hist_change"],
               cant60_hist_vf=s0["hist_vf"], cant60_design=s0["design"],
               cant60_compliance=np.array(s0["compliance"]),
               cant60_iterations=np.array(s0["iterations"]))
    out.update(_cant60_steps(R))
    out.update(_homog(R))

    # Heaviside projection: value and derivative at the fixture's spot values
    # and on a dense grid of rho_tilde, from the reference's own functions.
    rts = np.concatenate([[0.0, 0.3, 0.5, 0.7, 1.0], np.linspace(0.0, 1.0, 41)])
    betas = np.array([1.0, 2.0, 4.0, 8.0, 16.0, 32.0, 64.0])
    pv = np.zeros((betas.size, rts.size))
    pd = np.zeros_like(pv)
    for i, b in enumerate(betas):
        for j, rt in enumerate(rts):
            pv[i, j], pd[i, j] = R.project(float(rt), float(b), 0.5)
    out.update(proj_rt=rts, proj_beta=betas, proj_value=pv, proj_deriv=pd)
    bench = json.load(open(BENCH_JSON))
    unit = bench["projection_unit_reference"]
    for b in (1, 8, 32):
        for rt in ("0.0", "0.3", "0.5", "0.7", "1.0"):
            spot = unit[f"beta_{b}"][f"rt_{rt}"]
            v, d = R.project(float(rt), float(b), 0.5)
            assert abs(v - spot["value"]) <= 1e-12 * max(abs(spot["value"]), 1e-300) + \
                (1e-12 if spot["value"] == 0.0 else 0.0), (b, rt)
            assert abs(d - spot["derivative"]) <= 1e-12 * abs(spot["derivative"]), (b, rt)

    # A short projected run (three continuation stages) on the 12x4x4 cantilever.
    pstages = [(1.0, 0.2, 8), (4.0, 0.2, 8), (16.0, 0.1, 6)]
    sp = R.simp_optimize(pb3, volfrac=0.3, radius=1.5, change_tol=0.0, cg_tol=1e-10,
                         stages=pstages)
    out.update(psimp_stages=np.array(pstages), psimp_hist_c=sp["hist_c"],
               psimp_hist_change=sp["hist_change"], psimp_hist_vf=sp["hist_vf"],
               psimp_design=sp["design"], psimp_phys=sp["phys"],
               psimp_compliance=np.array(sp["compliance"]),
               psimp_volume_fraction=np.array(sp["volume_fraction"]),
               psimp_iterations=np.array(sp["iterations"]))

    # Gate V2: the two benchmark problems under the locked projected formulation,
    # run by the reference (300 iterations), and the fixture's gates.
    for name in GATE_V2:
        key = "gv2c" if name.startswith("cantilever") else "gv2b"
        g = gate_v2_problem(name)
        r = R.simp_optimize(g, volfrac=0.3, radius=2.5, change_tol=0.0, cg_tol=1e-9,
                            stages=CONTINUATION)
        b = bench["benchmarks"][name]
        ref, gates = b["reference"], b["gates"]
        se = ref["stage_end_compliance"]
        band = gates.get("final_analysis_compliance_band")
        final = gates.get("final_analysis_compliance")
        out.update({
            f"{key}_hist_c": r["hist_c"], f"{key}_hist_change": r["hist_change"],
            f"{key}_design": r["design"], f"{key}_phys": r["phys"],
            f"{key}_compliance": np.array(r["compliance"]),
            f"{key}_volume_fraction": np.array(r["volume_fraction"]),
            f"{key}_fix_stage_end": np.array([se[k] for k in ("1", "2", "4", "8", "16", "32")]),
            f"{key}_fix_final": np.array(ref["final_analysis_compliance"]),
            f"{key}_fix_vf": np.array(ref["achieved_projected_volume_fraction"]),
            f"{key}_gate_rel": np.array([gates["stage_end_compliance_beta_1"]["rel_tolerance"],
                                         gates["stage_end_compliance_beta_8"]["rel_tolerance"]]),
            f"{key}_gate_final": np.array(band if band else
                                          [final["value"], final["rel_tolerance"]]),
            f"{key}_gate_final_is_band": np.array(band is not None),
            f"{key}_gate_vf_abs": np.array(gates["achieved_projected_volume_fraction_abs_tolerance"]),
            f"{key}_gate_components": np.array(gates["connected_components_at_0p5"]),
            f"{key}_gate_ysym": np.array(gates["y_symmetry_error_max"]),
            f"{key}_gate_mnd": np.array(gates["discreteness_Mnd_max"]),
        })

    # Element stress (hex8_stress) at the centre and at random natural points.
    ues = rng.standard_normal((8, 24))
    mats = np.column_stack([rng.uniform(0.5, 3.0, 8), rng.uniform(0.0, 0.45, 8),
                            rng.uniform(0.3, 2.0, 8)])
    pts = np.vstack([np.zeros((4, 3)), rng.uniform(-1.0, 1.0, (4, 3))])
    sig = np.zeros((8, 6))
    vms = np.zeros(8)
    for q in range(8):
        sig[q], vms[q] = R.hex8_stress(*mats[q], ues[q], *pts[q])
    out.update(stress_ue=ues, stress_mat=mats, stress_pts=pts, stress_sigma=sig, stress_vm=vms)

    # The ladder walk and the fixed-design analysis on a tagged bracket: a
    # Fixture slab at x = 0, Load voxels at the loaded tip edge.
    lx, ly, lz = 20, 6, 8
    ltags = np.ones((lz, ly, lx), np.uint8)
    ltags[:, :, 0] = 5
    ltags[lz // 2 - 1:lz // 2 + 1, :, lx - 1] = 4
    ltags = ltags.ravel()
    pbl = cantilever(lx, ly, lz, solid=ltags)
    lad = [0.6, 0.45, 0.3, 0.2, 0.12]
    for tag, ms in (("a", 1.0), ("b", 25.0)):
        L = R.ladder(pbl, None, lad, max_it=25, yield_strength=30.0, margin_stop=ms, cg_tol=1e-9)
        out[f"lad{tag}_rung_d"] = np.array([[r["volume_fraction"], r["compliance"],
                                             r["analysis"]["max_von_mises"],
                                             r["analysis"]["max_interlayer"],
                                             r["analysis"]["margin_worst"],
                                             r["analysis"]["margin_effective"]]
                                            for r in L["rungs"]])
        out[f"lad{tag}_rung_i"] = np.array([[r["iterations"], r["trajectory_ok"], r["analysed"],
                                             r["accepted"], r["analysis"]["load_path_ok"]]
                                            for r in L["rungs"]])
        out[f"lad{tag}_out"] = np.array([L["evaluated"], L["recommended"],
                                         int(L["stopped_on_margin"])])
        out[f"lad{tag}_design"] = L["design"]
        out[f"lad{tag}_phys"] = L["phys"]
    out.update(lad_dims=np.array([lx, ly, lz]), lad_tags=ltags, lad_ladder=np.array(lad))
    dfix = out["lada_phys"]
    an, vmf = R.analyze_fixed_design(pbl, dfix, yield_strength=30.0, margin_stop=25.0,
                                     build_dir=(0.3, -0.2, 0.9), cg_tol=1e-10)
    out.update(ana_density=dfix, ana_vm=vmf,
               ana_d=np.array([an["compliance"], an["max_von_mises"], an["max_interlayer"],
                               an["margin_in_plane"], an["margin_interlayer"],
                               an["margin_worst"]]),
               ana_i=np.array([an["printed_voxels"], an["load_path_ok"], an["accepted"]]))
    # Load-path belt on a severed copy (the x = 10 slab carved away).
    sev = dfix.reshape(lz, ly, lx).copy()
    sev[:, :, 10] = 0.0
    out["lp_connected"] = np.array([R.load_path_connected(pbl, dfix),
                                    R.load_path_connected(pbl, sev.ravel())])

    # The MMA updater: a plateau-stopped plain run and a masked run.
    mp = R.simp_optimize_mma(pb3, max_it=200, cg_tol=1e-10)
    out.update(mma_hist_c=mp["hist_c"], mma_hist_change=mp["hist_change"],
               mma_hist_vf=mp["hist_vf"], mma_design=mp["design"], mma_phys=mp["phys"],
               mma_compliance=np.array(mp["compliance"]),
               mma_out=np.array([mp["iterations"], int(mp["converged"])]))
    mm = R.simp_optimize_mma(pbm, mask=mask, volfrac=0.35, max_it=40, cg_tol=1e-10)
    out.update(mmam_hist_c=mm["hist_c"], mmam_hist_change=mm["hist_change"],
               mmam_design=mm["design"], mmam_phys=mm["phys"],
               mmam_compliance=np.array(mm["compliance"]),
               mmam_volume_fraction=np.array(mm["volume_fraction"]))

    # On-disk formats, written by the reference's own writers.
    out.update(_formats(R, rng))

    # The active domain: masks and escape counts on a tagged grid, the auto band,
    # and armed runs covering each posture (restricted throughout, masked, the
    # escape latch, a failed restricted solve, the fraction latch).
    out.update(_active_domain(R, rng))

    old = os.path.join(HERE, "golden.npz")
    if os.path.exists(old):  # regenerating must not move any earlier vector
        with np.load(old) as z:
            for k in z.files:
                if k not in out:
                    continue
                same = (np.array_equal(z[k], out[k], equal_nan=True)
                        if np.issubdtype(z[k].dtype, np.floating) else np.array_equal(z[k], out[k]))
                if not same:
                    raise SystemExit(f"golden array {k} changed on regeneration")
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    print("wrote", os.path.join(HERE, "golden.npz"), len(out), "arrays")


def _cant60_steps(R):
    """Per-step inputs of the 60x20x20 configuration: the reference's physical
    density after 10, 25 and 50 design iterations (its own OC trajectory,
    filtered by its own filter) and its compliance, displacement and
    sensitivities on exactly that density, solved to 1e-12."""
    pb0 = cantilever(60, 20, 20)
    out = {}
    for k in (10, 25, 50):
        sk = R.simp_optimize(pb0, volfrac=0.3, radius=1.5, move=0.2, max_it=k, change_tol=0.0,
                             cg_tol=1e-10)
        xp = R.filter(pb0, sk["design"], 1.5)
        ck = R.simp_compliance(pb0, xp, tol=1e-12)
        out.update({f"cant60_it{k}_phys": xp, f"cant60_it{k}_c": np.array(ck["compliance"]),
                    f"cant60_it{k}_u": ck["u"], f"cant60_it{k}_dc": ck["dc"]})
    return out


def _homog_reference_operator(R, kind, vpc, rho, tol=1e-12):
    """C^H of one periodic unit cell with the reference's own compiled operator.

    The harness (core/tests/harness/lattice_homog_probe.cpp:290-412) assembles
    the periodic stiffness with Eigen, which is absent here; its operator is
    rebuilt from the reference's Eigen-free fea_matfree_apply on the
    (vpc+1)^3-node grid of the same cell:
      * periodic apply: torus values unfolded onto the grid (node vpc = node 0
        on every axis), the reference's apply, results folded back (wrapped
        nodes summed);
      * F_J: the apply of the global linear field of unit strain J -- on every
        element it differs from the harness's element-local chi0_J by a rigid
        translation, which Ke maps to zero;
      * node 0 and untouched DOFs pinned (identity rows), Jacobi-PCG to `tol`;
      * C^H_IJ = D_I . K D_J / |Y| with D_J = (linear field J) - unfold(chi_J),
        the harness's element sum of (chi0 - chi_e)^T ke (chi0 - chi_e).
    """
    from topopt_gb300 import lattice
    n = vpc
    cell = lattice.cell(kind, n, lattice.calibrate(kind, n, rho)).astype(np.uint8).ravel()
    pb = Problem(n, n, n, 1.0, cell)
    nn = n + 1
    idx = np.arange(nn)
    tor = (idx % n)
    cz, cy, cx = np.meshgrid(tor, tor, tor, indexing="ij")
    g2t = ((cz * n + cy) * n + cx).ravel()  # grid node -> torus node

    def unfold(v):
        return v.reshape(-1, 3)[g2t].ravel()

    def fold(v):
        out = np.zeros((n ** 3, 3))
        np.add.at(out, g2t, v.reshape(-1, 3))
        return out.ravel()

    def kfull(u):
        return R.apply(pb, u, None, E=1.0)

    z, y, x = np.meshgrid(idx, idx, idx, indexing="ij")
    X, Y, Z = x.ravel().astype(float), y.ravel().astype(float), z.ravel().astype(float)
    lin = []
    for J in range(6):  # the harness's chi0 columns: xx, yy, zz, xy, yz, zx
        u = np.zeros((nn ** 3, 3))
        if J == 0: u[:, 0] = X
        if J == 1: u[:, 1] = Y
        if J == 2: u[:, 2] = Z
        if J == 3: u[:, 0] = Y
        if J == 4: u[:, 1] = Z
        if J == 5: u[:, 2] = X
        lin.append(u.ravel())
    # touched DOFs and the Jacobi diagonal (uniform modulus: every diagonal entry of Ke equal)
    ke = R.hex8_stiffness(1.0, 0.3, 1.0).reshape(24, 24)
    cnt = np.zeros(n ** 3)
    c3 = cell.reshape(n, n, n)
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                cnt += np.roll(np.roll(np.roll(c3, dz, 0), dy, 1), dx, 2).ravel()
    diag = np.repeat(cnt * ke[0, 0], 3)
    pinned = np.repeat(cnt == 0, 3)
    pinned[:3] = True
    inv = np.where(pinned, 1.0, 1.0 / np.where(diag > 0, diag, 1.0))

    def kper(v):
        w = np.where(pinned, 0.0, v)
        out = fold(kfull(unfold(w)))
        return np.where(pinned, v, out)

    chis = []
    for J in range(6):
        b = np.where(pinned, 0.0, fold(kfull(lin[J])))
        xk = np.zeros_like(b)
        r = b.copy()
        bn2 = b @ b
        z_ = inv * r
        p = z_.copy()
        rz = r @ z_
        for _ in range(200000):
            if r @ r <= tol * tol * bn2:
                break
            q = kper(p)
            a = rz / (p @ q)
            xk += a * p
            r -= a * q
            z_ = inv * r
            rzn = r @ z_
            p = z_ + (rzn / rz) * p
            rz = rzn
        chis.append(xk)
    D = [lin[J] - unfold(chis[J]) for J in range(6)]
    KD = [kfull(d) for d in D]
    CH = np.array([[D[I] @ KD[J] for J in range(6)] for I in range(6)]) / float(n ** 3)
    return cell, CH


def _homog(R):
    out = {}
    for kind, vpc, rho in (("gyroid", 12, 0.3), ("octet", 12, 0.25)):
        cell, CH = _homog_reference_operator(R, kind, vpc, rho)
        out[f"homog_{kind}_cell"] = cell
        out[f"homog_{kind}_CH"] = CH
    return out


def update_section(name):
    """Recompute one section into the existing golden.npz (every other array is
    kept as it is)."""
    if build_reference() is None:
        raise SystemExit("reference tree not available; nothing generated")
    R = OracleLib("reference")
    R.set_threads(int(os.environ.get("GOLDEN_THREADS", "1")))
    path = os.path.join(HERE, "golden.npz")
    with np.load(path) as z:
        out = {k: z[k] for k in z.files}
    new = {"cant60_steps": _cant60_steps, "homog": _homog}[name](R)
    for k, v in new.items():
        if k in out and not np.array_equal(out[k], v, equal_nan=True):
            raise SystemExit(f"golden array {k} changed on regeneration")
    out.update(new)
    np.savez_compressed(path, **out)
    print("updated", path, sorted(new))


def _formats(R, rng):
    import ctypes as C
    import tempfile
    L = R.lib
    dp = np.ctypeslib.ndpointer(np.float64, flags="C")
    ip = np.ctypeslib.ndpointer(np.int32, flags="C")
    lp = np.ctypeslib.ndpointer(np.int64, flags="C")
    L.ref_write_design_file.argtypes = [C.c_char_p] + [C.c_int] * 3 + [dp, C.c_double, C.c_int,
                                                                      dp, ip, dp]
    L.ref_write_fields_file.argtypes = [C.c_char_p] + [C.c_int] * 3 + [dp, C.c_double, C.c_int,
                                                                      dp, ip, dp, dp]
    L.ref_iteration_csv.argtypes = [C.c_char_p, C.c_longlong, dp, ip, lp, C.c_longlong]
    L.ref_design_fingerprint.argtypes = [dp, C.c_longlong]
    L.ref_design_fingerprint.restype = C.c_uint64
    nx, ny, nz, h = 5, 4, 3, 0.8
    origin = np.array([1.5, -2.0, 0.25])
    nv, nd = nx * ny * nz, 3 * (nx + 1) * (ny + 1) * (nz + 1)
    dd = np.array([[0.6, 0.6012, 2.25, 2.0, 13.75, 0.0, 0.6, 0.8],
                   [0.45, 0.4497, 1.1, 0.9, 27.5, 0.0, 0.0, 1.0]])
    di = np.array([[1, 40, 0, 1], [0, 37, 1, 0]], np.int32)
    dens = rng.random(2 * nv)
    fd = np.array([0.6, 12.5, 0.45, 9.25])
    fi = np.array([17, 3], np.int32)
    vm = rng.random(2 * nv) * 40.0
    disp = rng.standard_normal(2 * nd) * 1e-3
    od = np.concatenate([[1234.5678901234, 0.3012345, 4.0, 0.875], rng.random(18) * 100.0,
                         [512.25, 600.5, -1.0, 8000.125]])
    oi = np.array([7, 0, 42, 1, 1, 9, 0, 0, 0, 0, 0, 0], np.int32)
    ol = np.array([1, 130, -1, 3], np.int64)
    with tempfile.TemporaryDirectory() as tmp:
        pd, pf, pc = (os.path.join(tmp, n) for n in ("design.bin", "fields.bin", "it.csv"))
        assert L.ref_write_design_file(pd.encode(), nx, ny, nz, origin, h, 2, dd.ravel(),
                                       di.ravel(), dens) == 0
        assert L.ref_write_fields_file(pf.encode(), nx, ny, nz, origin, h, 2, fd, fi, vm,
                                       disp) == 0
        assert L.ref_iteration_csv(pc.encode(), 2, od, oi, ol, 1733000000123) == 0
        bd, bf, bc = (np.frombuffer(open(q, "rb").read(), np.uint8) for q in (pd, pf, pc))
    return dict(fmt_dims=np.array([nx, ny, nz]), fmt_spacing=np.array(h), fmt_origin=origin,
                fmt_design_d=dd, fmt_design_i=di, fmt_design_dens=dens,
                fmt_design_bytes=bd, fmt_design_fp=np.array(
                    [L.ref_design_fingerprint(dens[:nv].copy(), nv),
                     L.ref_design_fingerprint(dens[nv:].copy(), nv)], np.uint64),
                fmt_fields_d=fd, fmt_fields_i=fi, fmt_fields_vm=vm, fmt_fields_disp=disp,
                fmt_fields_bytes=bf, fmt_csv_od=od, fmt_csv_oi=oi, fmt_csv_ol=ol,
                fmt_csv_bytes=bc)


def _active_domain(R, rng):
    out = {}
    nx, ny, nz = 11, 7, 5
    tags = rng.choice(np.array([0, 1, 1, 1, 2, 4, 5], np.uint8), nx * ny * nz)
    pb = Problem(nx, ny, nz, 1.0, tags)
    rho = np.where(rng.random(pb.nv) < 0.1, rng.random(pb.nv), 1e-3)
    rho[rng.random(pb.nv) < 0.03] = 1.5e-3  # on the core threshold: not core
    bands = np.array([0, 1, 2, 3, 64])
    prev = (rng.random(pb.nv) < 0.5).astype(np.uint8)
    radii = np.array([0.0, -1.0, 1.0, 1.2, 1.5, 2.5, 3.0, np.nan, np.inf])
    out.update(ad_dims=np.array([nx, ny, nz]), ad_tags=tags, ad_rho=rho, ad_bands=bands,
               ad_masks=np.stack([R.active_domain_mask(pb, rho, 1e-3, int(b)) for b in bands]),
               ad_prev=prev, ad_escapes=np.array(R.active_domain_escape_count(pb, rho, prev, 1e-3)),
               ad_radii=radii,
               ad_auto=np.array([R.active_domain_auto_band(float(r)) for r in radii]))
    for name in ACTIVE_DOMAIN_RUNS:
        pbr, mask, seed, band, radius, vf, its, upd = active_domain_case(name)
        r = R.simp_optimize_active(pbr, band, mask=mask, seed=seed, radius=radius, volfrac=vf,
                                   move=0.2, max_it=its, change_tol=0.0, cg_tol=1e-9,
                                   updater=upd)
        k = "adr_" + name
        out[k + "_hist_c"] = r["hist_c"]
        out[k + "_hist_af"] = r["hist_af"]
        out[k + "_phys"] = r["phys"]
        out[k + "_d"] = np.array([r["compliance"], r["volume_fraction"], r["fraction_mean"]])
        out[k + "_i"] = np.array([r["iterations"], r["band"], int(r["latched"]),
                                  r["latch_iteration"], r["escape_count"]])
        out[k + "_reason"] = np.frombuffer(r["reason"].encode(), np.uint8)
    return out


if __name__ == "__main__":
    if len(sys.argv) > 2 and sys.argv[1] == "--section":
        update_section(sys.argv[2])
    else:
        main()
