"""The on-disk formats (design.bin v1, fields.bin v1, the iterations.csv row)
written by the library byte-identical to the reference's own writers
(design_store.cpp, fields.cpp, IterationCsvWriter::append_at) on the same
inputs.  Host-only entry points: CPU."""
import numpy as np
import pytest

FIELDS = ("total_ms", "tail_prev_ms", "filter_ms", "project_ms", "solve_ms", "fea_ms", "sens_ms",
          "update_ms", "analysis_ms", "observe_ms", "residual_ms", "solver_build_ms",
          "mg_build_ms", "mg_ms", "cg_ms", "geneo_setup_ms", "geneo_apply_ms", "recycle_ms")


def _dims(golden):
    return tuple(int(v) for v in golden["fmt_dims"])


def test_design_file_bytes_match_reference(tg, golden, tmp_path):
    dims = _dims(golden)
    nv = int(np.prod(dims))
    dd, di, dens = golden["fmt_design_d"], golden["fmt_design_i"], golden["fmt_design_dens"]
    variants = []
    for k in range(2):
        variants.append(dict(requested_volume_fraction=dd[k][0], achieved_volume_fraction=dd[k][1],
                             margin_worst_case=dd[k][2], margin_effective=dd[k][3],
                             max_von_mises=dd[k][4], applied_build_dir=tuple(dd[k][5:8]),
                             accepted=di[k][0], iterations=int(di[k][1]),
                             build_direction_auto_applied=di[k][2], export_baked=di[k][3],
                             density=dens[k * nv:(k + 1) * nv]))
    p = tmp_path / "design.bin"
    assert tg.write_design_file(p, dims, variants, float(golden["fmt_spacing"]),
                                tuple(golden["fmt_origin"])) == 2
    assert np.array_equal(np.frombuffer(p.read_bytes(), np.uint8), golden["fmt_design_bytes"])
    assert not (tmp_path / "design.bin.part").exists()
    for k in range(2):
        assert tg.design_fingerprint(dens[k * nv:(k + 1) * nv]) == int(golden["fmt_design_fp"][k])
    back = tg.read_design_file(p)
    assert back["dims"] == dims and back["spacing"] == float(golden["fmt_spacing"])
    for k, v in enumerate(back["variants"]):
        assert np.array_equal(v["density"], dens[k * nv:(k + 1) * nv])
        assert v["iterations"] == int(di[k][1]) and v["accepted"] == di[k][0]
        assert v["fingerprint"] == int(golden["fmt_design_fp"][k])
    # A corrupted density is refused by its fingerprint; a wrong version by its byte.
    raw = bytearray(p.read_bytes())
    raw[-3] ^= 0x10
    (tmp_path / "bad.bin").write_bytes(bytes(raw))
    with pytest.raises(ValueError, match="fingerprint"):
        tg.read_design_file(tmp_path / "bad.bin")
    raw = bytearray(p.read_bytes())
    raw[0] = 2
    (tmp_path / "v2.bin").write_bytes(bytes(raw))
    with pytest.raises(ValueError, match="version"):
        tg.read_design_file(tmp_path / "v2.bin")
    # A header whose voxel count the file cannot hold is refused before any
    # allocation; so is a file cut short inside a variant.
    raw = bytearray(p.read_bytes())
    raw[4:16] = np.array([1 << 20] * 3, "<i4").tobytes()
    (tmp_path / "huge.bin").write_bytes(bytes(raw))
    with pytest.raises(ValueError, match="truncated"):
        tg.read_design_file(tmp_path / "huge.bin")
    (tmp_path / "cut.bin").write_bytes(p.read_bytes()[:-100])
    with pytest.raises(ValueError, match="truncated"):
        tg.read_design_file(tmp_path / "cut.bin")


def test_fields_file_bytes_match_reference(tg, golden, tmp_path):
    dims = _dims(golden)
    nv = int(np.prod(dims))
    nd = 3 * (dims[0] + 1) * (dims[1] + 1) * (dims[2] + 1)
    fd, fi = golden["fmt_fields_d"], golden["fmt_fields_i"]
    vm, disp = golden["fmt_fields_vm"], golden["fmt_fields_disp"]
    variants = [dict(requested_volume_fraction=fd[2 * k], mass_grams=fd[2 * k + 1],
                     support_volume_voxels=int(fi[k]), von_mises=vm[k * nv:(k + 1) * nv],
                     displacement=disp[k * nd:(k + 1) * nd]) for k in range(2)]
    p = tmp_path / "fields.bin"
    assert tg.write_fields_file(p, dims, variants, float(golden["fmt_spacing"]),
                                tuple(golden["fmt_origin"])) == 2
    assert np.array_equal(np.frombuffer(p.read_bytes(), np.uint8), golden["fmt_fields_bytes"])


def test_iteration_csv_matches_reference(tg, golden):
    od, oi, ol = golden["fmt_csv_od"], golden["fmt_csv_oi"], golden["fmt_csv_ol"]
    rec = dict(compliance=od[0], volume_fraction=od[1], beta=od[2], active_fraction=od[3],
               rss_mb=od[22], peak_rss_mb=od[23], compressed_mb=od[24], available_mb=od[25],
               iteration=int(oi[0]), plateau=int(oi[1]), cg_iterations=int(oi[2]),
               cg_multigrid=int(oi[3]), hier_built=int(oi[4]), mg_cycles_attempted=int(oi[5]),
               infeasible=int(oi[6]), recycle_dim=int(oi[7]), geneo_dim=int(oi[8]),
               geneo_action=int(oi[9]), geneo_burn=int(oi[10]), geneo_threshold=int(oi[11]),
               fea_solves=int(ol[0]), matvecs=int(ol[1]), major_faults=int(ol[2]),
               swapins=int(ol[3]))
    rec.update({k: od[4 + q] for q, k in enumerate(FIELDS)})
    text = tg.iteration_csv_header() + "\n" + tg.iteration_csv_row(2, rec, 1733000000123)
    assert text.encode() == golden["fmt_csv_bytes"].tobytes()
