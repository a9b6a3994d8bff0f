"""Output writers (gb300kf_io.h, gpukalmanfitter_gb300.writer) against the
restatement of the reference driver's writers (oracle/writers.py,
Run/Common/Writer.hpp): byte-identical files on oracle fits of a ragged
telescope (holes, outliers, short tracks, failed tracks), the params table
read back against the fit, and the error paths.  CPU only: the writers are
host code."""
import numpy as np
import pytest

import gpukalmanfitter_gb300 as kfpkg
from gpukalmanfitter_gb300 import writer

DIAG = [0, 6, 11, 15, 18, 20]


@pytest.fixture(scope="module")
def fitted(kf, orc):
    tel = kf.make_telescope(300, seed=77, hit_prob=0.85, outlier_prob=0.05, min_len=6,
                            max_len=10, mis_shift=0.05, mis_rot=5e-4)
    res = orc.fit(tel, kf.default_config(overstep_limit=0.1), threads=0, smoothed=True)
    res = dict(res)
    status = res["status"].copy()
    status[[3, 17, 18, 299]] = 3  # failed fits are skipped by every writer
    res["status"] = status
    return tel, res


def test_params_csv_matches_reference_writer(tmp_path, fitted):
    from oracle import writers as ow
    tel, res = fitted
    p = tmp_path / "params.csv"
    writer.write_params_csv(p, res)
    text = p.read_text()
    assert text == ow.params_csv(res["params"], res["status"])
    lines = text.splitlines()
    assert lines[0].startswith("trackIdx, fit_BoundLoc0,")
    assert len(lines) == 1 + int(np.sum(res["status"] == 0))
    assert not any(l.startswith("3,") or l.startswith("17,") for l in lines[1:])


def test_states_obj_matches_reference_writer(tmp_path, fitted):
    from oracle import writers as ow
    tel, res = fitted
    p = tmp_path / "states.obj"
    writer.write_states_obj(p, res, tel)
    text = p.read_text()
    ref = ow.states_obj(res["smoothed"], res["n_meas"], tel.hit_mask, res["status"],
                        tel.center, tel.rotation)
    assert text == ref
    nv = sum(1 for l in text.splitlines() if l.startswith("v "))
    ok = res["status"] == 0
    assert nv == int(res["n_meas"][ok].sum())
    # every line joins two vertices of the same track
    nl = sum(1 for l in text.splitlines() if l.startswith("l "))
    assert nl == int((res["n_meas"][ok] - 1).sum())
    # the vertices lie on their planes: x of plane k is x_first + k x_step
    xs = np.array([float(l.split()[1]) for l in text.splitlines() if l.startswith("v ")])
    planes = (tel.center[:, 0])
    assert np.all(np.min(np.abs(xs[:, None] - planes[None, :]), axis=1) < 1e-3 * np.abs(xs).max())


def test_sim_hits_obj_matches_reference_writer(tmp_path, fitted):
    from oracle import writers as ow
    tel, _ = fitted
    p = tmp_path / "hits.obj"
    writer.write_sim_hits_obj(p, tel)
    assert p.read_text() == ow.sim_hits_obj(writer.measurement_positions(tel), tel.hit_mask)


def test_obj_counter_with_an_empty_track(tmp_path, kf):
    """A track without hits still advances the reference's vertex counter
    (Writer.hpp:28-38), so the next track's line starts one further on."""
    from oracle import writers as ow
    pos = np.arange(3 * 3 * 3, dtype=np.float64).reshape(3, 3, 3)
    mask = np.array([0b111, 0, 0b101], dtype=np.uint64)
    p = tmp_path / "h.obj"
    kfpkg._check(writer._lib().kf_write_hits_obj(bytes(p), pos.ctypes.data, mask.ctypes.data,
                                                 None, 3, 3, 3))
    text = p.read_text()
    assert text == ow.sim_hits_obj(pos, mask)
    assert [l for l in text.splitlines() if l.startswith("l ")] == ["l 1 2", "l 2 3", "l 5 6"]


def test_params_table_matches_reference_writer(tmp_path, fitted):
    from oracle import writers as ow
    tel, res = fitted
    p = tmp_path / "table.csv"
    writer.write_params_table(p, res, tel)
    text = p.read_text()
    assert text == ow.params_table(res["params"], res["cov"], res["status"], tel.truth,
                                   tel.perigee)
    t = ow.read_table(p)
    ok = res["status"] == 0
    assert list(t.dtype.names) == ow.TABLE_COLUMNS
    assert len(t) == int(ok.sum())
    # the columns carry the fit, its errors and pulls (to print precision)
    assert np.allclose(t["eQOP_fit"], res["params"][4, ok], rtol=1e-5)
    assert np.allclose(t["err_eLOC0_fit"], np.sqrt(res["cov"][0, ok]), rtol=1e-5)
    pull = (res["params"][0, ok] - tel.truth[0, ok]) / np.sqrt(res["cov"][0, ok])
    assert np.allclose(t["pull_eLOC0"], pull, rtol=1e-4, atol=1e-5)
    assert np.all(np.abs(t["t_charge"]) == 1)
    assert np.allclose(t["t_vx"], tel.perigee[0, ok], atol=1e-5)


def test_writer_errors(tmp_path, fitted):
    tel, res = fitted
    with pytest.raises(kfpkg.KfError, match="cannot open"):
        writer.write_params_csv(tmp_path / "missing_dir" / "p.csv", res)
    lib = writer._lib()
    assert lib.kf_write_params_csv(b"x.csv", None, None, 1, 1) == -1
    st = np.zeros(4, dtype=np.int32)
    pr = np.zeros((6, 4))
    assert lib.kf_write_params_csv(bytes(tmp_path / "p.csv"), pr.ctypes.data, st.ctypes.data,
                                   4, 3) == -1  # stride < n
    assert lib.kf_write_hits_obj(bytes(tmp_path / "h.obj"), pr.ctypes.data, None, None, 0, 1,
                                 1) == -1


def test_large_file_is_chunk_independent(tmp_path, kf):
    """More tracks than one formatting chunk: the parallel writer's output
    equals the sequential restatement."""
    from oracle import writers as ow
    n = 20000
    rng = np.random.default_rng(3)
    params = rng.normal(size=(6, n))
    status = (rng.random(n) < 0.9).astype(np.int32) * 0
    status[rng.random(n) < 0.1] = 1
    p = tmp_path / "p.csv"
    writer.write_params_csv(p, {"params": params, "status": status})
    assert p.read_text() == ow.params_csv(params, status)


def test_resolution_report(tmp_path, kf, orc):
    """Pull fits of perigeeParamResolution.C on a written table: unit widths
    for the fitted parameters (10 planes, no material, 2000 tracks)."""
    pytest.importorskip("scipy")
    tel = kf.make_telescope(2000, seed=31)
    res = orc.fit(tel, kf.default_config(overstep_limit=0.1), threads=0)
    p = tmp_path / "t.csv"
    writer.write_params_table(p, res, tel)
    rep = writer.resolution_report(writer.read_params_table(p))
    for name in ("eLOC0", "eLOC1", "ePHI", "eTHETA", "eQOP"):
        assert rep[name]["pull"]["entries"] > 1900
        assert abs(rep[name]["pull"]["mean"]) < 0.1, (name, rep[name])
        assert 0.9 < rep[name]["pull"]["sigma"] < 1.1, (name, rep[name])
    assert rep["eLOC0"]["residual_rms"] < 0.1


def test_empty_and_all_failed(tmp_path, kf):
    """No tracks, or no fitted track: the CSV files hold their header only,
    the obj files are empty (the reference writes the header and skips every
    unsuccessful fit)."""
    from oracle import writers as ow
    for n in (0, 5):
        res = {"params": np.zeros((6, n)), "cov": np.ones((21, n)),
               "status": np.full(n, 3, dtype=np.int32), "n_meas": np.zeros(n, dtype=np.int32),
               "smoothed": np.zeros((10, 27, n))}
        tel = kf.make_telescope(max(n, 1), seed=1)
        if n == 0:
            tel.hit_mask = tel.hit_mask[:0]
            tel.truth = np.zeros((6, 0))
            tel.perigee = np.zeros((3, 0))
        p = tmp_path / f"p{n}.csv"
        writer.write_params_csv(p, res)
        assert p.read_text() == ow.params_csv(res["params"], res["status"])
        assert p.read_text().count("\n") == 1
        o = tmp_path / f"s{n}.obj"
        writer.write_states_obj(o, res, tel)
        assert o.read_text() == ""
        t = tmp_path / f"t{n}.csv"
        writer.write_params_table(t, res, tel)
        assert t.read_text().count("\n") == 1
