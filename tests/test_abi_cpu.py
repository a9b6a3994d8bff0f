"""CPU tests of the C ABI library: it loads, exports every declared symbol,
validates arguments without touching a GPU, and its input generator is
deterministic."""
import ctypes as C
import re
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    names = set()
    for h in sorted((ROOT / "include").glob("*.h")):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(kf_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol(kf):
    lib = kf.load()
    names = declared_functions()
    assert {"kf_fit_batch", "kf_fit_batch_host", "kf_workspace_size"} <= names
    for n in sorted(names):
        assert hasattr(lib, n), f"{n} declared in include/*.h but not exported"


def test_version_and_defaults(kf):
    lib = kf.load()
    assert lib.kf_version() == 1
    cfg = kf.default_config()
    assert cfg.max_steps == 1000 and cfg.max_rk_trials == 10000
    assert cfg.tolerance == 1e-4 and cfg.overstep_limit == 0.01
    assert abs(cfg.mass - 0.1056583755) < 1e-12
    assert cfg.faithful_jacobian == 1 and cfg.smoothing == 1


def test_workspace_size(kf):
    lib = kf.load()
    cfg = kf.default_config()
    assert lib.kf_workspace_size(C.byref(cfg), 1000, 10) == 10 * 37 * 1000 * 8
    assert lib.kf_workspace_size(C.byref(cfg), 0, 10) == 0
    assert lib.kf_host_staging_size(C.byref(cfg), 1000, 10, 0) > 10 * 37 * 1000 * 8


def test_adjoint_workspace_and_tape_mode(kf):
    lib = kf.load()
    taped = kf.default_config()
    segments = kf.default_config(adjoint_tape=1)
    w0 = lib.kf_adjoint_workspace_size(C.byref(taped), 1000, 20)
    w1 = lib.kf_adjoint_workspace_size(C.byref(segments), 1000, 20)
    # the whole-track tape holds 256 doubles a surface, the segment mode 3072
    assert w0 - w1 == (20 * 256 - 3072) * 1000 * 8
    assert lib.kf_adjoint_workspace_size(None, 1000, 20) == w0
    assert lib.kf_adjoint_workspace_size(C.byref(taped), 0, 20) == 0
    # an unknown tape mode is refused before any device work
    tel = kf.make_telescope(4, n_planes=20, x_first=50., x_step=50.)
    geo, keep = tel.geometry()
    fld = tel.field()
    ins = kf.KfInputs()
    ins.n_tracks, ins.stride, ins.n_surfaces = 4, 4, 20
    arr = [np.zeros(8) for _ in range(8)]
    ins.meas, ins.start_params, ins.start_cov, ins.perigee = (a.ctypes.data for a in arr[:4])
    outs = kf.KfAdjointOutputs(*(a.ctypes.data for a in arr[4:8]), None, None, None)
    bad = kf.default_config(adjoint_tape=2)
    assert lib.kf_adjoint_batch(C.byref(ins), C.byref(outs), C.byref(bad), C.byref(geo),
                                C.byref(fld), 1, None, 0, None) == -1
    assert b"adjoint_tape" in lib.kf_last_error_string()


def test_argument_validation_without_gpu(kf):
    lib = kf.load()
    cfg = kf.default_config()
    tel = kf.make_telescope(4)
    geo, keep = tel.geometry()
    fld = tel.field()
    ins = kf.KfInputs()
    ins.n_tracks, ins.stride, ins.n_surfaces = 4, 4, 10
    outs = kf.KfOutputs()
    # null inputs, bad surfaces, bad stride, missing outputs, small workspace
    assert lib.kf_fit_batch(None, C.byref(outs), C.byref(cfg), C.byref(geo), C.byref(fld), None,
                            0, None) == -1
    bad = kf.KfInputs(); bad.n_tracks, bad.stride, bad.n_surfaces = 4, 4, 65
    assert lib.kf_fit_batch(C.byref(bad), C.byref(outs), C.byref(cfg), C.byref(geo),
                            C.byref(fld), None, 0, None) == -1
    bad.n_surfaces, bad.stride = 10, 2
    assert lib.kf_fit_batch(C.byref(bad), C.byref(outs), C.byref(cfg), C.byref(geo),
                            C.byref(fld), None, 0, None) == -1
    assert lib.kf_fit_batch(C.byref(ins), C.byref(outs), C.byref(cfg), C.byref(geo),
                            C.byref(fld), None, 0, None) == -1
    assert b"output" in lib.kf_last_error_string()
    cfg2 = kf.default_config(precision=7)
    assert lib.kf_fit_batch(C.byref(ins), C.byref(outs), C.byref(cfg2), C.byref(geo),
                            C.byref(fld), None, 0, None) == -4


def test_generator_deterministic_and_thread_independent(kf):
    a = kf.make_telescope(3000, threads=1, hit_prob=0.9, outlier_prob=0.02, n_planes=30,
                          min_len=5, max_len=30, x_first=50., x_step=50.)
    b = kf.make_telescope(3000, threads=8, hit_prob=0.9, outlier_prob=0.02, n_planes=30,
                          min_len=5, max_len=30, x_first=50., x_step=50.)
    for k in ("meas", "hit_mask", "n_planes", "start", "start_cov", "perigee", "truth"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
    c = kf.make_telescope(3000, seed=7, hit_prob=0.9, outlier_prob=0.02, n_planes=30,
                          min_len=5, max_len=30, x_first=50., x_step=50.)
    assert not np.array_equal(a.meas, c.meas)


def test_generator_distributions(kf):
    tel = kf.make_telescope(20000)
    p = 1 / np.abs(tel.truth[4])
    assert 1.0 <= p.min() and p.max() <= 10.0
    assert np.all(np.abs(tel.truth[2]) <= 0.1)
    assert np.all(np.abs(tel.truth[3] - np.pi / 2) <= 0.1)
    assert abs(np.mean(tel.truth[4] > 0) - 0.5) < 0.02
    assert abs(tel.perigee[1].std() - 0.020) < 0.001
    dq = tel.start[4] / tel.truth[4] - 1
    assert abs(dq.std() - 0.05) < 0.002
    assert abs((tel.start[2] - tel.truth[2]).std() - 1e-3) < 5e-5
    # plane k sits at x = 100 (k + 1) with normal +x and local axes (y, z)
    assert np.allclose(tel.center[:, 0], 100.0 * np.arange(1, 11))
    assert np.allclose(tel.rotation[0], [0, 0, 1, 1, 0, 0, 0, 1, 0])


def test_generator_holes_outliers_lengths(kf):
    tel = kf.make_telescope(20000, n_planes=30, min_len=5, max_len=30, hit_prob=0.9,
                           outlier_prob=0.02, x_first=50., x_step=50.)
    L = tel.n_planes
    assert L.min() == 5 and L.max() == 30
    assert abs(L.mean() - 17.5) < 0.3
    bits = np.array([bin(int(m)).count("1") for m in tel.hit_mask])
    assert abs(bits.sum() / L.sum() - 0.9) < 0.01
    assert np.all(np.array([int(m) >> int(l) for m, l in zip(tel.hit_mask, L)]) == 0)


def test_field_map_values(kf):
    tel = kf.make_telescope(10, field_map=True, field_n=11, field_half=1500.)
    g = tel.field_grid.reshape(11, 11, 11, 4)
    T = kf.TESLA
    # on axis at z = 0: Bz = 2 T, Br = 0
    assert abs(g[5, 5, 5, 2] - 2 * T) < 1e-9 and g[5, 5, 5, 0] == 0
    # at r = 1.5 m (x = 1500, y = 0, z = 0): Bz = 2 T * 0.8
    assert abs(g[5, 5, 10, 2] - 1.6 * T) < 1e-9
    # Br = (r z / Z^2) Bz at x = 1500, z = 1500
    bz = 2 * T * 0.8 * np.exp(-0.25)
    assert abs(g[10, 5, 10, 0] - 1500 * 1500 / 9e6 * bz) < 1e-9
