"""GPU parity: the CUDA fitter (through the C ABI) against the oracle.

Tolerance: 1e-9 relative on fitted parameters (scale max(|x|, sigma_x)),
covariance elements (scale sqrt(C_ii C_jj)) and chi2 (scale max(chi2, 1));
status, measurement count, RK step and trial counts must be identical.  The
comparison point is the oracle's "precise" build (smoother in extended
precision), see _compare.
"""
import numpy as np
import pytest

from conftest import parity_report

pytestmark = pytest.mark.gpu

TOL = 1e-9
DIAG = [0, 6, 11, 15, 18, 20]


def _compare(g, o, tol=TOL):
    """Identical control flow and 1e-9 relative agreement on every track.

    ``o`` comes from the oracle's "precise" build, which evaluates the
    reference smoother formula in extended precision (its FP64 evaluation
    scatters by up to ~2e-8 relative on the q/p variance).
    """
    assert np.array_equal(g["status"], o["status"]), np.nonzero(g["status"] != o["status"])
    assert np.array_equal(g["n_meas"], o["n_meas"])
    assert np.array_equal(g["n_steps"], o["n_steps"])
    assert np.array_equal(g["n_trials"], o["n_trials"])
    ok = o["status"] == 0
    rep = parity_report(g, o, tol, mask=ok)
    print("gpu vs oracle:", rep)
    assert rep["params"] <= 1.0 and rep["chi2"] <= 1.0 and rep["cov"] <= 1.0, rep
    return rep


@pytest.mark.parametrize("overstep", [0.01, 0.1])
def test_config0_parity(kf, orc, overstep):
    """1000 tracks, 10-plane telescope, uniform 2 T (reference -d cpu -t 1000).
    At the reference's 0.01 mm overstep limit a quarter of the tracks skip
    planes and run to maxSteps: those paths must match too."""
    tel = kf.make_telescope(1000)
    cfg = kf.default_config(overstep_limit=overstep)
    g = kf.fit_device(tel, cfg)
    o = orc.fit(tel, cfg, threads=0, variant="precise")
    _compare(g, o)
    if overstep == 0.1:
        assert np.all(g["status"] == 0)


def test_host_api_matches_device_api(kf):
    tel = kf.make_telescope(777)
    cfg = kf.default_config(overstep_limit=0.1)
    a = kf.fit_device(tel, cfg, smoothed=True)
    b = kf.fit_host(tel, cfg, smoothed=True)
    for k in ("params", "cov", "chi2", "status", "n_meas", "n_steps", "smoothed"):
        assert np.array_equal(a[k], b[k]), k


def test_smoothed_states_parity(kf, orc):
    tel = kf.make_telescope(300)
    cfg = kf.default_config(overstep_limit=0.1)
    g = kf.fit_device(tel, cfg, smoothed=True)
    o = orc.fit(tel, cfg, threads=0, smoothed=True, variant="precise")
    sg, so = g["smoothed"], o["smoothed"]
    for k in range(tel.n_surfaces):
        sig = np.sqrt(so[k, 6 + np.array(DIAG)])
        scale = np.maximum(np.abs(so[k, :6]), sig)
        assert np.max(np.abs(sg[k, :6] - so[k, :6]) / scale) < TOL
        assert np.max(np.abs(sg[k, 6 + 0] - so[k, 6 + 0]) / so[k, 6]) < TOL


def test_config1_100k_parity(kf, orc):
    tel = kf.make_telescope(100_000, seed=42)
    cfg = kf.default_config(overstep_limit=0.1)
    g = kf.fit_device(tel, cfg)
    o = orc.fit(tel, cfg, threads=0, variant="precise")
    _compare(g, o)


def test_faithful_and_rebuilt_jacobian(kf, orc):
    tel = kf.make_telescope(500, seed=3)
    for faithful in (1, 0):
        cfg = kf.default_config(overstep_limit=0.1, faithful_jacobian=faithful)
        _compare(kf.fit_device(tel, cfg), orc.fit(tel, cfg, threads=0, variant="precise"))


def test_holes_outliers_parity(kf, orc):
    tel = kf.make_telescope(20_000, n_planes=30, x_first=50., x_step=50., min_len=5, max_len=30,
                           hit_prob=0.9, outlier_prob=0.02, seed=11)
    cfg = kf.default_config(overstep_limit=0.1, outlier_chi2_cut=25.0)
    _compare(kf.fit_device(tel, cfg), orc.fit(tel, cfg, threads=0, variant="precise"))


def test_field_map_parity(kf, orc):
    tel = kf.make_telescope(3000, n_planes=30, x_first=50., x_step=50., field_map=True, seed=5)
    cfg = kf.default_config(overstep_limit=0.1)
    _compare(kf.fit_device(tel, cfg), orc.fit(tel, cfg, threads=0, variant="precise"))


def test_edge_cases(kf, orc):
    cfg = kf.default_config(overstep_limit=0.1)
    for n in (1, 31, 33, 129):
        tel = kf.make_telescope(n, seed=n)
        _compare(kf.fit_device(tel, cfg), orc.fit(tel, cfg, threads=1, variant="precise"))
    tel = kf.make_telescope(64, seed=9)
    tel.start[4, 0] = 0.0
    tel.start[2, 1] = np.nan
    tel.hit_mask[2] = 0
    tel.hit_mask[3] = 1          # a single hit
    tel.n_planes[4] = 1
    g = kf.fit_device(tel, cfg)
    o = orc.fit(tel, cfg, threads=1, variant="precise")
    assert g["status"][0] == 5 and g["status"][1] == 5 and g["status"][2] == 4
    _compare(g, o)


def test_empty_batch(kf):
    tel = kf.make_telescope(1)
    b = kf.DeviceBatch(tel, kf.default_config())
    b.ins.n_tracks = 0
    b.fit()  # no launch, no error


def test_config1_1M_parity(kf, orc):
    """The headline workload at its full size, 1M tracks: the plain form
    (one thread per track) and the batched form (sorted queue, persistent
    kernel) each against the precise oracle at 1e-9, with identical status,
    measurement, RK step and trial counts on every track; then the
    size-independent properties: every track fits, unit pull widths, chi2 per
    degree of freedom 1, and reruns bitwise identical."""
    import torch
    tel = kf.make_telescope(1_000_000, seed=2024)
    cfg = kf.default_config(overstep_limit=0.1)
    b = kf.DeviceBatch(tel, cfg)
    b.fit()
    plain = b.results()
    b.fit_sorted()
    batched = b.results()
    o = orc.fit(tel, cfg, threads=0, variant="precise")
    rep_plain = _compare(plain, o)
    rep_batched = _compare(batched, o)
    print("1M plain:", rep_plain, "1M batched:", rep_batched)
    b.fit()
    torch.cuda.synchronize()
    again = b.results()
    for k in ("params", "cov", "chi2", "status", "n_steps"):
        assert np.array_equal(plain[k], again[k])
    assert np.all(plain["status"] == 0)
    pulls = (plain["params"] - tel.truth) / np.sqrt(plain["cov"][DIAG])
    assert np.all(np.abs(pulls[:5].std(axis=1) - 1) < 0.02)
    assert abs(plain["chi2"].mean() / 20 - 1) < 0.01


def test_config2_4M_batched_parity(kf, orc):
    """The batching workload at its full size: 4M tracks of 30 planes with
    uneven lengths U{5..30}, 10 % holes and 2 % outliers, fitted in one
    batched launch (sorted queue, persistent kernel); every fourth track
    (1M tracks) against the precise oracle at 1e-9 with identical control
    flow, and the whole batch for its properties."""
    from gpukalmanfitter_gb300 import shard
    tel = kf.make_telescope(4_000_000, n_planes=30, x_first=50., x_step=50., min_len=5,
                            max_len=30, hit_prob=0.9, outlier_prob=0.02, seed=1234567892)
    cfg = kf.default_config(overstep_limit=0.1, outlier_chi2_cut=25.0)
    b = kf.DeviceBatch(tel, cfg)
    b.fit_sorted()
    g = b.results()
    del b
    idx = np.arange(0, tel.n, 4)
    o = orc.fit(shard.subset(tel, idx), cfg, threads=0, variant="precise")
    rep = _compare({k: v[..., idx] for k, v in g.items()}, o)
    print("4M batched, 1M checked:", rep)
    ok = g["status"] == 0
    assert ok.mean() > 0.999
    hits = np.array([bin(int(m)).count("1") for m in tel.hit_mask[:20000]])
    assert np.mean(g["n_meas"][:20000][ok[:20000]] == hits[ok[:20000]]) == 1.0
