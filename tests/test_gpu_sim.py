"""GPU simulation (kf_simulate_tracks) against the host generator
(kf_synth_tracks), which its per-track code restates on the device: every
draw-driven quantity (hit masks, lengths, outliers, charges) identical, the
continuous ones equal to the math library's last-bit rounding; fits of the
GPU-simulated batch without a host round trip, with unit pulls.

Workloads: the 10-plane uniform-field telescope, 30 planes with holes,
outliers and uneven lengths, a misaligned telescope, 0.5 mm silicon planes,
and the 41^3 field map."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DIAG = [0, 6, 11, 15, 18, 20]

CASES = {
    "uniform10": dict(),
    "holes30": dict(n_planes=30, x_first=50., x_step=50., min_len=5, max_len=30, hit_prob=0.9,
                    outlier_prob=0.02),
    "misaligned20": dict(n_planes=20, x_first=50., x_step=50., mis_shift=0.1, mis_rot=1e-3),
    "material10": dict(material=0.5),
    "map10": dict(field_map=True, field_n=41),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_device_simulation_matches_host_generator(kf, case):
    kw = CASES[case]
    n = 20000
    host = kf.make_telescope(n, seed=555, **kw)
    dev = kf.make_telescope(n, seed=555, device="cuda", **kw).to_host()
    assert np.array_equal(host.hit_mask, dev.hit_mask)
    assert np.array_equal(host.n_planes, dev.n_planes)
    assert np.array_equal(np.sign(host.truth[4]), np.sign(dev.truth[4]))
    # draws identical: truth parameters exactly, smeared values to rounding
    assert np.array_equal(host.truth, dev.truth)
    assert np.array_equal(host.start_cov, dev.start_cov)
    assert np.max(np.abs(host.start - dev.start) / np.maximum(np.abs(host.start), 1e-3)) < 1e-13
    assert np.max(np.abs(host.perigee - dev.perigee)) < 1e-15
    # hits: the helix / RK solve through sin, cos and atan2 of either library
    tol = 1e-8 if case == "map10" else 1e-10  # mm
    assert np.max(np.abs(host.meas - dev.meas)) < tol, np.max(np.abs(host.meas - dev.meas))


def test_fit_of_gpu_simulated_batch(kf, orc):
    """The simulated arrays feed the fitter in place (no host copy); results
    equal the fit of the host-generated batch to the inputs' rounding, and
    the pulls against the truth are unit-width."""
    kw = CASES["holes30"]
    n = 50000
    cfg = kf.default_config(overstep_limit=0.1, outlier_chi2_cut=25.0)
    dev_tel = kf.make_telescope(n, seed=556, device="cuda", **kw)
    b = kf.DeviceBatch(dev_tel, cfg)
    b.fit_sorted()
    g = b.results()
    h = kf.fit_device(kf.make_telescope(n, seed=556, **kw), cfg)
    assert np.array_equal(g["status"], h["status"])
    ok = g["status"] == 0
    assert ok.mean() > 0.99
    rel = np.abs(g["params"][:, ok] - h["params"][:, ok]) / np.maximum(np.abs(h["params"][:, ok]), 1e-3)
    assert np.max(rel) < 1e-8, np.max(rel)
    truth = dev_tel.truth.cpu().numpy()
    w = ((g["params"] - truth)[:5, ok] / np.sqrt(np.abs(g["cov"][DIAG]))[:5, ok]).std(axis=1)
    assert np.all((w > 0.95) & (w < 1.1)), w


def test_simulation_rejects_bad_arguments(kf):
    with pytest.raises(kf.KfError):
        kf.make_telescope(10, seed=1, device="cuda", min_len=5, max_len=3)
    with pytest.raises(kf.KfError):
        kf.make_telescope(10, seed=1, device="cuda", material=0.5, field_map=True, field_n=11)


def test_zero_tracks_and_one_track(kf):
    t0 = kf.make_telescope(0, seed=3, device="cuda")
    assert t0.meas.shape[2] == 0
    h = kf.make_telescope(1, seed=3)
    d = kf.make_telescope(1, seed=3, device="cuda").to_host()
    assert np.array_equal(h.hit_mask, d.hit_mask) and np.array_equal(h.truth, d.truth)
