"""Track shards on one GPU: the multi-GPU split (gpukalmanfitter_gb300.shard)
run shard by shard on this device.  A batch dealt into k shards by work key,
each shard fitted on its own, and the results put back in track order must
equal the unsharded fit bitwise (tracks are independent); the chi2 adjoint's
global gradients summed over the shards must equal the unsharded ones to
1e-12 relative (only the order of the sums over tracks changes), and its
per-track gradients bitwise.  The reference splits by device the same way,
with no exchange (Run/GPU/KalmanFitterGPUTest.cu:389-510)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KEYS = ("params", "cov", "chi2", "status", "n_meas", "n_steps", "n_trials")


def _holes(kf, n, seed):
    return kf.make_telescope(n, n_planes=30, x_first=50., x_step=50., min_len=5, max_len=30,
                             hit_prob=0.9, outlier_prob=0.02, seed=seed)


@pytest.mark.parametrize("form", ["plain", "batched"])
@pytest.mark.parametrize("k", [2, 3])
def test_sharded_fit_equals_unsharded(kf, form, k):
    from gpukalmanfitter_gb300 import shard
    tel = _holes(kf, 60_000, seed=17 + k)
    cfg = kf.default_config(overstep_limit=0.1, outlier_chi2_cut=25.0, kernel=2,
                            block_size=128, min_blocks_per_sm=4)

    def fit(t):
        b = kf.DeviceBatch(t, cfg)
        b.fit() if form == "plain" else b.fit_sorted()
        return b.results()

    whole = fit(tel)
    parts = []
    ranges = [shard.rank_tracks(tel, r, k) for r in range(k)]
    assert sorted(np.concatenate(ranges).tolist()) == list(range(tel.n))
    for idx in ranges:
        res = fit(shard.subset(tel, idx))
        parts.append((idx, {key: res[key] for key in KEYS}))
    gathered = shard.place_tracks(parts, tel.n)
    for key in KEYS:
        assert np.array_equal(gathered[key], whole[key]), key
    sizes = [len(r) for r in ranges]
    assert max(sizes) - min(sizes) <= shard.CHUNK


def test_sharded_adjoint_sums(kf):
    from gpukalmanfitter_gb300 import shard
    tel = kf.make_telescope(9_000, n_planes=20, x_first=50., x_step=50., mis_shift=0.1,
                            mis_rot=1e-3, seed=44)
    cfg = kf.default_config(overstep_limit=0.1)
    whole = kf.AdjointBatch(tel, cfg).run(grad=True)
    k = 3
    ranges = [shard.rank_tracks(tel, r, k) for r in range(k)]
    parts, ga, gf, c2 = [], 0.0, 0.0, 0.0
    for idx in ranges:
        r = kf.AdjointBatch(shard.subset(tel, idx), cfg).run(grad=True)
        parts.append((idx, {key: r[key] for key in ("chi2", "status", "grad_start",
                                                    "grad_field_scale_track")}))
        ga = ga + r["grad_align"]
        gf = gf + r["grad_field_scale"][0]
        c2 = c2 + r["chi2_total"][0]
    g = shard.place_tracks(parts, tel.n)
    for key in ("chi2", "status", "grad_start", "grad_field_scale_track"):
        assert np.array_equal(g[key], whole[key]), key
    assert np.max(np.abs(ga - whole["grad_align"])) <= 1e-12 * np.max(np.abs(whole["grad_align"]))
    assert abs(gf - whole["grad_field_scale"][0]) <= 1e-12 * abs(whole["grad_field_scale"][0])
    assert abs(c2 - whole["chi2_total"][0]) <= 1e-12 * abs(whole["chi2_total"][0])
