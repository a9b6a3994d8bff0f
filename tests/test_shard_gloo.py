"""Multi-rank host logic on CPU (gloo, world size 2): balanced sharding of the
tracks, gathering the per-track results, summing the adjoint's global
gradients.  The per-rank fitter here is the oracle (no GPU on this host); on a
GPU machine each rank runs the same split with the device fit."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import gpukalmanfitter_gb300 as kf
        import oracle
        from gpukalmanfitter_gb300 import shard
        tel = kf.make_telescope(3000, n_planes=30, x_first=50., x_step=50., min_len=5, max_len=30,
                                hit_prob=0.9, outlier_prob=0.02, seed=31)
        cfg = kf.default_config(overstep_limit=0.1, outlier_chi2_cut=25.0)
        keys = shard.work_keys(tel.n_planes, tel.start[4], tel.n_surfaces)
        ranges = shard.balanced_ranges(keys, world)
        mine = ranges[rank]
        res = oracle.fit(shard.subset(tel, mine), cfg, threads=1)
        full = shard.gather_tracks({k: res[k] for k in ("params", "cov", "chi2", "status", "n_steps")},
                                   mine, tel.n)
        g = {"grad_align": np.full((30, 6), rank + 1.0), "grad_field_scale": np.array([2.0 * rank]),
             "chi2_total": np.array([float(res["chi2"][res["status"] == 0].sum())])}
        red = shard.reduce_gradients(g)
        if rank == 0:
            ref = oracle.fit(tel, cfg, threads=1)
            np.savez(os.path.join(out_dir, "r.npz"), **{f"s_{k}": v for k, v in full.items()},
                     **{f"o_{k}": ref[k] for k in ("params", "cov", "chi2", "status", "n_steps")},
                     ga=red["grad_align"], gfs=red["grad_field_scale"], c2=red["chi2_total"],
                     sizes=np.array([len(r) for r in ranges]),
                     work=np.array([keys[r].mean() for r in ranges]))
    finally:
        dist.destroy_process_group()


def test_two_rank_shard_gather_reduce(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    mp.spawn(_rank, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    r = np.load(tmp_path / "r.npz")
    for k in ("params", "cov", "chi2", "status", "n_steps"):
        assert np.array_equal(r[f"s_{k}"], r[f"o_{k}"]), k
    assert np.all(r["ga"] == 3.0) and r["gfs"][0] == 2.0
    ok = r["o_status"] == 0
    assert abs(r["c2"][0] - r["o_chi2"][ok].sum()) <= 1e-9 * r["c2"][0]
    assert abs(int(r["sizes"][0]) - int(r["sizes"][1])) <= 32
    assert abs(r["work"][0] - r["work"][1]) < 0.05 * r["work"].mean()
