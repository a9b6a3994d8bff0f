"""Track sharding over ranks (one process per GPU) and the host-side
collectives of the fit and the chi2 adjoint.

Tracks are independent, so a multi-GPU fit has no exchange on its data path:
each rank fits a subset of the tracks (the reference also splits by device
with no exchange, Run/GPU/KalmanFitterGPUTest.cu:389-510).  To balance the
ranks the tracks are ordered by the batched form's work key (sequence length,
then |q/p|) and dealt out in warp-sized chunks round-robin, so every rank gets
the same mix of long and short tracks.  The results are gathered back into
track order; the adjoint's global gradients (alignment 6 x planes, field
scale, total chi2) are summed over ranks.
"""
from __future__ import annotations

import numpy as np

CHUNK = 32  # tracks per warp of the persistent kernel


def work_keys(n_planes: np.ndarray | None, start_qop: np.ndarray, n_surfaces: int) -> np.ndarray:
    """Ascending key = descending expected work (the batched form's queue key)."""
    L = np.full(start_qop.shape, n_surfaces) if n_planes is None else np.clip(n_planes, 0, n_surfaces)
    q = np.abs(start_qop)
    with np.errstate(divide="ignore", invalid="ignore"):
        qb = np.where((q > 0) & np.isfinite(q), np.floor((np.log2(q) + 7.0) * 2.0), 0)
    qb = np.clip(qb, 0, 15).astype(np.int64)
    return (64 - L.astype(np.int64)) * 16 + (15 - qb)


def balanced_ranges(keys: np.ndarray, world: int, chunk: int = CHUNK) -> list[np.ndarray]:
    """Track indices of each rank: stable sort by key, chunks of `chunk`
    tracks dealt round-robin."""
    order = np.argsort(keys, kind="stable")
    chunks = [order[i:i + chunk] for i in range(0, len(order), chunk)]
    out = [[] for _ in range(world)]
    for c, idx in enumerate(chunks):
        out[c % world].append(idx)
    return [np.sort(np.concatenate(r)) if r else np.zeros(0, dtype=np.int64) for r in out]


def subset(tel, idx: np.ndarray):
    """A Telescope holding only the tracks idx, in that order (same geometry
    and field).  Host arrays stay numpy; the torch tensors of a telescope
    simulated on the GPU are gathered on their device."""
    import copy
    t = copy.copy(tel)
    t.n = int(len(idx))
    on_device = hasattr(tel.meas, "index_select")
    if on_device:
        import torch
        di = torch.as_tensor(np.asarray(idx, dtype=np.int64), device=tel.meas.device)
        take = lambda a: a.index_select(a.dim() - 1, di).contiguous()
    else:
        take = lambda a: np.ascontiguousarray(a[..., idx])
    for k in ("meas", "hit_mask", "n_planes", "start", "start_cov", "perigee", "truth"):
        setattr(t, k, take(getattr(tel, k)))
    return t


def rank_tracks(tel, rank: int, world: int, chunk: int = CHUNK) -> np.ndarray:
    """Track indices of `rank` in a batch split over `world` ranks by work
    key (balanced_ranges); the keys come from the telescope's lengths and
    start q/p, wherever its arrays live."""
    lengths, qop = tel.n_planes, tel.start[4]
    if hasattr(qop, "cpu"):
        lengths, qop = lengths.cpu().numpy(), qop.cpu().numpy()
    keys = work_keys(np.asarray(lengths), np.asarray(qop), tel.n_surfaces)
    return balanced_ranges(keys, world, chunk)[rank]


def place_tracks(parts, n: int) -> dict:
    """Per-track results of several shards, [(track indices, {name: array
    with the track axis last}), ...], put back into one batch of n tracks in
    track order."""
    out = {}
    for ridx, res in parts:
        for k, v in res.items():
            v = np.asarray(v)
            if k not in out:
                out[k] = np.zeros(v.shape[:-1] + (n,), dtype=v.dtype)
            out[k][..., np.asarray(ridx)] = v
    return out


def gather_tracks(local: dict, idx: np.ndarray, n: int, group=None) -> dict:
    """All ranks' per-track results back in track order (every array's last
    axis is the track axis)."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    parts = [None] * world
    dist.all_gather_object(parts, (np.asarray(idx), {k: np.asarray(v) for k, v in local.items()}),
                           group=group)
    return place_tracks(parts, n)


def reduce_gradients(grads: dict, group=None) -> dict:
    """Sum the adjoint's global results (grad_align, grad_field_scale,
    chi2_total) over ranks; per-track results stay with their rank."""
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    out = {}
    for k in ("grad_align", "grad_field_scale", "chi2_total"):
        if k in grads:
            t = torch.as_tensor(np.asarray(grads[k], dtype=np.float64)).clone().to(dev)
            dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
            out[k] = t.cpu().numpy()
    return out
