"""kf_fit_batch_noalloc: the fit entry point for callers that cannot allocate
device memory.  It takes its workspace from a static device array, so it must
give exactly the fits of kf_fit_batch with a caller workspace, call after
call, and refuse batches larger than that array with a clear message.

This file is collected last so that a run stopping at the first failure has
run every other test before it."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-9


def _noalloc(lib, b, cfg, stream):
    lib.kf_fit_batch_noalloc.restype = C.c_int32
    return lib.kf_fit_batch_noalloc(C.byref(b.ins), C.byref(b.outs), C.byref(cfg),
                                    C.byref(b.geo), C.byref(b.field), C.c_void_p(stream))


def test_noalloc_matches_fit_batch_on_consecutive_calls(kf):
    import torch
    lib = kf.load()
    lib.kf_noalloc_scratch_bytes.restype = C.c_size_t
    assert lib.kf_noalloc_scratch_bytes() == 64 << 20
    cfg = kf.default_config(overstep_limit=0.1)
    tels = [kf.make_telescope(4000, seed=5), kf.make_telescope(3000, seed=6, n_planes=30,
                                                              x_first=50., x_step=50.)]
    for call, tel in enumerate(tels + tels[:1]):
        ref = kf.fit_device(tel, cfg)                # kf_fit_batch, caller workspace
        b = kf.DeviceBatch(tel, cfg)
        for v in b.out.values():
            v.fill_(-1)
        stream = torch.cuda.current_stream()
        rc = _noalloc(lib, b, cfg, stream.cuda_stream)
        assert rc == 0, lib.kf_noalloc_last_error_string()
        torch.cuda.synchronize()
        got = b.results()
        for k in ("status", "n_meas", "n_steps", "n_trials"):
            assert np.array_equal(got[k], ref[k]), (call, k)
        diag = [0, 6, 11, 15, 18, 20]
        sig = np.sqrt(np.abs(ref["cov"][diag]))
        scale = np.where(np.maximum(np.abs(ref["params"]), sig) > 0,
                         np.maximum(np.abs(ref["params"]), sig), 1.0)
        assert np.max(np.abs(got["params"] - ref["params"]) / scale) <= TOL
        cscale = np.maximum(np.abs(ref["cov"]), 1e-300)
        assert np.max(np.abs(got["cov"] - ref["cov"]) / cscale) <= TOL
        assert np.max(np.abs(got["chi2"] - ref["chi2"]) / np.maximum(ref["chi2"], 1)) <= TOL


def test_noalloc_rejects_batches_beyond_its_scratch(kf):
    lib = kf.load()
    lib.kf_noalloc_last_error_string.restype = C.c_char_p
    cfg = kf.default_config(overstep_limit=0.1)
    tel = kf.make_telescope(64, seed=1)
    b = kf.DeviceBatch(tel, cfg)
    big = kf.KfInputs.from_buffer_copy(b.ins)
    big.n_tracks = big.stride = 1_000_000          # 1M x 10 planes x 296 B > 64 MiB
    lib.kf_fit_batch_noalloc.restype = C.c_int32
    rc = lib.kf_fit_batch_noalloc(C.byref(big), C.byref(b.outs), C.byref(cfg), C.byref(b.geo),
                                  C.byref(b.field), None)
    assert rc == -2
    msg = lib.kf_noalloc_last_error_string().decode()
    assert "scratch" in msg and str(64 << 20) in msg
    # a successful call after the refusal leaves no stale message behind
    rc = lib.kf_fit_batch_noalloc(C.byref(b.ins), C.byref(b.outs), C.byref(cfg), C.byref(b.geo),
                                  C.byref(b.field), None)
    assert rc == 0
    import torch
    torch.cuda.synchronize()
    assert lib.kf_noalloc_last_error_string().decode() == ""
