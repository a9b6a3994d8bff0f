"""Surface material effects (the reference's pointwise material interaction
after each measurement, KalmanFitter.hpp:405-449): the oracle's formulas
against values worked out by hand from RPP2018, the oracle's fit against the
truth of a generator that scatters and slows the particle by the same model,
and the CUDA fitter against the oracle (marked gpu).

Workload: the 10-plane telescope with 0.5 mm of silicon on every plane (the
reference driver's geometry, Run/GPU/KalmanFitterGPUTest.cu:253)."""
import math

import numpy as np
import pytest

DIAG = [0, 6, 11, 15, 18, 20]
MUON = 0.1056583755


def _interact(lib, fn, mat, flags, n, d, p, q, m):
    import ctypes as C
    out = (C.c_double * 5)()
    arr = lambda v: (C.c_double * len(v))(*v)
    getattr(lib, fn).restype = C.c_int32
    rc = getattr(lib, fn)(arr(mat), C.c_int32(flags), arr(n), arr(d), C.c_double(p),
                          C.c_double(q), C.c_double(m), out)
    return rc, np.array(list(out))


def test_interaction_by_hand(kf):
    """A 1 GeV muon crossing 0.5 mm of silicon at normal incidence: theta0
    (RPP2018 eq. 33.15) and the mean loss as the reference writes it
    (Interactions.ipp:150-176: prefactor K/2, so half of RPP's eq. 33.5
    mean), evaluated here in Python."""
    si = kf.silicon(0.5)
    t, X0, Z, rho = si[0], si[1], si[4], si[5]
    p, m = 1.0, MUON
    E = math.hypot(p, m)
    beta2 = (p / E) ** 2
    tt = math.sqrt(t / X0 / beta2)
    theta0 = 13.6e-3 / p * tt * (1 + float(np.float32(0.038)) * 2 * math.log(tt))
    bg, gamma, me = p / m, E / m, 0.5109989461e-3
    wmax = 2 * me * bg ** 2 / (1 + 2 * gamma * me / m + (me / m) ** 2)
    I = 16e-9 * Z ** float(np.float32(0.9))
    eps = 0.5 * 0.307075e-3 * 100 * Z * rho * t / beta2
    loss = eps * (0.5 * math.log(2 * me * bg ** 2 / I) + 0.5 * math.log(wmax / I) - beta2)
    sigma_e = 4 * eps / (2 * math.sqrt(2 * math.log(2.0)))
    sigma_qop = math.sqrt(1 / beta2) / p ** 2 * sigma_e
    rc, out = _interact(kf.load(), "kf_material_interaction", si, 3, [1, 0, 0], [1, 0, 0], p, 1.0, m)
    assert rc == 0
    assert abs(out[2] - theta0 ** 2) <= 1e-12 * theta0 ** 2
    assert abs(out[1] - theta0 ** 2) <= 1e-12 * theta0 ** 2  # phi: sin(theta) = 1
    assert abs(out[4] - loss) <= 1e-12 * loss
    assert abs(out[3] - sigma_qop ** 2) <= 1e-12 * sigma_qop ** 2
    assert abs(out[0] - math.sqrt((E - loss) ** 2 - m * m)) <= 1e-14
    assert _interact(kf.load(), "kf_material_interaction", si, 0, [1, 0, 0], [1, 0, 0], p, 1., m)[0] == 1
    assert _interact(kf.load(), "kf_material_interaction", kf.silicon(0.), 3, [1, 0, 0], [1, 0, 0], p, 1., m)[0] == 1


def test_interaction_library_against_oracle(kf, orc):
    """The library's interaction (kf_material.h, used by the fit kernels) and
    the oracle's restatement agree on random crossings."""
    rng = np.random.default_rng(5)
    lib, olib = kf.load(), orc.load("default")
    for _ in range(300):
        mat = kf.silicon(rng.uniform(0.05, 5.0))
        d = np.array([1.0, rng.normal(0, 0.3), rng.normal(0, 0.3)])
        d /= np.linalg.norm(d)
        n = np.array([1.0, rng.normal(0, 0.1), rng.normal(0, 0.1)])
        n /= np.linalg.norm(n)
        p, q = rng.uniform(0.2, 20.0), rng.choice([-1.0, 1.0])
        flags = int(rng.integers(1, 4))
        ra, a = _interact(lib, "kf_material_interaction", mat, flags, n, d, p, q, MUON)
        rb, b = _interact(olib, "oracle_material_interaction", mat, flags, n, d, p, q, MUON)
        assert ra == rb == 0
        assert abs(a[0] - b[0]) <= 1e-14 * b[0]
        for k in (1, 2, 3):
            assert abs(a[k] - b[k]) <= 1e-13 * max(b[k], 1e-300), (k, a, b)
        # the oracle's loss is the energy difference (rounding of E ~ p)
        assert abs(a[4] - b[4]) <= 1e-9 * abs(b[4]) + 1e-14 * math.hypot(p, MUON)


@pytest.mark.parametrize("thickness", [0.5, 2.0])
def test_oracle_pulls_with_material(kf, orc, thickness):
    """Fitting with the material model gives unit pull widths on tracks
    simulated with it; ignoring it gives wide pulls."""
    tel = kf.make_telescope(4000, seed=7, material=thickness)
    for me, lo, hi in ((3, 0.95, 1.06), (0, 1.1, 1e9)):
        cfg = kf.default_config(overstep_limit=0.1, material_effects=me)
        o = orc.fit(tel, cfg, threads=0)
        ok = o["status"] == 0
        assert ok.mean() == 1.0
        w = ((o["params"] - tel.truth)[:5, ok] / np.sqrt(np.abs(o["cov"][DIAG]))[:5, ok]).std(axis=1)
        if me:
            assert np.all((w > lo) & (w < hi)), w
        else:
            assert np.max(w) > lo, w


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["grid", "batched"])
def test_material_parity(kf, orc, form):
    """FP64 plain and batched forms against the oracle with material:
    identical control flow, parameters and chi2 to 1e-9, covariance to 1e-8
    (the general smoother's 6x6 solve in FP64 against the oracle's extended
    precision; cond(C_p) reaches 1e7)."""
    tel = kf.make_telescope(3000, seed=11, material=0.5)
    cfg = kf.default_config(overstep_limit=0.1, material_effects=3)
    b = kf.DeviceBatch(tel, cfg)
    if form == "grid":
        b.fit()
    else:
        b.fit_sorted()
    g = b.results()
    o = orc.fit(tel, cfg, threads=0, variant="precise")
    assert np.array_equal(g["status"], o["status"])
    assert np.array_equal(g["n_steps"], o["n_steps"])
    ok = o["status"] == 0
    from conftest import parity_report
    rep = parity_report(g, o, 1e-9, mask=ok)
    print("material gpu vs oracle:", rep)
    assert rep["params"] <= 1.0 and rep["chi2"] <= 1.0 and rep["cov"] <= 10.0, rep


@pytest.mark.gpu
def test_material_smoothed_states_and_pulls(kf, orc):
    tel = kf.make_telescope(2000, seed=12, material=0.5)
    cfg = kf.default_config(overstep_limit=0.1, material_effects=3)
    g = kf.fit_device(tel, cfg, smoothed=True)
    o = orc.fit(tel, cfg, threads=0, smoothed=True, variant="precise")
    sg, so = g["smoothed"], o["smoothed"]
    for k in range(tel.n_surfaces):
        sig = np.sqrt(so[k, 6 + np.array(DIAG)])
        scale = np.maximum(np.abs(so[k, :6]), sig)
        assert np.max(np.abs(sg[k, :6] - so[k, :6]) / scale) < 1e-9
    ok = g["status"] == 0
    w = ((g["params"] - tel.truth)[:5, ok] / np.sqrt(np.abs(g["cov"][DIAG]))[:5, ok]).std(axis=1)
    assert np.all((w > 0.95) & (w < 1.06)), w


@pytest.mark.gpu
def test_material_mixed_accuracy(kf, orc):
    """The mixed form with material against the FP64 oracle: median
    parameter error at most 1e-6 relative, pull widths within 1 %."""
    tel = kf.make_telescope(5000, seed=13, material=0.5)
    g = kf.fit_device(tel, kf.default_config(overstep_limit=0.1, material_effects=3, precision=1))
    o = orc.fit(tel, kf.default_config(overstep_limit=0.1, material_effects=3), threads=0,
                variant="precise")
    ok = (g["status"] == 0) & (o["status"] == 0)
    assert ok.mean() > 0.999
    sig = np.sqrt(np.abs(o["cov"][DIAG]))[:, ok]
    rel = np.abs(g["params"][:, ok] - o["params"][:, ok]) / np.maximum(np.abs(o["params"][:, ok]), sig)
    assert np.all(np.median(rel, axis=1) <= 1e-6), np.median(rel, axis=1)


@pytest.mark.gpu
def test_adjoint_rejects_material(kf):
    tel = kf.make_telescope(10, seed=1, material=0.5)
    with pytest.raises(kf.KfError):
        kf.AdjointBatch(tel, kf.default_config(material_effects=3)).run(grad=True)
