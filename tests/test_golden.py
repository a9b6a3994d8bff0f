"""The committed golden fixtures (tests/golden, written by make_golden.py):
the oracle reproduces its stored fits of the stored inputs (on any host, to
the libm differences between machines), the writers reproduce the stored
files, and the CUDA fitter's FP64 forms match the stored fits at the 1e-9
bar (marked gpu).  Cases: the 10-plane telescope at the benchmark's and at
the reference's overstep limit, 30 planes with holes / outliers / uneven
lengths, an 11^3 field map, 0.5 mm silicon planes, a misaligned
20-plane telescope."""
import numpy as np
import pytest

from golden import NAMES, HERE, load

DIAG = [0, 6, 11, 15, 18, 20]


def _rel(a, b, scale):
    return float(np.max(np.abs(a - b) / scale, initial=0.0))


def _compare(got, exp, tol, smoothed=True):
    assert np.array_equal(got["status"], exp["status"])
    assert np.array_equal(got["n_steps"], exp["n_steps"])
    assert np.array_equal(got["n_meas"], exp["n_meas"])
    ok = exp["status"] == 0
    sig = np.sqrt(np.abs(exp["cov"][DIAG]))
    scale = np.maximum(np.abs(exp["params"]), sig)[:, ok]
    assert _rel(got["params"][:, ok], exp["params"][:, ok], scale) < tol
    e = 0
    for i in range(6):
        for j in range(i, 6):
            s = np.sqrt(np.abs(exp["cov"][DIAG[i]] * exp["cov"][DIAG[j]]))[ok]
            assert _rel(got["cov"][e, ok], exp["cov"][e, ok], s) < 10 * tol, (i, j)
            e += 1
    assert _rel(got["chi2"][ok], exp["chi2"][ok], np.maximum(exp["chi2"][ok], 1.0)) < tol
    if smoothed and "smoothed" in exp:
        for k in range(exp["smoothed"].shape[0]):
            sg, se = got["smoothed"][k], exp["smoothed"][k]
            sc = np.maximum(np.abs(se[:6]), np.sqrt(np.abs(se[6 + np.array(DIAG)])))[:, ok]
            assert _rel(sg[:6, ok], se[:6, ok], np.where(sc > 0, sc, 1.0)) < tol, k


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_golden(orc, name):
    tel, cfg, exp = load(name)
    got = orc.fit(tel, cfg, threads=1, smoothed="smoothed" in exp, variant="precise")
    _compare(got, exp, 1e-12)


def test_writers_reproduce_golden(tmp_path, kf):
    from gpukalmanfitter_gb300 import writer
    tel, cfg, exp = load("holes30")
    for fn, fname in ((lambda p: writer.write_params_csv(p, exp), "holes30_params.csv"),
                      (lambda p: writer.write_states_obj(p, exp, tel), "holes30_states.obj"),
                      (lambda p: writer.write_params_table(p, exp, tel), "holes30_table.csv")):
        p = tmp_path / fname
        fn(p)
        assert p.read_text() == (HERE / fname).read_text(), fname


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("form", ["grid", "batched"])
def test_gpu_matches_golden(kf, name, form):
    tel, cfg, exp = load(name)
    b = kf.DeviceBatch(tel, cfg, smoothed="smoothed" in exp)
    b.fit() if form == "grid" else b.fit_sorted()
    _compare(b.results(), exp, 1e-9)
