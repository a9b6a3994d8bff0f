"""Field-map ingestion (gb300kf_fieldmap.h, gpukalmanfitter_gb300.fieldmap)
against the restatement of the reference's map construction and lookup
(oracle/field_map.py, src/MagneticField/BFieldMapUtils.cpp): grid values
bit-exact, lookups within float rounding over the reference's whole range
(including its fall to zero above the last point), mirrored octants and
quadrants, RZ maps, malformed files; and fits through an ingested map
(oracle on the CPU, the CUDA fitter against it marked gpu)."""
import numpy as np
import pytest

from gpukalmanfitter_gb300 import KfError, TESLA
from gpukalmanfitter_gb300 import fieldmap as FM


def _solenoid_xyz(x, y, z):
    """a smooth test field in tesla: Bz falling with r and |z|, Br from
    div B = 0 to first order, a small Bx offset"""
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    r2 = X ** 2 + Y ** 2
    bz = 2.0 * (1 - 0.2 * r2 / 1500.0 ** 2) * np.exp(-(Z / 3000.0) ** 2)
    dbz = bz * (-2 * Z / 3000.0 ** 2)
    return np.stack([-0.5 * X * dbz + 0.01, -0.5 * Y * dbz, bz], axis=-1)


@pytest.fixture(scope="module")
def xyz_file(tmp_path_factory):
    d = tmp_path_factory.mktemp("maps")
    x = np.linspace(-1200., 1200., 9)
    y = np.linspace(-600., 600., 7)
    z = np.linspace(-1000., 1000., 11)
    p = d / "xyz.txt"
    FM.write_field_map_xyz(p, x, y, z, _solenoid_xyz(x, y, z), fmt="%.17g")
    # comments, blank and whitespace lines are skipped
    text = "% comment\n# another\n\n   \n" + p.read_text()
    p.write_text(text)
    return p, (x, y, z)


def test_xyz_grid_values_exact(xyz_file):
    from oracle import field_map as OF
    p, (x, y, z) = xyz_file
    fm = FM.read_field_map_xyz(p)
    ref = OF.MapXYZ(p, field_unit=TESLA)
    assert fm.dims == (10, 8, 12)  # file points + the zero plane above the last
    assert np.allclose(fm.min, (-1200., -600., -1000.)) and np.allclose(fm.max, (1500., 800., 1200.))
    g = fm.grid
    for k in range(12):
        for j in range(8):
            for i in range(10):
                want = ref.bin_value((i, j, k)).astype(np.float32)
                assert np.array_equal(g[k, j, i, :3], want), (i, j, k)
    assert np.all(g[..., 3] == 0)


def test_xyz_lookup_matches_reference_over_its_range(xyz_file):
    from oracle import field_map as OF
    p, _ = xyz_file
    fm = FM.read_field_map_xyz(p)
    ref = OF.MapXYZ(p, field_unit=TESLA)
    rng = np.random.default_rng(1)
    bmax = np.abs(fm.grid).max()
    for _ in range(400):
        # [min, max + step): up to the reference's last bin, where it falls to 0
        pos = [rng.uniform(fm.min[a], fm.max[a] - 1e-9) for a in range(3)]
        a = OF.trilinear(fm.grid, fm.dims, fm.min, fm.max, pos)
        b = ref.field(pos)
        assert np.max(np.abs(a - b)) <= 2e-7 * bmax, (pos, a, b)


def test_xyz_units_and_mirrored_octant(tmp_path):
    from oracle import field_map as OF
    x = np.linspace(0., 1.2, 5)  # metres
    y = np.linspace(0., 0.6, 4)
    z = np.linspace(0., 1.0, 6)
    b = _solenoid_xyz(x * 1000, y * 1000, z * 1000) * 10.0  # kilogauss
    p = tmp_path / "octant.txt"
    FM.write_field_map_xyz(p, x, y, z, b, fmt="%.17g")
    fm = FM.read_field_map_xyz(p, length_unit=1000.0, field_unit=0.1 * TESLA, first_octant=True)
    ref = OF.MapXYZ(p, length_unit=1000.0, field_unit=0.1 * TESLA, first_octant=True)
    assert fm.dims == (10, 8, 12)
    assert np.allclose(fm.min, (-1200., -600., -1000.))
    for k in range(11):
        for j in range(7):
            for i in range(9):
                assert np.array_equal(fm.grid[k, j, i, :3], ref.bin_value((i, j, k)).astype(np.float32))
    # mirrored values are copies (the reference does not flip signs)
    assert np.array_equal(fm.grid[0, 0, 0], fm.grid[10, 6, 8])


def test_rz_map(tmp_path):
    from oracle import field_map as OF
    r = np.linspace(0., 1500., 16)
    z = np.linspace(-2000., 2000., 21)
    R, Z = np.meshgrid(r, z, indexing="ij")
    bz = 2.0 * (1 - 0.2 * R ** 2 / 1500.0 ** 2) * np.exp(-(Z / 3000.0) ** 2)
    br = -0.5 * R * bz * (-2 * Z / 3000.0 ** 2)
    p = tmp_path / "rz.txt"
    FM.write_field_map_rz(p, r, z, np.stack([br, bz], axis=-1), fmt="%.17g")
    fm = FM.read_field_map_rz(p, native=False)
    ref = OF.MapRZ(p, field_unit=TESLA)
    assert fm.dims == (31, 31, 21)
    assert np.allclose(fm.min, (-1500., -1500., -2000.)) and np.allclose(fm.max, (1500., 1500., 2000.))
    bmax = np.abs(fm.grid).max()
    nx, ny, nz = fm.dims
    rng = np.random.default_rng(2)
    for _ in range(300):
        i, j, k = rng.integers(nx), rng.integers(ny), rng.integers(nz)
        pos = [fm.min[0] + i * (fm.max[0] - fm.min[0]) / (nx - 1),
               fm.min[1] + j * (fm.max[1] - fm.min[1]) / (ny - 1),
               fm.min[2] + k * (fm.max[2] - fm.min[2]) / (nz - 1)]
        assert np.max(np.abs(fm.grid[k, j, i, :3] - ref.field(pos))) <= 1e-7 * bmax
    # on the axis: phi = 0
    c = fm.grid[10, 15, 15]
    assert c[1] == 0.0
    # a chosen Cartesian grid
    fm2 = FM.read_field_map_rz(p, n_xyz=(5, 5, 5), min_xyz=(-100., -100., -100.),
                               max_xyz=(100., 100., 100.), native=False)
    assert fm2.dims == (5, 5, 5)
    assert np.max(np.abs(fm2.grid[4, 4, 4, :3] - ref.field([100., 100., 100.]))) <= 1e-7 * bmax
    # mirrored quadrant
    half = np.linspace(0., 2000., 11)
    R2, Z2 = np.meshgrid(r, half, indexing="ij")
    q = tmp_path / "quadrant.txt"
    FM.write_field_map_rz(q, r, half, np.stack([R2 * 0 + 0.1, 2 - Z2 / 2000.], axis=-1),
                          fmt="%.17g")
    fq = FM.read_field_map_rz(q, first_quadrant=True, native=False)
    refq = OF.MapRZ(q, field_unit=TESLA, first_quadrant=True)
    assert fq.dims[2] == 21 and np.isclose(fq.min[2], -2000.)
    pos = [300., -400., -1234.]
    a = OF.trilinear(fq.grid, fq.dims, fq.min, fq.max, pos)
    # bz is linear in z, so only br's direction interpolation differs
    assert abs(a[2] - refq.field(pos)[2]) <= 1e-6 * abs(refq.field(pos)[2])


def _rz_test_map(path, r_step=100.0, z_step=200.0):
    """the analytic telescope map's (br, bz) on an (r, z) grid, as an RZ file
    in tesla"""
    r = np.arange(0., 1500. + r_step / 2, r_step)
    z = np.arange(-2000., 2000. + z_step / 2, z_step)
    R, Z = np.meshgrid(r, z, indexing="ij")
    bz = 2.0 * (1 - 0.2 * R ** 2 / 1500.0 ** 2) * np.exp(-(Z / 3000.0) ** 2)
    br = R * Z / 3000.0 ** 2 * bz
    FM.write_field_map_rz(path, r, z, np.stack([br, bz], axis=-1), fmt="%.17g")
    return r, z


def test_rz_native_map(orc, tmp_path):
    """The native (r, z) grid: the file's points plus the zero row above the
    last point on each axis; the oracle's lookup in it (the fit's) equals the
    reference's RZ interpolation restated in numpy (float32 grid values) over
    the whole range including the fall to zero, on the axis and with a
    mirrored quadrant; and the Cartesian resampling differs from it by the
    O(h^2 B'') of trilinear interpolation."""
    from oracle import field_map as OF
    p = tmp_path / "rz.txt"
    r, z = _rz_test_map(p)
    fm = FM.read_field_map_rz(p)
    assert fm.kind == 2 and fm.dims == (len(r) + 1, 1, len(z) + 1)
    assert np.allclose(fm.min, (0., 0., -2000.)) and np.allclose(fm.max, (1600., 0., 2200.))
    ref = OF.MapRZ(p, field_unit=TESLA)
    for ir in range(len(r)):
        for iz in range(len(z)):
            assert np.array_equal(fm.grid[iz, 0, ir, :2], ref.bin_value(ir, iz).astype(np.float32))
    assert np.all(fm.grid[-1] == 0) and np.all(fm.grid[:, :, -1] == 0)
    f = fm.field()
    bmax = np.abs(fm.grid).max()
    rng = np.random.default_rng(3)
    for _ in range(400):
        rr, ph, zz = rng.uniform(0, 1590.), rng.uniform(-np.pi, np.pi), rng.uniform(-1990., 2190.)
        pos = [rr * np.cos(ph), rr * np.sin(ph), zz]
        assert np.max(np.abs(orc.field_value(f, pos) - ref.field(pos))) <= 1e-7 * bmax
    on_axis = orc.field_value(f, [0., 0., 333.])
    assert on_axis[1] == 0.0 and np.allclose(on_axis, ref.field([0., 0., 333.]), atol=1e-7 * bmax)
    # mirrored quadrant
    q = tmp_path / "quadrant.txt"
    half = np.linspace(0., 2000., 11)
    R2, Z2 = np.meshgrid(r, half, indexing="ij")
    FM.write_field_map_rz(q, r, half, np.stack([0.1 + R2 * 0, 2 - Z2 / 2000.], axis=-1),
                          fmt="%.17g")
    fq = FM.read_field_map_rz(q, first_quadrant=True)
    refq = OF.MapRZ(q, field_unit=TESLA, first_quadrant=True)
    assert fq.dims[2] == 22 and np.isclose(fq.min[2], -2000.)
    for pos in ([300., -400., -1234.], [-20., 5., 1999.], [1000., 1000., -5.]):
        assert np.allclose(orc.field_value(fq.field(), pos), refq.field(pos), atol=1e-7 * bmax)
    # the Cartesian resampling at the r step: trilinear between its points
    fc = FM.read_field_map_rz(p, native=False)
    dev = 0.0
    for _ in range(400):
        pos = rng.uniform([-1000., -1000., -1900.], [1000., 1000., 1900.])
        dev = max(dev, float(np.max(np.abs(orc.field_value(fc.field(), pos) - ref.field(pos)))))
    assert 1e-6 * bmax < dev < 2e-2 * bmax, dev


@pytest.mark.gpu
def test_gpu_fit_in_native_rz_map(kf, orc, tmp_path):
    """Tracks simulated and fitted in a native (r, z) map: the FP64 plain and
    batched forms against the precise oracle at 1e-9, the mixed form at its
    accuracy bar."""
    p = tmp_path / "rz.txt"
    _rz_test_map(p, r_step=50.0, z_step=50.0)
    fm = FM.read_field_map_rz(p)
    tel = kf.make_telescope(3000, seed=24, field_map=fm, n_planes=10)
    cfg = kf.default_config(overstep_limit=0.1)
    o = orc.fit(tel, cfg, threads=0, variant="precise")
    assert np.mean(o["status"] == 0) > 0.99
    from conftest import parity_report
    for form in ("grid", "batched"):
        b = kf.DeviceBatch(tel, cfg)
        b.fit() if form == "grid" else b.fit_sorted()
        g = b.results()
        assert np.array_equal(g["status"], o["status"]) and np.array_equal(g["n_steps"], o["n_steps"])
        rep = parity_report(g, o, 1e-9, mask=o["status"] == 0)
        assert rep["params"] <= 1.0 and rep["chi2"] <= 1.0 and rep["cov"] <= 1.0, (form, rep)
    g = kf.fit_device(tel, kf.default_config(overstep_limit=0.1, precision=1))
    ok = (g["status"] == 0) & (o["status"] == 0)
    sig = np.sqrt(np.abs(o["cov"][[0, 6, 11, 15, 18, 20]]))[:, ok]
    rel = np.abs(g["params"][:, ok] - o["params"][:, ok]) / np.maximum(np.abs(o["params"][:, ok]), sig)
    assert np.all(np.median(rel, axis=1) <= 1e-6), np.median(rel, axis=1)


def test_malformed_files(tmp_path):
    bad = tmp_path / "bad.txt"
    bad.write_text("0 0 0 1 2 3\n0 0 1 1 2 x\n")
    with pytest.raises(KfError, match="bad.txt:2"):
        FM.read_field_map_xyz(bad)
    short = tmp_path / "short.txt"
    short.write_text("0 0 0 1 2 3\n0 0 1 1 2 3\n0 1 0 1 2 3\n1 0 0 1 2 3\n")
    with pytest.raises(KfError, match="points"):
        FM.read_field_map_xyz(short)
    order = tmp_path / "order.txt"
    x = y = z = np.array([0., 1.])
    FM.write_field_map_xyz(order, x, y, z, np.zeros((2, 2, 2, 3)))
    lines = order.read_text().splitlines()
    lines[1], lines[2] = lines[2], lines[1]
    order.write_text("\n".join(lines) + "\n")
    with pytest.raises(KfError, match="out of order"):
        FM.read_field_map_xyz(order)
    with pytest.raises(KfError, match="cannot open"):
        FM.read_field_map_xyz(tmp_path / "missing.txt")
    flat = tmp_path / "flat.txt"
    flat.write_text("0 0 0 1 2 3\n0 0 1 1 2 3\n")
    with pytest.raises(KfError, match="fewer than two"):
        FM.read_field_map_xyz(flat)


def _dump_synth_map(kf, tmp_path, n=41, half=1500.0):
    """the analytic test map of the telescope workloads, written as an XYZ
    file in GeV/(e mm) and read back"""
    tel = kf.make_telescope(1, field_map=True, field_n=n, field_half=half)
    g = tel.field_grid.reshape(n, n, n, 4).astype(np.float64)  # [z][y][x]
    ax = np.linspace(-half, half, n)
    p = tmp_path / "synth_map.txt"
    FM.write_field_map_xyz(p, ax, ax, ax, np.transpose(g[..., :3], (2, 1, 0, 3)), fmt="%.17g")
    return FM.read_field_map_xyz(p, field_unit=1.0), tel


def test_ingested_map_fits_like_the_map_itself(kf, orc, tmp_path):
    """The analytic map written to a file and read back: the grid equals the
    original on its points, and the oracle's fits in it agree with fits in
    the original grid (the cell arithmetic differs only by the rounding of
    the cell width)."""
    fm, tel0 = _dump_synth_map(kf, tmp_path)
    n = 41
    assert np.array_equal(fm.grid[:n, :n, :n], tel0.field_grid.reshape(n, n, n, 4))
    a = kf.make_telescope(400, seed=21, field_map=True, field_n=n, n_planes=10)
    b = kf.make_telescope(400, seed=21, field_map=fm, n_planes=10)
    assert np.array_equal(a.meas, b.meas)
    cfg = kf.default_config(overstep_limit=0.1)
    ra, rb = orc.fit(a, cfg, threads=0), orc.fit(b, cfg, threads=0)
    assert np.array_equal(ra["status"], rb["status"]) and np.all(ra["status"] == 0)
    assert np.array_equal(ra["n_steps"], rb["n_steps"])
    assert np.max(np.abs(ra["params"] - rb["params"]) / np.maximum(np.abs(ra["params"]), 1e-3)) < 1e-10


@pytest.mark.gpu
def test_gpu_fit_in_ingested_map(kf, orc, tmp_path):
    """FP64 fit through a map read from a file against the precise oracle in
    the same grid (bar 1e-9), plain and batched forms; the mixed form at its
    accuracy bar."""
    fm, _ = _dump_synth_map(kf, tmp_path)
    tel = kf.make_telescope(3000, seed=22, field_map=fm, n_planes=10)
    cfg = kf.default_config(overstep_limit=0.1)
    o = orc.fit(tel, cfg, threads=0, variant="precise")
    from conftest import parity_report
    for form in ("grid", "batched"):
        b = kf.DeviceBatch(tel, cfg)
        b.fit() if form == "grid" else b.fit_sorted()
        g = b.results()
        assert np.array_equal(g["status"], o["status"])
        rep = parity_report(g, o, 1e-9, mask=o["status"] == 0)
        assert rep["params"] <= 1.0 and rep["chi2"] <= 1.0, (form, rep)
    g = kf.fit_device(tel, kf.default_config(overstep_limit=0.1, precision=1))
    ok = (g["status"] == 0) & (o["status"] == 0)
    sig = np.sqrt(np.abs(o["cov"][[0, 6, 11, 15, 18, 20]]))[:, ok]
    rel = np.abs(g["params"][:, ok] - o["params"][:, ok]) / np.maximum(np.abs(o["params"][:, ok]), sig)
    assert np.all(np.median(rel, axis=1) <= 1e-6)


def test_two_point_axes_and_zero_padding(tmp_path):
    """The smallest map (2 points per axis): 3 grid points per axis, the top
    plane zero, and the lookup halfway into the padded cell is half the
    last point's value (the reference's fall to zero)."""
    from oracle import field_map as OF
    x = y = z = np.array([0., 10.])
    b = np.ones((2, 2, 2, 3)) * np.array([0.1, 0.2, 2.0])
    p = tmp_path / "tiny.txt"
    FM.write_field_map_xyz(p, x, y, z, b, fmt="%.17g")
    fm = FM.read_field_map_xyz(p)
    assert fm.dims == (3, 3, 3) and fm.max == (20., 20., 20.)
    assert np.all(fm.grid[2] == 0) and np.all(fm.grid[:, 2] == 0) and np.all(fm.grid[:, :, 2] == 0)
    a = OF.trilinear(fm.grid, fm.dims, fm.min, fm.max, [5., 5., 15.])
    r = OF.MapXYZ(p, field_unit=TESLA).field([5., 5., 15.])
    assert np.allclose(a, r, rtol=1e-6) and np.allclose(a[2], 1.0 * TESLA, rtol=1e-6)
