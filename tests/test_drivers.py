"""End to end through the C99 drivers: data_in text files -> hydrocode_[12]D.out
(the library's scheme call) -> data_out %.10g text files, with the reference's
directory conventions (the drivers run from <root>/src/hydrocode_[12]D and read
../../data_in, write ../../data_out), compared with the oracle."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BUILD = os.path.join(ROOT, "hydrocode-fusion_gb300", "_build")
# the drivers write %.10g text: half a unit in the 10th significant digit is up to 5e-10 relative
RTOL_TEXT = 6e-10


def _write_grid(path, arr2d_rows):
    with open(path, "w") as f:
        for row in arr2d_rows:
            f.write("\t".join(f"{x:.17g}" for x in row) + "\n")


def _read_dat(path, nrows=None):
    rows = []
    for line in open(path):
        line = line.strip()
        if line:
            rows.append([float(x) for x in line.split()])
    return np.array(rows)


@pytest.mark.gpu
def test_2d_driver_end_to_end(gpu_lib, port, tmp_path):
    hg = gpu_lib
    from hydro_gb300 import cases

    exe = os.path.join(BUILD, "hydrocode_2D.out")
    assert os.path.exists(exe)
    m, n = 30, 20  # x cells (columns), y cells (lines)
    rho, u, v, p = cases.four_quadrant(m, n, seed=12)
    case = tmp_path / "data_in" / "two-dim" / "FQ"
    case.mkdir(parents=True)
    for name, a in (("RHO", rho), ("U", u), ("V", v), ("P", p)):
        _write_grid(case / f"{name}.txt", a.T)  # file line i = y index i
    (case / "config.txt").write_text("1 -1\n5 25\n4 1e-9\n6 1.4\n7 0.45\n10 %r\n11 %r\n17 -4\n18 -4\n" % (1 / m, 1 / n))
    run_dir = tmp_path / "src" / "hydrocode_2D"
    run_dir.mkdir(parents=True)
    r = subprocess.run([exe, "FQ", "fq_out", "2", "EUL"], cwd=run_dir, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    out = tmp_path / "data_out" / "two-dim" / "EUL_2_order" / "fq_out"
    cfg = hg.config_2d(t_all=-1, steps=25, hx=1 / m, hy=1 / n, bx=-4, by=-4)
    want = port.run_2d(rho, u, v, p, cfg)
    for name, key in (("RHO", "rho"), ("U", "u"), ("V", "v"), ("P", "p"), ("E", "E")):
        got = _read_dat(out / f"{name}.dat")
        assert got.shape == (2 * n, m)  # initial and final state, one line per y row
        np.testing.assert_allclose(got[n:].T, want[key], rtol=RTOL_TEXT, atol=1e-12)
        np.testing.assert_allclose(got[:n].T, {"rho": rho, "u": u, "v": v, "p": p}.get(key, got[:n].T), rtol=RTOL_TEXT)
    assert (out / "log.dat").exists() and (out / "time_plot.dat").exists()
    assert any(f.name.startswith("FLU_VAR_") for f in out.iterdir())


@pytest.mark.gpu
@pytest.mark.parametrize("order", [1, 2])
def test_1d_driver_sod(gpu_lib, tmp_path, order):
    exe = os.path.join(BUILD, "hydrocode_1D.out")
    from hydro_gb300 import cases

    rho, u, p = cases.sod(400)
    case = tmp_path / "data_in" / "one-dim" / "SOD"
    case.mkdir(parents=True)
    for name, a in (("RHO", rho), ("U", u), ("P", p)):
        (case / f"{name}.txt").write_text("\n".join(f"{x:.17g}" for x in a) + "\n")
    (case / "config.txt").write_text("1 0.2\n4 1e-9\n5 100000\n6 1.4\n7 0.45\n10 0.0025\n17 -4\n")
    run_dir = tmp_path / "src" / "hydrocode_1D"
    run_dir.mkdir(parents=True)
    r = subprocess.run([exe, "SOD", "sod_out", str(order), "EUL"], cwd=run_dir, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    out = tmp_path / "data_out" / "one-dim" / f"EUL_{order}_order" / "sod_out"
    gold = np.load(os.path.join(ROOT, "tests", "golden", "runs_1d.npz"))
    for name, key in (("RHO", "rho"), ("U", "u"), ("P", "p")):
        got = _read_dat(out / f"{name}.dat")
        np.testing.assert_allclose(got[-1], gold[f"sod{order}/{key}"], rtol=RTOL_TEXT, atol=1e-12)
    tp = _read_dat(out / "time_plot.dat").ravel()
    assert abs(tp[-1] - 0.2) < 1e-12


def _read_bin(path):
    raw = open(path, "rb").read()
    assert raw[:8] == b"HCFBIN01"
    ndim, n_x, n_y, nsnap, _ = np.frombuffer(raw[8:28], "<i4")
    times = np.frombuffer(raw[28:28 + 8 * nsnap], "<f8")
    data = np.frombuffer(raw[28 + 8 * nsnap:], "<f8").reshape(nsnap, n_y, n_x)
    return int(ndim), times, data


def _write_bin(path, plane_rows):
    a = np.ascontiguousarray(plane_rows, np.float64)
    hdr = b"HCFBIN01" + np.array([2, a.shape[1], a.shape[0], 1, 0], "<i4").tobytes()
    open(path, "wb").write(hdr + np.zeros(1, "<f8").tobytes() + a.astype("<f8").tobytes())


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [1, 2])
def test_2d_driver_binary_formats(gpu_lib, port, tmp_path, mode):
    """Initial data given as <var>.bin (no text), config[302] = 1 (text and
    binary output) or 2 (binary only): the binary output holds the FP64 state
    itself, within the FP64 form's 1e-12 of the oracle, and the text beside it
    is what the %.10g writer makes of the same numbers."""
    hg = gpu_lib
    from hydro_gb300 import cases

    exe = os.path.join(BUILD, "hydrocode_2D.out")
    m, n = 26, 18
    rho, u, v, p = cases.four_quadrant(m, n, seed=21)
    case = tmp_path / "data_in" / "two-dim" / "FQB"
    case.mkdir(parents=True)
    for name, a in (("RHO", rho), ("U", u), ("V", v), ("P", p)):
        _write_bin(case / f"{name}.bin", a.T)  # row i = y index i, as the text files
    (case / "config.txt").write_text("1 -1\n5 20\n4 1e-9\n6 1.4\n7 0.45\n10 %r\n11 %r\n17 -7\n18 -2\n302 %d\n"
                                     % (1 / m, 1 / n, mode))
    run_dir = tmp_path / "src" / "hydrocode_2D"
    run_dir.mkdir(parents=True)
    r = subprocess.run([exe, "FQB", "fqb_out", "2", "EUL"], cwd=run_dir, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    out = tmp_path / "data_out" / "two-dim" / "EUL_2_order" / "fqb_out"
    cfg = hg.config_2d(t_all=-1, steps=20, hx=1 / m, hy=1 / n, bx=-7, by=-2)
    want = port.run_2d(rho, u, v, p, cfg)
    for name, key in (("RHO", "rho"), ("U", "u"), ("V", "v"), ("P", "p"), ("E", "E")):
        ndim, times, data = _read_bin(out / f"{name}.bin")
        assert ndim == 2 and data.shape == (2, n, m) and times[0] == 0.0
        assert np.array_equal(data[0].T, {"rho": rho, "u": u, "v": v, "p": p}.get(key, data[0].T))
        rel = np.abs(data[1].T - want[key]).sum() / np.abs(want[key]).sum()
        assert rel <= 1e-12, (name, rel)
        if mode == 1:
            txt = (out / f"{name}.dat").read_text()
            blocks = [b for b in txt.split("\n\n\n") if b.strip()]
            assert len(blocks) == 2
            assert blocks[1].strip("\n") == "\n".join("".join("%.10g\t" % x for x in row) for row in data[1])
        else:
            assert not (out / f"{name}.dat").exists()
    _, _, xc = _read_bin(out / "X.bin")
    np.testing.assert_allclose(xc[0][0], (np.arange(m) + 0.5) / m, rtol=1e-14)


@pytest.mark.gpu
@pytest.mark.parametrize("order", [1, 2])
def test_1d_driver_lagrangian_sod(gpu_lib, tmp_path, order):
    """hydrocode_1D.out ... LAG: the Lagrangian schemes through the driver;
    output under data_out/one-dim/LAG_<order>_order, cell centres from the
    moved nodes."""
    exe = os.path.join(BUILD, "hydrocode_1D.out")
    from hydro_gb300 import cases

    rho, u, p = cases.sod(400)
    case = tmp_path / "data_in" / "one-dim" / "SOD"
    case.mkdir(parents=True)
    for name, a in (("RHO", rho), ("U", u), ("P", p)):
        (case / f"{name}.txt").write_text("\n".join(f"{x:.17g}" for x in a) + "\n")
    (case / "config.txt").write_text("1 0.2\n4 1e-9\n5 100000\n6 1.4\n7 0.45\n10 0.0025\n17 -4\n")
    run_dir = tmp_path / "src" / "hydrocode_1D"
    run_dir.mkdir(parents=True)
    r = subprocess.run([exe, "SOD", "sod_lag", str(order), "LAG"], cwd=run_dir, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Lagrangian scheme" in r.stdout
    out = tmp_path / "data_out" / "one-dim" / f"LAG_{order}_order" / "sod_lag"
    import oracle as orc

    cfg = orc.default_config_1d(t_all=0.2, steps=100000, hx=0.0025, bx=-4, cfl=0.45)
    want = orc.Oracle("port").run_1d_lag(rho, u, p, cfg, order)
    for name, key in (("RHO", "rho"), ("U", "u"), ("P", "p")):
        got = _read_dat(out / f"{name}.dat")
        np.testing.assert_allclose(got[-1], want[key], rtol=RTOL_TEXT, atol=1e-12)
    xc = _read_dat(out / "X.dat")
    X = want["X"]
    np.testing.assert_allclose(xc[-1], 0.5 * (X[1:] + X[:-1]), rtol=RTOL_TEXT, atol=1e-12)
    np.testing.assert_allclose(xc[0], (np.arange(400) + 0.5) / 400, rtol=RTOL_TEXT)
