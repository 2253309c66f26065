"""The drivers' multi-threaded data-file reader and writer and the binary
format (hydrocode-fusion_gb300/host/hydro_fastio.c), on the CPU.

The reader must give the numbers strtod gives for each token (Python's float
is correctly rounded, as glibc's strtod is), the line/column counts and the
first error of the reference's one-pass getc reader
(src/file_io/io_control.c:163-261), whatever the number of threads; the
writer must write the bytes of one fprintf("%.10g\\t") per value."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "hydrocode-fusion_gb300")
SO = os.path.join(PKG, "_build", "libhydro_fastio.so")

VALFN = ctypes.CFUNCTYPE(ctypes.c_double, ctypes.c_void_p, ctypes.c_int, ctypes.c_int)


@pytest.fixture(scope="module")
def fio():
    subprocess.run(["make", "-s", "-C", PKG, "_build/libhydro_fastio.so"], check=True)
    L = ctypes.CDLL(SO)
    L.hio_read_table.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                 ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_longlong),
                                 ctypes.POINTER(ctypes.POINTER(ctypes.c_double))]
    L.hio_write_text.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, VALFN, ctypes.c_void_p]
    L.hio_bin_create.restype = ctypes.c_void_p
    L.hio_bin_create.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                 ctypes.POINTER(ctypes.c_double)]
    L.hio_bin_plane.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, VALFN, ctypes.c_void_p]
    L.hio_bin_read.argtypes = [ctypes.c_char_p] + [ctypes.POINTER(ctypes.c_int)] * 4 + \
        [ctypes.POINTER(ctypes.POINTER(ctypes.c_double))] * 2
    libc = ctypes.CDLL(None)
    libc.fopen.restype = ctypes.c_void_p
    libc.fopen.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
    libc.fclose.argtypes = [ctypes.c_void_p]
    libc.free.argtypes = [ctypes.c_void_p]
    libc.fflush.argtypes = [ctypes.c_void_p]
    return L, libc


def read(fio, path, threads, check=1):
    L, libc = fio
    os.environ["HYDRO_IO_THREADS"] = str(threads)
    try:
        lines, cols, cnt = ctypes.c_int(), ctypes.c_int(), ctypes.c_longlong()
        ptr = ctypes.POINTER(ctypes.c_double)()
        rc = L.hio_read_table(str(path).encode(), check, ctypes.byref(lines), ctypes.byref(cols), ctypes.byref(cnt),
                              ctypes.byref(ptr))
        data = None
        if rc == 0:
            data = np.ctypeslib.as_array(ptr, shape=(cnt.value,)).copy() if cnt.value else np.zeros(0)
            libc.free(ptr)
        return rc, lines.value, cols.value, data
    finally:
        del os.environ["HYDRO_IO_THREADS"]


def make_table(rng, nl, nc):
    vals = rng.standard_normal((nl, nc)) * np.exp(rng.uniform(-30, 30, (nl, nc)))
    fmts = ["{:.17g}", "{:.10g}", "{:.3e}", "{:.6f}"]
    rows = []
    for r in range(nl):
        # the reference's reader takes no '+' (io_control.c:190-199): exponents are written e05, e-05
        toks = [fmts[(r + c) % 4].format(vals[r, c]).replace("e+", "e") for c in range(nc)]
        sep = ["\t", " ", "  \t "][r % 3]
        rows.append(sep.join(toks))
    return rows


@pytest.mark.parametrize("threads", [1, 3, 8, 16])
def test_reader_values_and_shape(fio, tmp_path, threads):
    rng = np.random.default_rng(5)
    rows = make_table(rng, 240, 301)
    text = ""
    for r, row in enumerate(rows):
        text += row + ("\r\n" if r % 7 == 0 else "\n")
        if r % 50 == 3:
            text += "   \t\n\n"  # blank lines are not lines of the table
    text = text.rstrip("\n")  # no newline after the last number: still read
    p = tmp_path / "RHO.txt"
    p.write_text(text)
    rc, nl, nc, data = read(fio, p, threads)
    assert rc == 0 and nl == 240 and nc == 301
    want = np.array([float(t) for row in rows for t in row.split()])
    assert np.array_equal(data, want)


def test_reader_errors_match_across_threads(fio, tmp_path, capfd):
    rng = np.random.default_rng(6)
    rows = make_table(rng, 400, 64)
    cases = {}
    bad = list(rows)
    bad[311] = bad[311] + " 1.0x"
    cases["illegal"] = ("\n".join(bad) + "\n", 1, "illigal character(ASCII=120, flag=1)")
    bad = list(rows)
    bad[257] = bad[257] + " 2.5"
    cases["columns"] = ("\n".join(bad) + "\n", 2, "line=257, column=65, n_x=64")
    bad = list(rows)
    bad[300] = "1.2.3 " + " ".join(bad[300].split()[1:])
    cases["entry"] = ("\n".join(bad) + "\n", 3, "The 19201th entry")
    bad = list(rows)
    bad[10] = "1e999 " + " ".join(bad[10].split()[1:])
    cases["range"] = ("\n".join(bad) + "\n", 3, "The 641th entry")
    for name, (text, code, msg) in cases.items():
        p = tmp_path / f"{name}.txt"
        p.write_text(text)
        outs = []
        for t in (1, 8):
            rc, _, _, _ = read(fio, p, t)
            assert rc == code, (name, t, rc)
            fio[1].fflush(None)  # the C messages are in stdio's buffers until flushed
            outs.append(capfd.readouterr())
        assert outs[0] == outs[1], name
        assert msg in outs[0].out + outs[0].err, (name, outs[0])


def test_reader_counts_all_numbers_without_column_check(fio, tmp_path):
    """1D files: one number per line or all on one line; no column rule."""
    p = tmp_path / "P.txt"
    vals = np.linspace(-1, 1, 5001)
    p.write_text("\n".join(f"{v:.17g}" for v in vals[:2000]) + "\n" + " ".join(f"{v:.17g}" for v in vals[2000:]) + "\n")
    rc, nl, nc, data = read(fio, p, 4, check=0)
    assert rc == 0 and len(data) == 5001 and np.array_equal(data, vals)


@pytest.mark.parametrize("threads", [1, 5, 16])
def test_writer_bytes(fio, tmp_path, threads):
    L, libc = fio
    rng = np.random.default_rng(7)
    a = rng.standard_normal((97, 131)) * np.exp(rng.uniform(-40, 40, (97, 131)))
    a[3, 4] = 0.0
    a[5, 6] = -0.0
    a[7, 8] = np.inf
    a[9, 10] = 1e-310  # subnormal

    @VALFN
    def val(ctx, r, c):
        return float(a[r, c])

    p = tmp_path / f"out{threads}.dat"
    os.environ["HYDRO_IO_THREADS"] = str(threads)
    try:
        fp = libc.fopen(str(p).encode(), b"w")
        assert L.hio_write_text(fp, a.shape[0], a.shape[1], val, None) == 0
        libc.fclose(fp)
    finally:
        del os.environ["HYDRO_IO_THREADS"]
    want = "".join("".join("%.10g\t" % x for x in row) + "\n" for row in a)
    assert p.read_text() == want


def test_binary_round_trip(fio, tmp_path):
    L, libc = fio
    rng = np.random.default_rng(8)
    planes = rng.standard_normal((3, 20, 33))
    times = np.array([0.0, 0.125, 0.25])
    cur = {"k": 0}

    @VALFN
    def val(ctx, r, c):
        return float(planes[cur["k"], r, c])

    p = tmp_path / "RHO.bin"
    fp = L.hio_bin_create(str(p).encode(), 2, 33, 20, 3, times.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    assert fp
    for k in range(3):
        cur["k"] = k
        assert L.hio_bin_plane(fp, 20, 33, val, None) == 0
    libc.fclose(fp)
    raw = p.read_bytes()
    assert raw[:8] == b"HCFBIN01"
    assert list(np.frombuffer(raw[8:28], "<i4")) == [2, 33, 20, 3, 0]
    assert np.array_equal(np.frombuffer(raw[28:52], "<f8"), times)
    assert np.array_equal(np.frombuffer(raw[52:], "<f8").reshape(3, 20, 33), planes)
    dims = [ctypes.c_int() for _ in range(4)]
    tp, dp = ctypes.POINTER(ctypes.c_double)(), ctypes.POINTER(ctypes.c_double)()
    assert L.hio_bin_read(str(p).encode(), *[ctypes.byref(d) for d in dims], ctypes.byref(tp), ctypes.byref(dp)) == 0
    assert [d.value for d in dims] == [2, 33, 20, 3]
    assert np.array_equal(np.ctypeslib.as_array(dp, shape=(3 * 20 * 33,)).reshape(3, 20, 33), planes)
    libc.free(tp)
    libc.free(dp)
    (tmp_path / "bad.bin").write_bytes(b"NOTAFILE" + raw[8:])
    assert L.hio_bin_read(str(tmp_path / "bad.bin").encode(), *[ctypes.byref(d) for d in dims], ctypes.byref(tp),
                          ctypes.byref(dp)) == 4
