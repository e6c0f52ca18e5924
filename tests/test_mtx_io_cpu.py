"""The library's Matrix Market reader and writer (host code, no GPU).

The reader parses regular files (one entry per line) on all host threads
with its own integer and decimal parsers and sorts them in parallel; it
falls back to a token-by-token reader (fscanf's semantics,
mtx/readMtx.hpp:84-147) and to std::sort (customSort, mtx/readMtx.hpp:56-82)
where that could change the result.  Each case is read both ways
(VNM_MTX_READER=scalar forces the fallbacks, in a child process since the
switch is read per call) and must agree bit for bit, and with the oracle's
reader where the oracle defines the case."""
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(REPO, "vnm-graph-reordering_gb300", "libvnm_gb300.so")

pytestmark = pytest.mark.skipif(not os.path.exists(LIB), reason="libvnm_gb300.so not built")

_CHILD = r'''
import sys, numpy as np
sys.path.insert(0, sys.argv[1])
import vnm_gb300
nr, nc, r, c, v = vnm_gb300.read_mtx(sys.argv[2], int(sys.argv[3]))
np.savez(sys.argv[4], nr=nr, nc=nc, r=r, c=c, v=v)
'''


def _read(path, aligned, scalar, tmp):
    out = str(tmp / ("scalar.npz" if scalar else "fast.npz"))
    env = dict(os.environ)
    env.pop("VNM_MTX_READER", None)
    if scalar:
        env["VNM_MTX_READER"] = "scalar"
    r = subprocess.run([sys.executable, "-c", _CHILD, os.path.join(REPO, "vnm-graph-reordering_gb300"), path,
                        str(aligned), out], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    d = np.load(out)
    return int(d["nr"]), int(d["nc"]), d["r"], d["c"], d["v"]


def _same(a, b):
    assert a[0] == b[0] and a[1] == b[1]
    for x, y in zip(a[2:], b[2:]):
        assert x.dtype == y.dtype and np.array_equal(x.view(np.uint32) if x.dtype == np.float32 else x,
                                                     y.view(np.uint32) if y.dtype == np.float32 else y)


def _write(path, text):
    with open(path, "w", newline="") as f:
        f.write(text)
    return str(path)


def _general(n, rows, cols, vals, fmt="%.6g", field="real", nz=None, crlf=False, pad=""):
    eol = "\r\n" if crlf else "\n"
    lines = ["%%%%MatrixMarket matrix coordinate %s general" % field, "%d %d %d" % (n, n, len(rows) if nz is None else nz)]
    for r, c, v in zip(rows, cols, vals):
        if field == "pattern":
            lines.append("%s%d %d" % (pad, r + 1, c + 1))
        elif field == "integer":
            lines.append("%s%d %d %d" % (pad, r + 1, c + 1, int(v)))
        else:
            lines.append(("%s%d %d " + fmt) % (pad, r + 1, c + 1, v))
    return eol.join(lines) + eol


def _rand(n, nnz, seed, dup=False):
    rng = np.random.default_rng(seed)
    idx = rng.choice(n * n, nnz, replace=dup)
    rng.shuffle(idx)
    return (idx // n).astype(np.int64), (idx % n).astype(np.int64), rng.standard_normal(nnz) * 10.0 ** rng.integers(-9, 9, nnz)


CASES = {
    "general_g6": lambda: _general(300, *_rand(300, 4000, 1)),
    "general_many_digits": lambda: _general(300, *_rand(300, 4000, 2), fmt="%.17g"),
    "general_e_format": lambda: _general(300, *_rand(300, 4000, 3), fmt="%.3e"),
    "general_fixed": lambda: _general(300, *_rand(300, 4000, 4), fmt="%.9f"),
    "crlf_and_indent": lambda: _general(200, *_rand(200, 900, 5), crlf=True, pad="  "),
    "pattern": lambda: _general(200, *_rand(200, 900, 6), field="pattern"),
    "integer": lambda: _general(200, *_rand(200, 900, 7), field="integer"),
    "repeats": lambda: _general(64, *_rand(64, 900, 8, dup=True)),
    "more_entries_than_promised": lambda: _general(100, *_rand(100, 500, 9), nz=300),
    "fewer_entries_than_promised": lambda: _general(100, *_rand(100, 300, 10), nz=500),
    "comment_in_body": lambda: _general(100, *_rand(100, 300, 11)).replace("\n5 ", "\n% note\n5 ", 1),
    "special_tokens": lambda: ("%%MatrixMarket matrix coordinate real general\n4 4 5\n1 1 inf\n2 2 -0\n"
                               "3 3 0x1p-3\n4 4 1e-45\n1 4 +.5\n"),
    "split_lines": lambda: "%%MatrixMarket matrix coordinate real general\n3 3 3\n1 1\n2.5\n2 2 1.5 3 3\n-1\n",
    "symmetric": lambda: _general(150, *_rand(150, 800, 12)).replace("general", "symmetric", 1),
    "big_threaded": lambda: _general(20000, *_rand(20000, 300000, 13)),
    "big_threaded_symmetric": lambda: _general(20000, *_rand(20000, 200000, 14)).replace("general", "symmetric", 1),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_fast_reader_matches_token_reader(tmp_path, name):
    p = _write(tmp_path / (name + ".mtx"), CASES[name]())
    for aligned in (1, 8):
        _same(_read(p, aligned, False, tmp_path), _read(p, aligned, True, tmp_path))


@pytest.mark.parametrize("name", ["general_g6", "general_e_format", "pattern", "integer", "symmetric",
                                  "big_threaded", "big_threaded_symmetric", "crlf_and_indent"])
def test_fast_reader_matches_oracle(tmp_path, name):
    p = _write(tmp_path / (name + ".mtx"), CASES[name]())
    got = _read(p, 8, False, tmp_path)
    want = oracle.read_mtx(p, 8)
    _same(got, want)


def test_writer_matches_oracle_writer(tmp_path):
    import vnm_gb300
    rng = np.random.default_rng(3)
    n = 5000
    r, c, v = rng.integers(0, n, 200000), rng.integers(0, n, 200000), (rng.standard_normal(200000) * 3).astype(np.float32)
    v[:5] = [0.125, -0.125, 0.005, -0.004999, 1e30]  # ties and edges of "%.2f"
    a, b = str(tmp_path / "lib.mtx"), str(tmp_path / "orc.mtx")
    vnm_gb300.write_mtx(a, n, n, r, c, v)
    oracle.write_mtx(b, n, n, r, c, v)
    assert open(a).read() == open(b).read()
