"""The drop-in `spmm` command against the oracle's emulation of the
reference command (find_best_2toX + hybrid_reordering with its file round
trips): the 15 CSV fields other than the time, and the output .mtx text."""
import os
import subprocess

import numpy as np
import pytest

import oracle
from golden_cases import nm_input

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SPMM = os.path.join(REPO, "vnm-graph-reordering_gb300", "spmm")


def _cli(tmp_path, mtx, N, M, V, maxiter):
    out = str(tmp_path / "out.mtx")
    r = subprocess.run([SPMM, "--mtxfile", mtx, "--outmtxfile", out, "--maxiter", str(maxiter), "--n", "64",
                        "--sched", "0", "--v", str(V), "--N", str(N), "--M", str(M)],
                       cwd=str(tmp_path), capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    fields = [float(x) for x in r.stdout.strip().split(",")]
    with open(out) as f:
        text = f.read()
    return fields, text


def _oracle(tmp_path, mtx, N, M, V, maxiter):
    csv, best, nr, r, c, v = oracle.spmm_cli(mtx, N, M, V, maxiter)
    p = str(tmp_path / "oracle_out.mtx")
    oracle.write_mtx(p, nr, nr, r, c, v)
    with open(p) as f:
        return csv, f.read()


def _write_input(tmp_path, name, nr, r, c, v):
    from vnm_gb300 import synth
    p = str(tmp_path / (name + ".mtx"))
    synth.write_mtx(p, nr, r, c, v)
    return p


CASES = [("u256", 2, 8, 32, 2), ("u256", 2, 4, 64, 1), ("rmat1k", 2, 8, 32, 3), ("fixture_lund", 2, 8, 32, 2),
         ("fixture_gd95", 2, 8, 4, 2), ("sym96", 2, 8, 8, 2), ("u256", 2, 8, 32, 0)]


@pytest.mark.parametrize("name,N,M,V,maxiter", CASES)
def test_cli_matches_oracle(tmp_path, goldens, name, N, M, V, maxiter):
    from vnm_gb300 import synth
    if name == "u256":
        mtx = _write_input(tmp_path, name, *synth.uniform(256, 0.05, 3))
    elif name == "rmat1k":
        mtx = _write_input(tmp_path, name, *synth.rmat(10, 4096, 5, "uniform"))
    elif name == "sym96":
        n, r, c, v = synth.rmat(7, 300, 22, "uniform", R=96)
        lo, hi = np.minimum(r, c), np.maximum(r, c)
        v = np.round(np.sin(lo * 7.0 + hi * 3.0) * 0.9, 2).astype(np.float32)  # symmetric values
        mtx = _write_input(tmp_path, name, n, r, c, v)
    else:
        key = {"fixture_lund": "lund_b__n2_m8", "fixture_gd95": "GD95_a__n2_m8"}[name]
        nr, r, c, v = nm_input(goldens, key)
        mtx = _write_input(tmp_path, name, nr, r, c, v)
    fields, text = _cli(tmp_path, mtx, N, M, V, maxiter)
    ocsv, otext = _oracle(tmp_path, mtx, N, M, V, maxiter)
    assert len(fields) == 16
    np.testing.assert_allclose(fields[:15], ocsv[:15], rtol=1e-5, atol=1e-6)
    assert text == otext
