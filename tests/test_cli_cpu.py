"""The drop-in `spmm` command's argument and input errors, which it reports
before touching a GPU: a missing matrix file prints the reference's message
("File <name> not found", mtx/readMtx.hpp:370-373) and exits 1, and N/M/V
values the kernels cannot take are refused."""
import os
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SPMM = os.path.join(REPO, "vnm-graph-reordering_gb300", "spmm")


def _run(args, cwd):
    if not os.path.exists(SPMM):
        pytest.skip("the spmm command is not built (python __graft_entry__.py build)")
    return subprocess.run([SPMM] + args, cwd=cwd, capture_output=True, text=True, timeout=60)


def test_missing_file(tmp_path):
    r = _run(["--mtxfile", "nope.mtx", "--outmtxfile", "o.mtx", "--maxiter", "2", "--n", "64", "--sched", "0",
              "--v", "32"], str(tmp_path))
    assert r.returncode == 1
    assert r.stdout.strip() == "File nope.mtx not found"
    assert not os.path.exists(tmp_path / "o.mtx")


@pytest.mark.parametrize("extra", [["--M", "9"], ["--N", "8"], ["--N", "0"], ["--v", "0"]])
def test_refused_parameters(tmp_path, extra):
    p = tmp_path / "a.mtx"
    p.write_text("%%MatrixMarket matrix coordinate real general\n8 8 1\n1 1 1.0\n")
    args = ["--mtxfile", str(p), "--outmtxfile", "o.mtx", "--maxiter", "1", "--v", "32"]
    r = _run(args + extra if "--v" not in extra else args[:-2] + extra, str(tmp_path))
    assert r.returncode == 1 and "need 1 <= N < M <= 8" in r.stderr


def test_bench_flags():
    """bench.py parses its flags without a GPU (the measured runs need one)."""
    import sys
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--help"], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    for flag in ("--gpus", "--steps", "--warmup", "--impl", "--no-cpu-baseline", "--no-extended", "--c5-spmm-only"):
        assert flag in r.stdout
