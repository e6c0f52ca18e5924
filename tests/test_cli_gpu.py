"""The drop-in `spmm` command against the reference's own command and the
oracle's emulation of it.

Reference: tests/golden/cli_ref_goldens.npz holds what the reference's
`spmm` (main.cu built from its sources, its VNM stage the real
reordering.py) printed and wrote on each case, with temp.mtx in its working
directory a copy of the input (main.cu:207 evaluates whatever temp.mtx is
there first).  The drop-in runs in a directory prepared the same way; its 15
CSV fields other than the time and its output .mtx text must match, with the
schedule fixed (VNM_SPMM_SCHED) to one of those tied at the largest improve
rate: the reference breaks that tie by measured wall time (main.cu:90-99).
Oracle: orc_spmm_cli, which composes the oracle's pinned pieces with the
file round trips, on the same cases plus --maxiter 0 (which the reference
cannot run: it indexes an empty vector, main.cu:331)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle
from golden_cases import CLI_CASES, cli_input, tied_schedules

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SPMM = os.path.join(REPO, "vnm-graph-reordering_gb300", "spmm")
REF = os.path.join(REPO, "tests", "golden", "cli_ref_goldens.npz")


def _cli(wd, mtx, N, M, V, maxiter, sched=None):
    out = os.path.join(wd, "out.mtx")
    env = dict(os.environ)
    if sched is not None:
        env["VNM_SPMM_SCHED"] = str(sched)
    r = subprocess.run([SPMM, "--mtxfile", mtx, "--outmtxfile", out, "--maxiter", str(maxiter), "--n", "64",
                        "--sched", "0", "--v", str(V), "--N", str(N), "--M", str(M)],
                       cwd=wd, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr
    fields = [float(x) for x in r.stdout.strip().split(",")]
    with open(out) as f:
        text = f.read()
    return fields, text


def _write_input(wd, name, goldens, fname=None):
    from vnm_gb300 import synth
    p = os.path.join(wd, (fname or name) + ".mtx")
    synth.write_mtx(p, *cli_input(name, goldens))
    return p


@pytest.mark.parametrize("case,name,N,M,V,maxiter", CLI_CASES)
def test_cli_matches_oracle(tmp_path, goldens, case, name, N, M, V, maxiter):
    mtx = _write_input(str(tmp_path), name, goldens)
    fields, text = _cli(str(tmp_path), mtx, N, M, V, maxiter)
    csv, best, nr, r, c, v = oracle.spmm_cli(mtx, N, M, V, maxiter)
    p = str(tmp_path / "oracle_out.mtx")
    oracle.write_mtx(p, nr, nr, r, c, v)
    with open(p) as f:
        otext = f.read()
    assert len(fields) == 16
    np.testing.assert_allclose(fields[:15], csv[:15], rtol=1e-5, atol=1e-6)
    assert text == otext


@pytest.mark.parametrize("case", [c[0] for c in CLI_CASES if c[5] > 0])
def test_cli_matches_reference_command(tmp_path, goldens, case):
    if not os.path.exists(REF):
        pytest.skip("the reference command's goldens are not collected yet (tests/golden/make_cli_goldens.py)")
    g = np.load(REF)
    _, name, N, M, V, maxiter = next(c for c in CLI_CASES if c[0] == case)
    wd = str(tmp_path)
    mtx = _write_input(wd, name, goldens, fname="input")
    want = [float(x) for x in str(g["csv__" + case]).split(",")]
    matched = []
    for s in tied_schedules(mtx, N, M):
        shutil.copyfile(mtx, os.path.join(wd, "temp.mtx"))  # the stale file the first evaluation reads
        fields, text = _cli(wd, "input.mtx", N, M, V, maxiter, sched=s)
        assert len(fields) == len(want) == 16
        if np.allclose(fields[:15], want[:15], rtol=1e-5, atol=1e-6) and text.encode() == g["out__" + case].tobytes():
            matched.append(s)
    assert matched, case
