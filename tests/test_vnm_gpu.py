"""Parity of the CUDA VNM stage with reordering.py (golden outputs of the
reference script, tests/golden/vnm_ref_goldens.npz) and with the oracle."""
import os

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def vg():
    return np.load(os.path.join(REPO, "tests", "golden", "vnm_ref_goldens.npz"))


def _case(g, case):
    name, mv = case.split("__")
    M, V = int(mv.split("_")[0][1:]), int(mv.split("_")[1][1:])
    n = int(g["in__%s__n" % name])
    return name, M, V, n, g["in__%s__row" % name], g["in__%s__col" % name]


def test_vnm_eval_matches_reordering_py(ctx, vg):
    for case in vg["cases"].tolist():
        name, M, V, n, r, c = _case(vg, case)
        assert ctx.vnm_eval(n, n, r, c, M, V).tolist() == vg["eval__" + case].tolist(), case


def test_vnm_reorder_matches_reordering_py(ctx, vg):
    for case in vg["cases"].tolist():
        name, M, V, n, r, c = _case(vg, case)
        out5, r2, c2, newpos = ctx.vnm_reorder(n, n, r, c, M, V)
        assert out5.tolist() == vg["out__" + case].tolist(), case
        want = set(zip(vg["wrow__" + case].tolist(), vg["wcol__" + case].tolist()))
        assert set(zip(r2.tolist(), c2.tolist())) == want, case


def test_vnm_reorder_matches_oracle_larger(ctx):
    from vnm_gb300 import synth
    for (nr, r, c, v), M, V in ((synth.rmat(12, 20000, 41, "uniform"), 8, 32),
                                (synth.rmat(13, 60000, 42, "uniform"), 4, 64),
                                (synth.uniform(3000, 0.004, 43), 8, 128)):
        out5, r2, c2, pos = ctx.vnm_reorder(nr, nr, r, c, M, V)
        o5, or2, oc2, opos = oracle.vnm_run(nr, nr, r, c, M, V)
        assert out5.tolist() == o5.tolist(), (nr, M, V)
        assert np.array_equal(r2, or2) and np.array_equal(c2, oc2)
        assert np.array_equal(pos, opos)
