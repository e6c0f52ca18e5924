"""Batched NM reorder: one persistent launch for many matrices of uneven
size; every matrix's result must equal its own standalone run (and the
oracle's) bit for bit."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def test_batch_equals_per_matrix_runs(ctx):
    from vnm_gb300 import synth
    # rows padded to a multiple of M, as Mtx::init_from_file does
    mats = [((nr + 7) // 8 * 8, r, c, v) for nr, r, c, v in synth.rmat_batch(count=24, seed=77, lo=256, hi=2048)]
    for sched in (0, 3):
        res, pos = ctx.nm_reorder_batch(mats, 2, 8, sched)
        for b, (nr, r, c, v) in enumerate(mats):
            r1, p1 = ctx.nm_reorder(nr, r, c, v, 2, 8, sched)
            assert np.array_equal(res[b], r1), (b, sched)
            assert np.array_equal(pos[b], p1), (b, sched)
    for b in (0, 5, 11):
        nr, r, c, v = mats[b]
        ores, _, _, opos = oracle.nm_run(nr, r, c, v, 2, 8, 3)
        assert np.array_equal(res[b], ores) and np.array_equal(pos[b], opos)


def test_batch_reports_bad_matrix(ctx):
    import vnm_gb300
    from vnm_gb300 import synth
    mats = [synth.uniform(64, 0.05, 1), synth.uniform(64, 0.05, 2)]
    bad = (mats[1][0], mats[1][1][::-1].copy(), mats[1][2][::-1].copy(), mats[1][3])
    with pytest.raises(vnm_gb300.VnmError) as e:
        ctx.nm_reorder_batch([mats[0], bad], 2, 8, 0)
    assert e.value.status == 3
