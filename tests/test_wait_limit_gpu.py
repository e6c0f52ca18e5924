"""A bounded wait inside the round kernel (or the tensor-core SpMM) that
runs out fails the job (or the call) with VNM_ERR_INTERNAL instead of
hanging, and the context keeps working.

The walk (one warp) waits for the swap heaps' pops with a poll limit.  The
test hooks VNM_NM_TEST_HOLD_HEAPS=1 (the heaps publish nothing: a flag that
nothing sets) and VNM_NM_TEST_WAIT_LIMIT (a small limit) make the wait run
out on a matrix whose first round must wait: one invalid segment, so the
walk pairs it with the emptiest segment and waits for that pair's first pop
(reorder/reorder.h:1837-1860).  The round kernel has no bulk or
asynchronous copies in flight while the walk waits."""
import os

import numpy as np
import pytest

import oracle
from golden_cases import nm_input

pytestmark = pytest.mark.gpu


class _env:
    def __init__(self, **kv):
        self.kv = kv

    def __enter__(self):
        self.old = {k: os.environ.get(k) for k in self.kv}
        os.environ.update({k: str(v) for k, v in self.kv.items()})

    def __exit__(self, *a):
        for k, v in self.old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def _one_invalid_segment():
    nr = 64
    r = np.array([5, 5, 5, 9], np.int32)   # row 5 holds three nodes of segment 0 at 2:4
    c = np.array([0, 1, 2, 40], np.int32)
    return nr, r, c, np.ones(4, np.float32)


@pytest.mark.parametrize("cluster", ["1", "8"])
def test_walk_wait_that_runs_out_fails_the_job(ctx, goldens, cluster):
    import vnm_gb300
    nr, r, c, v = _one_invalid_segment()
    with _env(VNM_NM_CLUSTER=cluster):
        ores, _, _, opos = oracle.nm_run(nr, r, c, v, 2, 4, 0)
        res, pos = ctx.nm_reorder(nr, r, c, v, 2, 4, 0)   # without the hooks: the oracle's result
        assert np.array_equal(res, ores) and np.array_equal(pos, opos)
        with _env(VNM_NM_TEST_HOLD_HEAPS=1, VNM_NM_TEST_WAIT_LIMIT=4096):
            with pytest.raises(vnm_gb300.VnmError) as e:
                ctx.nm_reorder(nr, r, c, v, 2, 4, 0)
            assert e.value.status == 6  # VNM_ERR_INTERNAL
            with pytest.raises(vnm_gb300.VnmError) as e:
                ctx.nm_search(nr, r, c, v, 2, 4)
            assert e.value.status == 6
        # the same context afterwards: results as before, and on a golden case
        res, pos = ctx.nm_reorder(nr, r, c, v, 2, 4, 0)
        assert np.array_equal(res, ores) and np.array_equal(pos, opos)
        gnr, gr, gc, gv = nm_input(goldens, "rmat_1024__n2_m4")
        for s in range(4):
            ores, _, _, opos = oracle.nm_run(gnr, gr, gc, gv, 2, 4, s)
            res, pos = ctx.nm_reorder(gnr, gr, gc, gv, 2, 4, s)
            assert np.array_equal(res, ores) and np.array_equal(pos, opos), s


def test_spmm_pipeline_wait_that_runs_out_fails_the_call(ctx):
    """The tensor-core SpMM's pipeline waits (copies -> MMA, MMA -> copies)
    with a limit of one poll (test hook VNM_SPMM_TEST_WAIT_LIMIT): the
    kernel stops issuing, lets the copies in flight land (that wait keeps
    its full limit), skips the epilogue and reports VNM_ERR_INTERNAL; the
    same operand afterwards gives the oracle's product."""
    import torch
    import vnm_gb300
    from vnm_gb300 import synth
    nr, r, c, v = synth.vnm_structured(1024, 8, 128, seed=5)  # 32 K-steps a tile: more than the stages
    B = torch.randn((nr, 128), generator=torch.Generator().manual_seed(2)).to(torch.bfloat16)
    ref = oracle.spmm_f64(nr, r, c, v.astype(np.float64), B.float().numpy().astype(np.float64))
    with _env(VNM_SPMM_DENSE_MIN=0):
        A = vnm_gb300.SpmmMatrix(ctx, nr, r, c, v, 8, 128, "bf16")
    assert A.info()["residual_nnz"] == 0 and A.info()["ksteps"] > 8
    Bd = B.cuda()
    C = A.run(Bd).cpu().numpy().astype(np.float64)  # also picks the column-block width
    assert oracle.rowwise_rel_err(C, ref) < 1e-2
    with _env(VNM_SPMM_TEST_WAIT_LIMIT=1):
        with pytest.raises(vnm_gb300.VnmError) as e:
            A.run(Bd)
        assert e.value.status == 6  # VNM_ERR_INTERNAL
    C = A.run(Bd).cpu().numpy().astype(np.float64)
    assert oracle.rowwise_rel_err(C, ref) < 1e-2
    A.close()
