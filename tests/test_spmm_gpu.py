"""V:N:M SpMM on tcgen05 against the FP64 oracle (orc_spmm_f64).

Error measure: max |C - C64| / max |C64| (normwise), tolerance 1e-2 as the
north star states for BF16/FP16 operands with FP32 accumulation."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
TOL = 1e-2


def _run(ctx, nr, r, c, v, M, V, n, dtype, seed=0):
    import torch
    import vnm_gb300
    tdt = torch.bfloat16 if dtype == "bf16" else torch.float16
    g = torch.Generator().manual_seed(seed)
    B = torch.randn((nr, n), generator=g).to(tdt)
    A = vnm_gb300.SpmmMatrix(ctx, nr, r, c, v, M, V, dtype)
    C = A.run(B.cuda()).cpu().numpy().astype(np.float64)
    ref = oracle.spmm_f64(nr, r, c, v.astype(np.float64), B.float().numpy().astype(np.float64))
    err = np.abs(C - ref).max() / max(np.abs(ref).max(), 1e-30)
    return err, A.info()


def test_spmm_identity_is_exact(ctx):
    nr = 256
    idx = np.arange(nr, dtype=np.int32)
    err, info = _run(ctx, nr, idx, idx, np.ones(nr, np.float32), 4, 64, 128, "bf16")
    assert err < 1e-6, err
    assert info["slices"] == info["blocks"] == info["valid_blocks"]


@pytest.mark.parametrize("dtype", ["bf16", "fp16"])
@pytest.mark.parametrize("n", [64, 128, 256])
def test_spmm_random_matches_fp64(ctx, dtype, n):
    from vnm_gb300 import synth
    nr, r, c, v = synth.uniform(384, 0.03, 5)
    err, info = _run(ctx, nr, r, c, v, 8, 32, n, dtype)
    assert err < TOL, (err, info)


def test_spmm_rmat_blocks_that_violate_vnm(ctx):
    from vnm_gb300 import synth
    nr, r, c, v = synth.rmat(11, 12000, 9, "normal")   # dense hubs: many blocks need extra slices
    err, info = _run(ctx, nr, r, c, v, 4, 64, 128, "bf16")
    assert info["slices"] > info["valid_blocks"]
    assert err < TOL, (err, info)


def test_spmm_partial_last_tile_and_empty_tiles(ctx):
    nr = 328   # 3 tiles, the last one partly outside the matrix
    r = np.array([0, 5, 130, 300, 327], np.int32)
    c = np.array([3, 320, 9, 4, 327], np.int32)
    v = np.array([1.5, -2.0, 0.25, 3.0, -1.0], np.float32)
    err, info = _run(ctx, nr, r, c, v, 8, 64, 64, "bf16")
    assert err < TOL


@pytest.mark.parametrize("width", [64, 128, 256])
def test_spmm_every_column_block_width(ctx, width):
    """The kernel's column-block widths (the call picks one by timing) each
    match the FP64 oracle; VNM_SPMM_WIDTH fixes the width."""
    import os
    from vnm_gb300 import synth
    old = os.environ.get("VNM_SPMM_WIDTH")
    os.environ["VNM_SPMM_WIDTH"] = str(width)
    try:
        nr, r, c, v = synth.rmat(10, 1024 * 6, 9, "normal")
        err, info = _run(ctx, nr, r, c, v, 8, 64, 256, "bf16")
        assert err < TOL, (width, err)
    finally:
        if old is None:
            os.environ.pop("VNM_SPMM_WIDTH", None)
        else:
            os.environ["VNM_SPMM_WIDTH"] = old


def test_storage_reuse_and_operand_outliving_its_context():
    """A freed operand's storage serves the context's next compression (a
    smaller matrix in a larger block, results still the oracle's), and an
    operand freed after its context is destroyed is released cleanly."""
    import torch
    import vnm_gb300
    from vnm_gb300 import synth
    c2 = vnm_gb300.Context(0)
    big = synth.uniform(2048, 0.01, 11)
    small = synth.uniform(384, 0.03, 12)
    nr, r, c, v = big
    vnm_gb300.SpmmMatrix(c2, nr, r, c, v, 8, 32, "bf16").close()
    err, _ = _run(c2, *small, 8, 32, 128, "bf16")
    assert err <= TOL, err
    nr, r, c, v = small
    A = vnm_gb300.SpmmMatrix(c2, nr, r, c, v, 8, 32, "bf16")
    B = torch.randn((nr, 64)).to(torch.bfloat16).cuda()
    C = A.run(B).cpu().numpy().astype(np.float64)
    c2.close()
    ref = oracle.spmm_f64(nr, r, c, v.astype(np.float64), B.float().cpu().numpy().astype(np.float64))
    assert np.abs(C - ref).max() / max(np.abs(ref).max(), 1e-30) <= TOL
    A.close()


def test_host_outputs_given_by_the_caller(ctx):
    """permute_coo and SpmmMatrix.run fill caller-given (pinned) host arrays
    with the same results they return otherwise."""
    import torch
    import vnm_gb300
    from vnm_gb300 import synth
    nr, r, c, v = synth.uniform(512, 0.02, 21)
    newpos = np.random.default_rng(3).permutation(nr).astype(np.int32)
    pr, pc = ctx.permute_coo(nr, r, c, newpos)
    orow = torch.empty(len(r), dtype=torch.int32).pin_memory().numpy()
    ocol = torch.empty(len(c), dtype=torch.int32).pin_memory().numpy()
    qr, qc = ctx.permute_coo(nr, r, c, newpos, out=(orow, ocol))
    assert qr is orow and qc is ocol
    assert np.array_equal(qr, pr) and np.array_equal(qc, pc) and np.array_equal(pr, newpos[r])
    B = torch.randn((nr, 64)).to(torch.bfloat16).view(torch.int16).numpy()
    A = vnm_gb300.SpmmMatrix(ctx, nr, pr, pc, v, 8, 32, "bf16")
    C0 = A.run(B)
    hC = torch.full((nr, 64), float("nan")).pin_memory().numpy()
    C1 = A.run(B, C=hC)
    assert C1 is hC and np.array_equal(C0, C1)
    A.close()
