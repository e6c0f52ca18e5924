"""V:N:M SpMM on tcgen05 against the FP64 oracle (orc_spmm_f64).

Error measure: the largest per-row relative error
max_i ||C_i - C64_i||_inf / ||C64_i||_inf (oracle.rowwise_rel_err; a row whose
reference is zero must come out zero), tolerance 1e-2 for BF16/FP16
operands with FP32 accumulation.  Per row, so that a
low-degree row cannot hide behind the hub rows of a power-law graph."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
TOL = 1e-2


class _dense_min:
    """VNM_SPMM_DENSE_MIN for the operands compressed inside the block: 0
    puts every V:N:M block on the tensor cores, a huge value every block on
    the CUDA-core residual path."""

    def __init__(self, value):
        self.value = value

    def __enter__(self):
        import os
        self.old = os.environ.get("VNM_SPMM_DENSE_MIN")
        if self.value is None:
            os.environ.pop("VNM_SPMM_DENSE_MIN", None)
        else:
            os.environ["VNM_SPMM_DENSE_MIN"] = str(self.value)

    def __exit__(self, *a):
        import os
        if self.old is None:
            os.environ.pop("VNM_SPMM_DENSE_MIN", None)
        else:
            os.environ["VNM_SPMM_DENSE_MIN"] = self.old


TENSOR_ONLY, RESIDUAL_ONLY, DEFAULT = 0, 1 << 30, None


def _run(ctx, nr, r, c, v, M, V, n, dtype, seed=0):
    import torch
    import vnm_gb300
    tdt = torch.bfloat16 if dtype == "bf16" else torch.float16
    g = torch.Generator().manual_seed(seed)
    B = torch.randn((nr, n), generator=g).to(tdt)
    A = vnm_gb300.SpmmMatrix(ctx, nr, r, c, v, M, V, dtype)
    C = A.run(B.cuda()).cpu().numpy().astype(np.float64)
    ref = oracle.spmm_f64(nr, r, c, v.astype(np.float64), B.float().numpy().astype(np.float64))
    return oracle.rowwise_rel_err(C, ref), A.info()


@pytest.mark.parametrize("split", [TENSOR_ONLY, RESIDUAL_ONLY])
def test_spmm_identity_is_exact(ctx, split):
    nr = 256
    idx = np.arange(nr, dtype=np.int32)
    with _dense_min(split):
        err, info = _run(ctx, nr, idx, idx, np.ones(nr, np.float32), 4, 64, 128, "bf16")
    assert err < 1e-6, err
    if split == TENSOR_ONLY:
        assert info["slices"] == info["blocks"] == info["valid_blocks"] and info["residual_nnz"] == 0
    else:
        assert info["residual_nnz"] == nr and info["ksteps"] == 0


@pytest.mark.parametrize("split", [TENSOR_ONLY, RESIDUAL_ONLY, DEFAULT])
@pytest.mark.parametrize("dtype", ["bf16", "fp16"])
@pytest.mark.parametrize("n", [64, 128, 192, 256])
def test_spmm_random_matches_fp64(ctx, dtype, n, split):
    from vnm_gb300 import synth
    nr, r, c, v = synth.uniform(384, 0.03, 5)
    with _dense_min(split):
        err, info = _run(ctx, nr, r, c, v, 8, 32, n, dtype)
    assert err < TOL, (err, info)


def test_spmm_rmat_blocks_that_violate_vnm(ctx):
    from vnm_gb300 import synth
    nr, r, c, v = synth.rmat(11, 12000, 9, "normal")   # dense hubs: many blocks need extra slices
    with _dense_min(TENSOR_ONLY):
        err, info = _run(ctx, nr, r, c, v, 4, 64, 128, "bf16")
    assert info["slices"] > info["valid_blocks"]
    assert err < TOL, (err, info)


@pytest.mark.parametrize("n", [64, 128, 256])
def test_spmm_hybrid_split_and_hub_rows(ctx, n):
    """Dense blocks on the tensor cores, sparse ones on the CUDA cores in one
    product: R-MAT hubs plus three rows with 700-1900 nonzeros, which the
    residual path cuts into chunks and adds back in chunk order."""
    from vnm_gb300 import synth
    nr, r, c, v = synth.rmat(11, 12000, 9, "normal")  # 2048 rows
    rng = np.random.default_rng(2)
    extra_r = np.concatenate([np.full(1900, 7), np.full(1500, 700), np.full(700, 1999)])
    extra_c = np.concatenate([rng.choice(nr, 1900, replace=False), rng.choice(nr, 1500, replace=False),
                              rng.choice(nr, 700, replace=False)])
    key = np.unique(np.concatenate([r.astype(np.int64) * nr + c, extra_r.astype(np.int64) * nr + extra_c]))
    r, c = (key // nr).astype(np.int32), (key % nr).astype(np.int32)
    v = rng.standard_normal(len(r)).astype(np.float32)
    with _dense_min(4):
        err, info = _run(ctx, nr, r, c, v, 4, 64, n, "bf16")
    assert info["residual_nnz"] > 0 and info["tensor_tiles"] > 0 and info["split_chunks"] > 0, info
    assert err < TOL, (err, info)


@pytest.mark.parametrize("n", [64, 192, 256])
def test_spmm_row_of_hundreds_of_chunks(ctx, n):
    """A hub row of 60000 nonzeros (235 chunks of 256, more than a thread
    group of the partial-sum kernel covers in one pass at every n) beside
    short rows: per-row error against FP64, and two runs bit-identical
    (the partial rows are added in a fixed order)."""
    import torch
    import vnm_gb300
    nr = 65536
    rng = np.random.default_rng(11)
    hub_c = rng.choice(nr, 60000, replace=False)
    sr = rng.integers(0, nr, 200000)
    sc = rng.integers(0, nr, 200000)
    key = np.unique(np.concatenate([np.full(60000, 4321, np.int64) * nr + hub_c, sr.astype(np.int64) * nr + sc]))
    r, c = (key // nr).astype(np.int32), (key % nr).astype(np.int32)
    v = rng.standard_normal(len(r)).astype(np.float32)
    B = torch.randn((nr, n), generator=torch.Generator().manual_seed(3)).to(torch.bfloat16)
    with _dense_min(RESIDUAL_ONLY):
        A = vnm_gb300.SpmmMatrix(ctx, nr, r, c, v, 8, 64, "bf16")
    info = A.info()
    assert info["split_chunks"] >= 235, info
    Bd = B.cuda()
    C1 = A.run(Bd).cpu().numpy()
    C2 = A.run(Bd).cpu().numpy()
    assert np.array_equal(C1.view(np.uint32), C2.view(np.uint32))
    ref = oracle.spmm_f64(nr, r, c, v.astype(np.float64), B.float().numpy().astype(np.float64))
    err = oracle.rowwise_rel_err(C1.astype(np.float64), ref)
    assert err < TOL, (err, info)


@pytest.mark.parametrize("split", [TENSOR_ONLY, RESIDUAL_ONLY, 4])
def test_spmm_partial_last_tile_and_empty_tiles(ctx, split):
    nr = 328   # 3 tiles, the last one partly outside the matrix
    r = np.array([0, 5, 130, 300, 327], np.int32)
    c = np.array([3, 320, 9, 4, 327], np.int32)
    v = np.array([1.5, -2.0, 0.25, 3.0, -1.0], np.float32)
    with _dense_min(split):
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
        for split in (TENSOR_ONLY, 4):
            with _dense_min(split):
                err, info = _run(ctx, nr, r, c, v, 8, 64, 256, "bf16")
            assert err < TOL, (width, split, err)
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
    assert oracle.rowwise_rel_err(C, ref) <= TOL
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


@pytest.mark.parametrize("M", [2, 3, 5, 6, 7])
@pytest.mark.parametrize("split", [TENSOR_ONLY, RESIDUAL_ONLY])
def test_spmm_every_group_size(ctx, M, split):
    """Group sizes other than 4 and 8 (the compressor's sort keys hold the
    column inside a segment in ceil(log2 M) bits), on both paths."""
    rng = np.random.default_rng(M)
    nr = 13440  # a multiple of 128 and of every M
    idx = np.unique(rng.integers(0, nr * nr, 120000))
    r, c = (idx // nr).astype(np.int32), (idx % nr).astype(np.int32)
    v = rng.standard_normal(len(r)).astype(np.float32)
    with _dense_min(split):
        err, info = _run(ctx, nr, r, c, v, M, 32, 64, "bf16")
    assert err < TOL, (M, err, info)


@pytest.mark.parametrize("V", [32, 64, 128])
def test_full_vnm_blocks_go_to_the_tensor_cores(ctx, V):
    """A matrix in full V:2:8 form (every block 2V nonzeros): by default
    every block runs on the tensor cores, and the product matches FP64."""
    from vnm_gb300 import synth
    nr, r, c, v = synth.vnm_structured(512, 8, V, seed=V)
    err, info = _run(ctx, nr, r, c, v, 8, V, 128, "bf16")
    assert info["residual_nnz"] == 0 and info["valid_blocks"] == info["blocks"] == info["slices"], info
    assert info["tensor_tiles"] == info["tiles"]
    assert err < TOL, (err, info)
