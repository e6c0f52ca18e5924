"""PyTorch op around the V:N:M SpMM, for GCN-style neighbourhood aggregation.

The reference's GNN scripts aggregate node features with a sparse
adjacency (the role of `gnn/single/pyg_gcn.py`).  Here the adjacency is
compressed once into the V:N:M operand of the tensor-core SpMM
(`vnm_spmm_compress`) and every aggregation is one `vnm_spmm_run`:

    adj = VnmAdjacency(ctx, n, row, col, val, M=8, V=128)   # reordered COO
    Y = vnm_spmm(adj, X)                                      # Y = A @ X, autograd-aware

Forward: X (n x F, any float dtype, CUDA) is rounded to the operand's
16-bit type, padded to a multiple of 64 columns, multiplied with FP32
accumulation, and returned as FP32.  Backward: dX = A^T dY through a
second operand built from the transposed pattern, or through the same
operand when the adjacency is symmetric (the normalised adjacency
D^-1/2 A D^-1/2 of an undirected graph is).

Every aggregation is enqueued on PyTorch's current stream of X's device
(vnm_spmm_run_async) after the work that produced X, and the op returns
without waiting for it, so a training loop does not stall the host at each
layer.  The first aggregation of an operand shape and feature width times
the kernel's widths once (a one-time wait).
"""
import numpy as np

from . import SpmmMatrix


def _pad_cols(X, mult=64):
    import torch
    n, F = X.shape
    Fp = (F + mult - 1) // mult * mult
    if Fp == F:
        return X.contiguous(), F
    out = torch.zeros((n, Fp), dtype=X.dtype, device=X.device)
    out[:, :F] = X
    return out, F


def _host(a, dtype):
    if hasattr(a, "detach"):
        a = a.detach().cpu().numpy()
    return np.ascontiguousarray(a, dtype=dtype)


def _sorted_coo(r, c, v):
    o = np.lexsort((c, r))
    return r[o], c[o], v[o]


class VnmAdjacency:
    """A square sparse matrix (COO, any order) compressed for the SpMM,
    with its transpose for the backward pass."""

    def __init__(self, ctx, n, row, col, val, M=8, V=128, dtype="bf16", symmetric=None):
        r, c, v = _host(row, np.int32), _host(col, np.int32), _host(val, np.float32)
        if symmetric is None:  # same entries with the same values both ways
            a = _sorted_coo(r, c, v)
            b = _sorted_coo(c, r, v)
            symmetric = all(np.array_equal(x, y) for x, y in zip(a, b))
        self.n, self.dtype, self.symmetric = n, dtype, bool(symmetric)
        self.fwd = SpmmMatrix(ctx, n, r, c, v, M, V, dtype)
        self.bwd = self.fwd if self.symmetric else SpmmMatrix(ctx, n, c, r, v, M, V, dtype)

    @property
    def torch_dtype(self):
        import torch
        return torch.bfloat16 if self.dtype == "bf16" else torch.float16

    def matmul(self, X, transpose=False):
        """A @ X (or A^T @ X) as FP32, X an n x F CUDA tensor."""
        import torch
        assert X.is_cuda and X.dim() == 2 and X.shape[0] == self.n
        Xp, F = _pad_cols(X.detach().to(self.torch_dtype))
        Y = (self.bwd if transpose else self.fwd).run_async(Xp, stream=torch.cuda.current_stream(X.device))
        return Y[:, :F] if Y.shape[1] != F else Y

    def close(self):
        if self.bwd is not self.fwd:
            self.bwd.close()
        self.fwd.close()


def _function():
    import torch

    class VnmSpmm(torch.autograd.Function):
        @staticmethod
        def forward(fctx, X, adj):
            fctx.adj = adj
            fctx.in_dtype = X.dtype
            return adj.matmul(X)

        @staticmethod
        def backward(fctx, dY):
            dX = fctx.adj.matmul(dY, transpose=True).to(fctx.in_dtype)
            return dX, None

    return VnmSpmm


_FN = None


def vnm_spmm(adj, X):
    """Y = A @ X on the tensor cores, differentiable in X."""
    global _FN
    if _FN is None:
        _FN = _function()
    return _FN.apply(X, adj)


def gcn_layer(adj, H, W, bias=None):
    """One GCN layer, relu(A (H W) + b): the dense product on cuBLAS, the
    aggregation on the V:N:M SpMM."""
    import torch
    Y = vnm_spmm(adj, H @ W)
    if bias is not None:
        Y = Y + bias
    return torch.relu(Y)
