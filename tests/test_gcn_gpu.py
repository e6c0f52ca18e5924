"""The PyTorch aggregation op over the V:N:M SpMM (vnm_gb300.gcn), checked
against a float64 scipy product of the same inputs: forward, the backward
pass (A^T dY) through the symmetric shortcut and through a transposed
operand, and one GCN layer.  Tolerance as for the SpMM itself: relative
error 1e-2 against float64 on BF16-rounded operands, per row for the
aggregation (oracle.rowwise_rel_err); the layer's ReLU output is compared
normwise, since ReLU turns entries near zero into exact zeros on one side
and not the other."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

TOL = 1e-2


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def _csr(n, r, c, v):
    import scipy.sparse as sp
    return sp.csr_matrix((v.astype(np.float64), (r, c)), shape=(n, n))


def _bf16(t):
    import torch
    return t.detach().to(torch.bfloat16).to(torch.float64).cpu().numpy()


def _graph(symmetric):
    from vnm_gb300 import synth
    n, r, c, v = synth.chung_lu(4096, 2.1, 10.0, 5)
    if not symmetric:
        v = np.random.default_rng(1).uniform(-1, 1, len(v)).astype(np.float32)
    return n, r, c, v


@pytest.mark.parametrize("symmetric", [True, False])
def test_forward_and_backward_match_float64(ctx, symmetric):
    import torch
    from vnm_gb300 import gcn
    n, r, c, v = _graph(symmetric)
    adj = gcn.VnmAdjacency(ctx, n, r, c, v, M=8, V=128)
    assert adj.symmetric == symmetric
    A = _csr(n, r, c, v)
    g = torch.Generator().manual_seed(3)
    X = torch.randn((n, 100), generator=g).cuda().requires_grad_(True)
    Y = gcn.vnm_spmm(adj, X)
    assert Y.shape == (n, 100) and Y.dtype == torch.float32
    assert oracle.rowwise_rel_err(Y.detach().cpu().numpy(), A @ _bf16(X)) <= TOL
    G = torch.randn((n, 100), generator=g).cuda()
    (Y * G).sum().backward()
    assert oracle.rowwise_rel_err(X.grad.cpu().numpy(), A.T @ _bf16(G)) <= TOL
    adj.close()


def test_gcn_layer(ctx):
    import torch
    from vnm_gb300 import gcn
    n, r, c, v = _graph(True)
    adj = gcn.VnmAdjacency(ctx, n, r, c, v)
    g = torch.Generator().manual_seed(4)
    H = torch.randn((n, 64), generator=g).cuda()
    W = (torch.randn((64, 128), generator=g) / 8).cuda().requires_grad_(True)
    b = torch.zeros(128, device="cuda", requires_grad=True)
    out = gcn.gcn_layer(adj, H, W, b)
    ref = np.maximum(_csr(n, r, c, v) @ _bf16(H @ W), 0.0)
    assert _rel(out.detach().cpu().numpy(), ref) <= TOL
    out.sum().backward()
    assert W.grad is not None and torch.isfinite(W.grad).all() and b.grad.shape == (128,)
    adj.close()


def test_aggregation_runs_on_a_caller_stream_without_waiting(ctx):
    """Forward and backward on a side stream: the op enqueues there and
    returns while the stream is still busy (a 0.5 s sleep kernel enqueued
    first), and the results match float64 once the stream is done."""
    import time
    import torch
    from vnm_gb300 import gcn
    n, r, c, v = _graph(False)
    adj = gcn.VnmAdjacency(ctx, n, r, c, v, M=8, V=128)
    A = _csr(n, r, c, v)
    g = torch.Generator().manual_seed(5)
    X0 = torch.randn((n, 128), generator=g).cuda()
    G = torch.randn((n, 128), generator=g).cuda()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):  # first calls: the widths are timed once
        X = X0.clone().requires_grad_(True)
        (gcn.vnm_spmm(adj, X) * G).sum().backward()
    s.synchronize()
    with torch.cuda.stream(s):
        torch.cuda._sleep(int(1e9))  # about half a second of device time
        X = X0.clone().requires_grad_(True)
        t0 = time.perf_counter()
        Y = gcn.vnm_spmm(adj, X)
        (Y * G).sum().backward()
        host_s = time.perf_counter() - t0
        busy = not s.query()
    assert busy and host_s < 0.2, (busy, host_s)
    s.synchronize()
    adj.fwd.check(s)
    assert oracle.rowwise_rel_err(Y.detach().cpu().numpy(), A @ _bf16(X0)) <= TOL
    assert oracle.rowwise_rel_err(X.grad.cpu().numpy(), A.T @ _bf16(G)) <= TOL
    adj.close()
