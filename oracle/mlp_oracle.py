"""CPU restatement of the learned-proposal pieces (numpy, float64).

TEST INFRASTRUCTURE ONLY: tests/ use this module as the checker of the
library's proposal network (tensor-core inference, training gradients) and
of the learned-mode bookkeeping.  The product never imports it.  The
reference has no learned mode; these functions restate this project's own
definitions:

  network   32 -> 128 -> 128 -> 1, ReLU; the forward pass rounds the inputs
            of the two hidden layers and their weights to BF16 (round to
            nearest even), accumulates in FP32 or better, and rounds the
            second hidden activation to BF16 before the FP32 output dot;
  loss      L = mean((y - t)^2) / 2 over a batch;
  gradient  straight through the BF16 roundings;
  objective retained nonzeros of an N:M pruning = sum over (row, M-column
            segment) groups of min(popcount, N); invalid groups = groups
            with popcount > N.
"""
import numpy as np

F, H = 32, 128
OFF_W1 = 0
OFF_B1 = OFF_W1 + H * F
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H
NPARAM = OFF_B3 + 1


def bf16(x):
    """Round float32 values to the nearest BF16 (ties to even), as float64."""
    x = np.asarray(x, np.float32)
    b = x.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) >> 16 << 16
    return (b.astype(np.uint32)).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, np.float64)
    return (p[OFF_W1:OFF_B1].reshape(H, F), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(H, H), p[OFF_B2:OFF_W3],
            p[OFF_W3:OFF_B3], p[OFF_B3])


def forward(p, X, rounding=True):
    """Returns y and the activations (H1, H2) after ReLU."""
    r = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    W1, b1, W2, b2, w3, b3 = unpack(p)
    X = np.asarray(X, np.float64)
    H1 = np.maximum(r(X) @ r(W1).T + b1, 0.0)
    H2 = np.maximum(r(H1) @ r(W2).T + b2, 0.0)
    y = r(H2) @ w3 + b3
    return y, H1, H2


def loss_grad(p, X, t, rounding=True):
    """(loss, gradient) of L = mean((y - t)^2) / 2, flat like p."""
    r = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    W1, b1, W2, b2, w3, b3 = unpack(p)
    X = np.asarray(X, np.float64)
    t = np.asarray(t, np.float64)
    B = len(X)
    y, H1, H2 = forward(p, X, rounding)
    d = y - t
    loss = 0.5 * np.mean(d * d)
    dy = d / B
    g = np.zeros(NPARAM)
    g[OFF_W3:OFF_B3] = r(H2).T @ dy
    g[OFF_B3] = dy.sum()
    dH2 = dy[:, None] * w3[None, :] * (H2 > 0)
    g[OFF_W2:OFF_B2] = (dH2.T @ r(H1)).ravel()
    g[OFF_B2:OFF_W3] = dH2.sum(0)
    dH1 = (dH2 @ r(W2)) * (H1 > 0)
    g[OFF_W1:OFF_B1] = (dH1.T @ r(X)).ravel()
    g[OFF_B1:OFF_W2] = dH1.sum(0)
    return loss, g


def groups(nrows, row, col, val, M):
    """popcount of every nonempty (row, segment) group of the nonzero-valued
    pattern, as a dict-free array (one entry per group)."""
    row = np.asarray(row, np.int64)
    col = np.asarray(col, np.int64)
    keep = np.asarray(val) != 0
    key = row[keep] * (nrows // M + 1) + col[keep] // M
    _, counts = np.unique(key, return_counts=True)
    return counts


def nm_totals(nrows, row, col, val, N, M):
    """(invalid groups, retained nonzeros) of the matrix."""
    c = groups(nrows, row, col, val, M)
    return int((c > N).sum()), int(np.minimum(c, N).sum())
