"""CPU checks of the learned-mode oracle (oracle/mlp_oracle.py): the BF16
rounding against torch's, and the restated gradient against central finite
differences (rounding off, float64)."""
import numpy as np
import torch

import mlp_oracle as mo


def test_bf16_rounding_matches_torch():
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.normal(0, 1, 4096), rng.normal(0, 1e4, 1024), rng.normal(0, 1e-4, 1024),
                        [0.0, -0.0, 1.0, 1.00390625, 1.01171875, 65504.0]]).astype(np.float32)
    want = torch.from_numpy(x).to(torch.bfloat16).to(torch.float64).numpy()
    np.testing.assert_array_equal(mo.bf16(x), want)


def test_param_layout():
    assert mo.NPARAM == 32 * 128 + 128 + 128 * 128 + 128 + 128 + 1


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    p = rng.normal(0, 0.2, mo.NPARAM)
    X = rng.normal(0, 1, (16, mo.F))
    t = rng.normal(0, 1, 16)
    _, g = mo.loss_grad(p, X, t, rounding=False)
    idx = np.concatenate([rng.choice(np.arange(mo.OFF_W1, mo.OFF_B1), 8), rng.choice(np.arange(mo.OFF_B1, mo.OFF_W2), 4),
                          rng.choice(np.arange(mo.OFF_W2, mo.OFF_B2), 8), rng.choice(np.arange(mo.OFF_B2, mo.OFF_W3), 4),
                          rng.choice(np.arange(mo.OFF_W3, mo.OFF_B3), 4), [mo.OFF_B3]])
    h = 1e-6
    for i in idx:
        q = p.copy()
        q[i] += h
        lp, _ = mo.loss_grad(q, X, t, rounding=False)
        q[i] -= 2 * h
        lm, _ = mo.loss_grad(q, X, t, rounding=False)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, g[i])


def test_nm_totals_small_case():
    # 2 rows, M=4: row 0 holds cols 0,1,2 (one group of 3), row 1 holds 4, 7
    row = np.array([0, 0, 0, 1, 1])
    col = np.array([0, 1, 2, 4, 7])
    val = np.ones(5, np.float32)
    assert mo.nm_totals(8, row, col, val, 2, 4) == (1, 4)
    val[1] = 0.0  # zero values are not in the pattern
    assert mo.nm_totals(8, row, col, val, 2, 4) == (0, 4)
