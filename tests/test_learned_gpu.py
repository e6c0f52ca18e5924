"""Learned-proposal reorder on the GPU, checked against the CPU oracle
(oracle/mlp_oracle.py, oracle/vnm_oracle.cpp):

  - the tensor-core inference of the proposal network against the numpy
    forward with the same BF16 roundings;
  - the training gradient against the numpy gradient, and Adam reducing the
    loss;
  - every mode (network / exhaustive / random proposals, both objectives):
    the permutation is a permutation, the invalid-group and retained counts
    the library reports equal the oracle's counts of the permuted matrix,
    the accepted exact gains add up to the change of the objective, and the
    objective never gets worse;
  - a trained network (the shipped weights, and one trained here by the
    library's own kernels) proposes better swaps than random proposals at
    the same exact-scoring budget, and comes close to exhaustive scoring
    with a fraction of its exact scores.
"""
import numpy as np
import pytest

import mlp_oracle as mo

pytestmark = pytest.mark.gpu


def _net(ctx, seed, scale=1.0):
    import vnm_gb300
    net = vnm_gb300.Mlp(ctx, seed)
    p = net.get()
    p[mo.OFF_B1:mo.OFF_W2] = np.random.default_rng(seed).normal(0, 0.1, mo.H)
    p *= scale
    net.set(p)
    return net


@pytest.mark.parametrize("n", [1, 127, 128, 1000, 4096])
def test_mlp_forward_matches_oracle(ctx, n):
    net = _net(ctx, 3)
    X = np.random.default_rng(n).normal(0, 1, (n, mo.F)).astype(np.float32)
    y = net.forward(X)
    want, _, _ = mo.forward(net.get(), X)
    # fp32 accumulation in a different order can flip a BF16 rounding of a
    # hidden activation; each flip moves y by at most 2^-8 |h w3|
    tol = 2e-3 * (np.abs(want) + 1.0)
    assert np.all(np.abs(y - want) <= tol), float(np.max(np.abs(y - want) / (np.abs(want) + 1)))


def test_mlp_grad_matches_oracle(ctx):
    net = _net(ctx, 5)
    rng = np.random.default_rng(7)
    X = rng.normal(0, 1, (256, mo.F)).astype(np.float32)
    t = rng.normal(0, 2, 256).astype(np.float32)
    g, loss = net.grad(X, t)
    wl, wg = mo.loss_grad(net.get(), X, t)
    assert abs(loss - wl) <= 1e-4 * (abs(wl) + 1e-3)
    scale = np.abs(wg).max()
    np.testing.assert_allclose(g, wg, rtol=2e-3, atol=2e-5 * scale)


def test_mlp_train_reduces_loss(ctx):
    import vnm_gb300
    net = vnm_gb300.Mlp(ctx, 11)
    rng = np.random.default_rng(8)
    X = rng.normal(0, 1, (8192, mo.F)).astype(np.float32)
    t = (np.maximum(X[:, 0], 0) * 2 - X[:, 1] + 0.5 * X[:, 2] * X[:, 3]).astype(np.float32)
    l0, _, _ = mo.forward(net.get(), X[:1024])
    loss0 = 0.5 * np.mean((l0 - t[:1024]) ** 2)
    loss = net.train(X, t, batch=256, epochs=8, lr=2e-3)
    y = net.forward(X[:1024])
    loss1 = 0.5 * np.mean((y - t[:1024]) ** 2)
    assert loss < 0.2 * loss0 and loss1 < 0.2 * loss0, (loss0, loss, loss1)


def _mat(seed, scale=11, deg=12, M=8):
    from vnm_gb300 import synth
    n, r, c, v = synth.rmat(scale, (1 << scale) * deg // 2, seed, "normal")
    assert n % M == 0
    return n, r, c, v


def _check_result(res, n, r, c, v, N, M, newpos, objective):
    assert np.array_equal(np.sort(newpos), np.arange(n))
    rr, cc = newpos[r], newpos[c]
    assert mo.nm_totals(n, r, c, v, N, M) == (res["init_invalid"], res["init_retained"])
    assert mo.nm_totals(n, rr, cc, v, N, M) == (res["final_invalid"], res["final_retained"])
    if objective == 1:
        assert res["final_retained"] - res["init_retained"] == res["gain"]
        assert res["final_retained"] >= res["init_retained"]
    else:
        assert res["init_invalid"] - res["final_invalid"] == res["gain"]
        assert res["final_invalid"] <= res["init_invalid"]


@pytest.mark.parametrize("N,M", [(2, 8), (2, 4), (1, 4)])
@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("objective", [0, 1])
def test_learned_modes_are_consistent(ctx, N, M, mode, objective):
    import vnm_gb300
    n, r, c, v = _mat(21 + M, M=M)
    net = _net(ctx, 1) if mode == 0 else None
    res, newpos, _ = vnm_gb300.nm_learned(ctx, n, r, c, v, N, M, mode=mode, net=net, objective=objective,
                                          targets=8, max_rounds=12, patience=3, seed=4)
    _check_result(res, n, r, c, v, N, M, newpos, objective)
    assert res["rounds"] >= 1 and res["swaps"] >= 1
    if mode == 1:
        assert res["exact_scored"] > 0


def test_learned_is_deterministic(ctx):
    import vnm_gb300
    n, r, c, v = _mat(31)
    net = _net(ctx, 2)
    a = vnm_gb300.nm_learned(ctx, n, r, c, v, 2, 8, mode=0, net=net, targets=8, max_rounds=6, seed=9)
    b = vnm_gb300.nm_learned(ctx, n, r, c, v, 2, 8, mode=0, net=net, targets=8, max_rounds=6, seed=9)
    assert a[0] == b[0] and np.array_equal(a[1], b[1])


def test_empty_and_tiny_inputs(ctx):
    import vnm_gb300
    e = np.zeros(0, np.int32)
    res, newpos, _ = vnm_gb300.nm_learned(ctx, 16, e, e, np.zeros(0, np.float32), 2, 8, mode=1)
    assert res["rounds"] == 0 and np.array_equal(newpos, np.arange(16))
    r = np.array([0, 0, 0], np.int32)
    c = np.array([0, 1, 2], np.int32)
    v = np.ones(3, np.float32)
    res, newpos, _ = vnm_gb300.nm_learned(ctx, 8, r, c, v, 2, 8, mode=1)  # one segment: nothing to swap with
    assert res["final_invalid"] == 1 and np.array_equal(newpos, np.arange(8))


def test_stop_gain_stops_at_the_target(ctx):
    import vnm_gb300
    n, r, c, v = _mat(41, scale=12, deg=32)
    full, _, _ = vnm_gb300.nm_learned(ctx, n, r, c, v, 2, 8, mode=2, max_rounds=40, patience=3, seed=2)
    target = full["gain"] // 2
    res, pos, _ = vnm_gb300.nm_learned(ctx, n, r, c, v, 2, 8, mode=2, max_rounds=40, patience=3, seed=2,
                                       stop_gain=target)
    _check_result(res, n, r, c, v, 2, 8, pos, 1)
    assert target <= res["gain"] < full["gain"] and res["rounds"] < full["rounds"]


def _net_vs_random(ctx, net, n, r, c, v, N, M, rounds):
    import vnm_gb300
    kw = dict(targets=16, topk=1, max_rounds=rounds, patience=100, seed=3)
    res_n, pos_n, _ = vnm_gb300.nm_learned(ctx, n, r, c, v, N, M, mode=0, net=net, **kw)
    res_r, pos_r, _ = vnm_gb300.nm_learned(ctx, n, r, c, v, N, M, mode=2, **kw)
    _check_result(res_n, n, r, c, v, N, M, pos_n, 1)
    _check_result(res_r, n, r, c, v, N, M, pos_r, 1)
    return res_n, res_r


def test_shipped_network_beats_random_proposals(ctx):
    """The network's ranking against random ranking at the same exact-scoring
    budget (one exactly scored proposal per segment and round) on a graph
    outside its training set."""
    from vnm_gb300 import learned
    net = learned.load(ctx, 2, 8)
    n, r, c, v = _mat(777, scale=13, deg=32)
    for rounds in (1, 2):
        res_n, res_r = _net_vs_random(ctx, net, n, r, c, v, 2, 8, rounds)
        print("rounds %d: network %d random %d" % (rounds, res_n["gain"], res_r["gain"]))
        assert res_n["gain"] > 1.2 * res_r["gain"], rounds


def test_training_pipeline_learns_a_useful_ranking(ctx):
    """Pairs from the exact scorer -> GPU training -> a network that ranks
    better than random; and the network needs far fewer exact scores than
    exhaustive scoring for the same number of rounds."""
    import vnm_gb300
    from vnm_gb300 import learned
    N, M = 2, 8
    train = [_mat(100 + i, scale=13, deg=32) for i in range(4)]
    X, y = learned.training_pairs(ctx, train, N, M, targets=16, rounds=8, dump_every=128, cap_per_matrix=60000)
    assert len(X) > 100000 and np.all(np.isfinite(X))
    net, loss = learned.train_proposal_net(ctx, X, y, epochs=4, batch=1024, lr=1e-3)
    assert np.isfinite(loss) and loss < 0.5 * y.var()
    n, r, c, v = _mat(200, scale=13, deg=32)
    res_n, res_r = _net_vs_random(ctx, net, n, r, c, v, N, M, 1)
    print("network %d random %d" % (res_n["gain"], res_r["gain"]))
    assert res_n["gain"] > 1.15 * res_r["gain"]
    kw = dict(targets=16, max_rounds=4, patience=100, seed=3)
    res_8, _, _ = vnm_gb300.nm_learned(ctx, n, r, c, v, N, M, mode=0, net=net, topk=8, **kw)
    res_e, _, _ = vnm_gb300.nm_learned(ctx, n, r, c, v, N, M, mode=1, **kw)
    assert res_8["exact_scored"] * 50 < res_e["exact_scored"]
    assert res_8["gain"] > 0.95 * res_e["gain"]
