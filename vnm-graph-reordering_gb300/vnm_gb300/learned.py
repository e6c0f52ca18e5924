"""Training pipeline of the swap-proposal network.

Training pairs come from the exact scorer itself: an exhaustive-mode run of
vnm_nm_learned scores every candidate swap exactly and keeps a sample of
(features, exact gain) pairs.  The network is then fitted on the GPU with
the library's own forward/backward/Adam kernels (vnm_mlp_train).
"""
import numpy as np

from . import LEARNED_EXHAUSTIVE, OBJ_RETAINED, Mlp, nm_learned


def training_pairs(ctx, mats, N, M, objective=OBJ_RETAINED, targets=16, rounds=8, dump_every=16,
                   cap_per_matrix=32768, seed=0):
    """(X [n][32], gains [n]) from exhaustive runs over `mats`, a list of
    (nrows, row, col, val) with nrows a multiple of M."""
    xs, ys = [], []
    for i, (n, r, c, v) in enumerate(mats):
        _, _, (dx, dy) = nm_learned(ctx, n, r, c, v, N, M, mode=LEARNED_EXHAUSTIVE, objective=objective,
                                    targets=targets, max_rounds=rounds, patience=rounds, seed=seed + i,
                                    dump_every=dump_every, dump_cap=cap_per_matrix, want_newpos=False)
        xs.append(dx)
        ys.append(dy)
    return np.concatenate(xs), np.concatenate(ys)


def train_proposal_net(ctx, X, y, epochs=4, batch=1024, lr=1e-3, seed=0):
    """A new network fitted to (X, y); returns (net, mean loss of the last epoch)."""
    net = Mlp(ctx, seed)
    perm = np.random.default_rng(seed).permutation(len(X))
    n = (len(X) // batch) * batch
    loss = net.train(X[perm][:n], y[perm][:n], batch=batch, epochs=epochs, lr=lr)
    return net, loss


WEIGHTS_DIR = __import__("os").path.dirname(__import__("os").path.abspath(__file__))


def weights_path(N, M):
    """Where the trained network of an N:M pattern is kept in the package."""
    import os
    return os.path.join(WEIGHTS_DIR, "proposal_net_n%d_m%d.npy" % (N, M))


def training_matrices(count=64, lo=8192, hi=32768, degree=32, seed=5000):
    """The training graphs: R-MAT with row counts log-uniform in [lo, hi]
    (rounded to multiples of 8) and the given average degree."""
    from . import synth
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        R = int(round(np.exp(rng.uniform(np.log(lo), np.log(hi))) / 8)) * 8
        scale = int(np.ceil(np.log2(R)))
        out.append(synth.rmat(scale, R * degree // 2, seed + 1 + i, "normal", R=R))
    return out


def train_recipe(ctx, N=2, M=8, count=64, degree=32, dump_every=256, cap_per_matrix=20000, epochs=4, seed=0,
                 log=print):
    """Train the proposal network the way the shipped weights were trained:
    exhaustive-mode pairs from `count` R-MAT graphs of 8192-32768 rows
    (~1M pairs), then Adam on the GPU.  Returns (net, info dict)."""
    import time
    t0 = time.time()
    mats = training_matrices(count, degree=degree)
    t1 = time.time()
    X, y = training_pairs(ctx, mats, N, M, targets=16, rounds=8, dump_every=dump_every,
                          cap_per_matrix=cap_per_matrix, seed=seed)
    t2 = time.time()
    net, loss = train_proposal_net(ctx, X, y, epochs=epochs, batch=1024, lr=1e-3, seed=seed)
    t3 = time.time()
    info = {"pairs": int(len(X)), "matrices": count, "gain_mean": float(y.mean()), "gain_var": float(y.var()),
            "positive_frac": float((y > 0).mean()), "final_loss": float(loss), "epochs": epochs,
            "synth_s": round(t1 - t0, 2), "pairs_s": round(t2 - t1, 2), "train_s": round(t3 - t2, 2)}
    log("trained proposal net: %s" % info)
    return net, info


def load(ctx, N, M, path=None):
    """A network with the shipped weights of N:M (raises if there are none)."""
    from . import Mlp
    net = Mlp(ctx, 0)
    net.set(np.load(path or weights_path(N, M)))
    return net


if __name__ == "__main__":
    import argparse
    import json

    from . import Context
    ap = argparse.ArgumentParser(description="train the swap-proposal network and save its weights")
    ap.add_argument("--N", type=int, default=2)
    ap.add_argument("--M", type=int, default=8)
    ap.add_argument("--out", default=None)
    ap.add_argument("--count", type=int, default=64)
    a = ap.parse_args()
    with Context(0) as ctx:
        net, info = train_recipe(ctx, a.N, a.M, count=a.count)
        out = a.out or weights_path(a.N, a.M)
        np.save(out, net.get())
        with open(out[:-4] + ".json", "w") as f:
            json.dump(info, f, indent=1)
