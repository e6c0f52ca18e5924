"""Accessors for the committed golden fixtures (tests/golden/*.npz)."""
import numpy as np


def nm_cases(g):
    """Yield (case, key, N, M, sched) for every NM golden case."""
    for case in g["cases"].tolist():
        key, s = case.rsplit("__s", 1)
        nm = key.split("__", 1)[1]
        N = int(nm.split("_")[0][1:])
        M = int(nm.split("_")[1][1:])
        yield case, key, N, M, int(s)


def nm_input(g, key):
    return (int(g["in__%s__nrows" % key]), g["in__%s__row" % key], g["in__%s__col" % key],
            g["in__%s__val" % key])


# The `spmm` command's cases: (case id, input name, N, M, V, maxiter).  The
# reference command itself is run on all but maxiter 0, where it indexes an
# empty result vector (main.cu:321, :331); that case is checked against the
# oracle only.
CLI_CASES = [("u256_n2m8_v32_i2", "u256", 2, 8, 32, 2), ("u256_n2m4_v64_i1", "u256", 2, 4, 64, 1),
             ("rmat1k_n2m8_v32_i3", "rmat1k", 2, 8, 32, 3), ("lund_n2m8_v32_i2", "fixture_lund", 2, 8, 32, 2),
             ("gd95_n2m8_v4_i2", "fixture_gd95", 2, 8, 4, 2), ("sym96_n2m8_v8_i2", "sym96", 2, 8, 8, 2),
             ("u256_n2m8_v32_i0", "u256", 2, 8, 32, 0)]


def cli_input(name, goldens):
    """The COO of a command case's input matrix (written out with
    vnm_gb300.synth.write_mtx before the command reads it)."""
    from vnm_gb300 import synth
    if name == "u256":
        return synth.uniform(256, 0.05, 3)
    if name == "rmat1k":
        return synth.rmat(10, 4096, 5, "uniform")
    if name == "sym96":
        n, r, c, v = synth.rmat(7, 300, 22, "uniform", R=96)
        lo, hi = np.minimum(r, c), np.maximum(r, c)
        v = np.round(np.sin(lo * 7.0 + hi * 3.0) * 0.9, 2).astype(np.float32)  # symmetric values
        return n, r, c, v
    key = {"fixture_lund": "lund_b__n2_m8", "fixture_gd95": "GD95_a__n2_m8"}[name]
    return nm_input(goldens, key)


def tied_schedules(mtxfile, N, M):
    """The schedules find_best_2toX can pick for this matrix: those of the
    largest improve rate (main.cu:72-114).  The reference breaks a tie by
    each schedule's measured wall time (main.cu:90-99), so a recorded run
    may hold any of them; the library and the oracle take the lowest."""
    import oracle
    nr, _, r, c, v = oracle.read_mtx(mtxfile, M)
    _, out = oracle.find_best(nr, r, c, v, N, M)
    rate = out[:, 7]
    return [s for s in range(4) if rate[s] == rate.max()]
