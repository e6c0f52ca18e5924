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
