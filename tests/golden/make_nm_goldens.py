"""Golden vectors for the NM reorder, produced by the reference's own code.

The reference's NM path is CUDA, so its goldens are made on a GPU machine
with the binaries that oracle/ref_build.py builds from the reference sources.

  prepare  (where the reference checkout is): write the synthetic inputs to
           tests/golden/nm_inputs/ and copy the reference's shipped matrices
           (mtxfile/*.mtx) to oracle/_ref/fixtures/.  Neither folder is
           committed: the npz below holds every input's COO as the
           reference's reader returned it, which is what the tests use.
  run      (GPU machine, after `ref_build.py compile`): run every input x
           (N, M) x schedule through oracle/_ref/ref_nm_n<N>_m<M>; raw text
           results go to --out (default oracle/_ref/nm_raw; on a machine
           whose files do not come back, a folder that is copied back).
  collect  (anywhere): read the raw results and the inputs, write
           tests/golden/nm_ref_goldens.npz.

The npz holds, per input, the COO exactly as the reference's reader returns
it, and per case (input, N, M, sched) the five result integers of
run_onepair* and the final position of every node that carries an entry
(-1 for nodes without entries, whose position the output cannot show).
"""
import argparse
import glob
import hashlib
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "vnm-graph-reordering_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

from vnm_gb300 import synth  # noqa: E402

IN_DIR = os.path.join(HERE, "nm_inputs")
FIX_DIR = os.path.join(REPO, "oracle", "_ref", "fixtures")
REF_BIN = os.path.join(REPO, "oracle", "_ref")
OUT_NPZ = os.path.join(HERE, "nm_ref_goldens.npz")
CONFIGS = [(2, 8), (2, 4), (1, 4), (3, 8)]
FIXTURES = ["small", "GD95_a", "GD01_c", "bcsstm02", "lund_b"]


def _write_int(path, n, row, col, rng):
    vals = rng.integers(-3, 4, len(row))
    with open(path, "w") as f:
        f.write("%%%%MatrixMarket matrix coordinate integer general\n%d %d %d\n" % (n, n, len(row)))
        for r, c, v in zip(row.tolist(), col.tolist(), vals.tolist()):
            f.write("%d %d %d\n" % (r + 1, c + 1, v))


def _write_sym(path, n, row, col, val):
    keep = row >= col
    with open(path, "w") as f:
        f.write("%%%%MatrixMarket matrix coordinate real symmetric\n%d %d %d\n" % (n, n, int(keep.sum())))
        for r, c, v in zip(row[keep].tolist(), col[keep].tolist(), val[keep].tolist()):
            f.write("%d %d %.6g\n" % (r + 1, c + 1, v))


def prepare(ref):
    os.makedirs(IN_DIR, exist_ok=True)
    w = synth.write_mtx
    w(os.path.join(IN_DIR, "c1_512.mtx"), *synth.uniform_c1(0))
    w(os.path.join(IN_DIR, "u64_d10.mtx"), *synth.uniform(64, 0.10, 1))
    w(os.path.join(IN_DIR, "u100_d08.mtx"), *synth.uniform(100, 0.08, 2))
    w(os.path.join(IN_DIR, "u256_d05.mtx"), *synth.uniform(256, 0.05, 3))
    w(os.path.join(IN_DIR, "u1000_d01.mtx"), *synth.uniform(1000, 0.01, 4))
    w(os.path.join(IN_DIR, "rmat_1024.mtx"), *synth.rmat(10, 4096, 5, "uniform"))
    w(os.path.join(IN_DIR, "rmat_2048.mtx"), *synth.rmat(11, 16384, 6, "uniform"))
    n, r, c, v = synth.uniform(256, 0.06, 7)
    v = v.copy()
    v[np.random.default_rng(7).random(len(v)) < 0.1] = 0.0  # explicit zeros: not in the N:M bitmap
    w(os.path.join(IN_DIR, "zeros_256.mtx"), n, r, c, v)
    n, r, c, v = synth.uniform(200, 0.05, 8)
    _write_int(os.path.join(IN_DIR, "int_200.mtx"), n, r, c, np.random.default_rng(8))
    n, r, c, v = synth.uniform(300, 0.04, 9)
    w(os.path.join(IN_DIR, "pattern_300.mtx"), n, r, c, v, field="pattern")
    n, r, c, v = synth.rmat(9, 1200, 10, "uniform")
    _write_sym(os.path.join(IN_DIR, "sym_512.mtx"), n, r, c, v)
    w(os.path.join(IN_DIR, "rmat_4096.mtx"), *synth.rmat(12, 32768, 11, "uniform"))
    os.makedirs(FIX_DIR, exist_ok=True)
    for name in FIXTURES:
        shutil.copy(os.path.join(ref, "mtxfile", name + ".mtx"), os.path.join(FIX_DIR, name + ".mtx"))


def inputs():
    files = sorted(glob.glob(os.path.join(IN_DIR, "*.mtx")))
    files += [os.path.join(FIX_DIR, n + ".mtx") for n in FIXTURES]
    return files


def run(out):
    os.makedirs(out, exist_ok=True)
    jobs = []
    for f in inputs():
        if not os.path.exists(f):
            continue
        name = os.path.splitext(os.path.basename(f))[0]
        for N, M in CONFIGS:
            exe = os.path.join(REF_BIN, "ref_nm_n%d_m%d" % (N, M))
            for s in range(4):
                jobs.append((exe, f, s, os.path.join(out, "%s__n%d_m%d__s%d.txt" % (name, N, M, s))))

    def one(j):
        exe, f, s, o = j
        r = subprocess.run([exe, f, str(s), o], capture_output=True, text=True, timeout=900)
        return j, r.returncode, r.stderr[-500:]

    bad = 0
    with ThreadPoolExecutor(max_workers=8) as ex:
        for j, rc, err in ex.map(one, jobs):
            if rc != 0:
                bad += 1
                print("FAILED", j, rc, err)
    print("ran %d jobs, %d failed" % (len(jobs), bad))
    return bad


def collect(src):
    import oracle  # the reader only; every number below comes from the reference run

    data = {}
    names = []
    for f in inputs():
        name = os.path.splitext(os.path.basename(f))[0]
        for N, M in CONFIGS:
            key = "%s__n%d_m%d" % (name, N, M)
            if not os.path.exists(os.path.join(src, key + "__s0.txt")):
                continue
            nr, nc, row, col, val = oracle.read_mtx(f, M)
            data["in__%s__row" % key] = row
            data["in__%s__col" % key] = col
            data["in__%s__val" % key] = val
            data["in__%s__nrows" % key] = np.int32(nr)
            for s in range(4):
                p = os.path.join(src, "%s__s%d.txt" % (key, s))
                with open(p) as fh:
                    head = fh.readline().split()
                    body = np.loadtxt(fh, dtype=np.int64, ndmin=2).reshape(-1, 2)
                nrows, nnz = int(head[0]), int(head[1])
                res = np.array([int(x) for x in head[2:7]], np.int32)
                assert nrows == nr and nnz == len(row), (p, nrows, nr, nnz, len(row))
                newpos = np.full(nrows, -1, np.int64)
                newpos[row] = body[:, 0]
                newpos[col] = body[:, 1]
                ok = np.array_equal(newpos[row], body[:, 0]) and np.array_equal(newpos[col], body[:, 1])
                assert ok, "final COO is not a relabelling of the input: %s" % p
                case = "%s__s%d" % (key, s)
                data["res__" + case] = res
                data["pos__" + case] = newpos.astype(np.int32)
                data["sha__" + case] = np.frombuffer(
                    hashlib.sha256(body.astype(np.int32).tobytes()).digest(), np.uint8)
                names.append(case)
    data["cases"] = np.array(names)
    np.savez_compressed(OUT_NPZ, **data)
    print("wrote %s with %d cases" % (OUT_NPZ, len(names)))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("step", choices=["prepare", "run", "collect"])
    ap.add_argument("--ref", default=os.environ.get("VNM_REF_DIR", "/root/reference"))
    ap.add_argument("--out", default=os.path.join(REPO, "oracle", "_ref", "nm_raw"))
    a = ap.parse_args()
    if a.step == "prepare":
        prepare(a.ref)
    elif a.step == "run":
        sys.exit(1 if run(a.out) else 0)
    else:
        collect(a.out)


if __name__ == "__main__":
    main()
