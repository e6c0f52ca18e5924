"""Golden vectors for the VNM stage, made by running the reference's own
reordering.py (Python, runs anywhere with numpy/scipy).

For each input, the script is run the way main.cu runs it -- on a temp.mtx
written by the NM stage ("%d %d %.2f", general), in a scratch directory:
  python3 reordering.py --evalonly --m M --v V   -> output.txt (2 ints)
  python3 reordering.py --m M --v V              -> output.txt (5 ints) and
                                                    the rewritten temp.mtx
The npz stores the input COO, both outputs and the rewritten matrix as
scipy reads it back.  A second table pins scipy's mmwrite(precision=1)
number format: value -> text it writes.

usage: python tests/golden/make_vnm_goldens.py [--ref DIR]
"""
import argparse
import io
import os
import shutil
import subprocess
import sys
import tempfile
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "vnm-graph-reordering_gb300"))
from vnm_gb300 import synth  # noqa: E402

OUT = os.path.join(HERE, "vnm_ref_goldens.npz")


def nm_text(path, n, row, col, val):
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix coordinate real general\n%d %d %d\n" % (n, n, len(row)))
        for r, c, v in zip(row.tolist(), col.tolist(), val.tolist()):
            f.write("%d %d %.2f\n" % (r + 1, c + 1, v))


def inputs(ref):
    out = []
    out.append(("u64", *synth.uniform(64, 0.10, 1)))
    out.append(("u256", *synth.uniform(256, 0.05, 3)))
    out.append(("c1_512", *synth.uniform_c1(0)))
    out.append(("rmat_512", *synth.rmat(9, 2048, 21, "uniform")))
    out.append(("rmat_1024", *synth.rmat(10, 4096, 5, "uniform")))
    n, r, c, v = synth.rmat(7, 300, 22, "uniform", R=96)
    lo, hi = np.minimum(r, c), np.maximum(r, c)
    v = np.round(np.sin(lo * 7.0 + hi * 3.0) * 0.9, 2).astype(np.float32)  # symmetric values
    out.append(("u96_sym", n, r, c, v))
    from scipy.io import mmread
    for name in ("GD95_a", "lund_b", "GD01_c"):
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            m = mmread(os.path.join(ref, "mtxfile", name + ".mtx"))
        out.append((name, m.shape[0], m.row.astype(np.int32), m.col.astype(np.int32),
                    np.asarray(m.data, np.float32)))
    return out


def run_script(ref, tmp, args):
    r = subprocess.run([sys.executable, os.path.join(ref, "reordering.py")] + args, cwd=tmp,
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stderr[-2000:])
    with open(os.path.join(tmp, "output.txt")) as f:
        return np.array([int(x) for x in f.read().strip().split(",")], np.int32)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("VNM_REF_DIR", "/root/reference"))
    a = ap.parse_args()
    from scipy.io import mmread, mmwrite
    from scipy.sparse import coo_matrix
    data = {}
    cases = []
    for name, n, row, col, val in inputs(a.ref):
        data["in__%s__n" % name] = np.int32(n)
        data["in__%s__row" % name] = row
        data["in__%s__col" % name] = col
        data["in__%s__val" % name] = val
        for M, V in ((8, 32), (4, 64), (8, 4), (4, 8)):
            tmp = tempfile.mkdtemp()
            try:
                nm_text(os.path.join(tmp, "temp.mtx"), n, row, col, val)
                ev = run_script(a.ref, tmp, ["--evalonly", "--m", str(M), "--v", str(V)])
                out = run_script(a.ref, tmp, ["--m", str(M), "--v", str(V)])
                with warnings.catch_warnings():
                    warnings.simplefilter("ignore")
                    mm = mmread(os.path.join(tmp, "temp.mtx"))
                with open(os.path.join(tmp, "temp.mtx")) as f:
                    banner = f.readline().strip()
            finally:
                shutil.rmtree(tmp, ignore_errors=True)
            case = "%s__m%d_v%d" % (name, M, V)
            data["eval__" + case] = ev
            data["out__" + case] = out
            data["wrow__" + case] = mm.row.astype(np.int32)
            data["wcol__" + case] = mm.col.astype(np.int32)
            data["wval__" + case] = np.asarray(mm.data, np.float64)
            data["wsym__" + case] = np.int32(1 if "symmetric" in banner else 0)
            cases.append(case)
            print(case, ev.tolist(), out.tolist(), banner)
    data["cases"] = np.array(cases)
    # scipy mmwrite(precision=1): the text each value turns into
    rng = np.random.default_rng(0)
    vals = np.concatenate([rng.standard_normal(2000), rng.uniform(-1, 1, 2000) * 10.0 ** rng.integers(-4, 4, 2000),
                           np.array([0.0, -0.0, 0.05, 0.15, 0.25, 0.35, 0.45, 0.95, 1.5, 2.5, 9.5, 12.5, 99.5,
                                     0.005, 0.0049, 1e-5, 123456.0])])
    vals = np.round(vals, 2)  # what the NM writer's "%.2f" leaves
    buf = io.BytesIO()
    mmwrite(buf, coo_matrix((vals, (np.arange(len(vals)), np.zeros(len(vals), int))), shape=(len(vals), 200)),
            precision=1)
    lines = buf.getvalue().decode().splitlines()
    body = [ln for ln in lines if ln and not ln.startswith("%")][1:]
    data["fmt__in"] = vals
    data["fmt__text"] = np.array([ln.split()[2] for ln in body])
    np.savez_compressed(OUT, **data)
    print("wrote", OUT, len(cases), "cases")


if __name__ == "__main__":
    main()
