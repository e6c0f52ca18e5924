"""Golden vectors for the NM reorder at the benchmarked sizes, from the oracle.

The oracle (oracle/vnm_oracle.cpp, a CPU restatement of reorder/reorder.h
and main.cu:72-114, pinned against the reference's own GPU code on the 272
cases of nm_ref_goldens.npz) needs minutes per schedule at these sizes, too
long for a test run, so its results are computed once here and committed:

  c2   R-MAT 16384 (131072 edges drawn, symmetrised, N(0,1) values), 2:4 --
       the matrix of the headline benchmark step
  c4   R-MAT 65536 (1048576 edges drawn, symmetrised, N(0,1) values), 2:8 --
       the plain reorder of the learned-proposal comparison

Per workload the npz holds, for schedules 0..3, the five result integers of
run_onepair* and the final position of every node, the schedule that
find_best_2toX picks (largest improve rate, ties to the lower id), and a
SHA-256 of the input COO, so that a test on another machine can check that
the seeded generator gave it the same matrix.  The inputs themselves are
not stored: vnm_gb300.synth regenerates them from their seeds.

The reference's own GPU code is also run on the c2 matrix (all four
schedules, the flattened unit oracle/_ref/ref_nm_n2_m4 that
oracle/ref_build.py makes): `ref-run` on a GPU machine writes its raw output,
`ref-collect` turns it into scale_ref_c2.npz (result integers, final
position of every node that carries an entry, seconds per schedule).

The reference's VNM stage, `python3 reordering.py --m 8 --v 64`, is run on
the c2 matrix as well (`vnm-ref`, where the reference checkout is, about 5
minutes on one core): scale_vnm_c2.npz holds the five integers it writes to
output.txt, the (row, col) of the matrix it writes back in entry order,
and its wall seconds (this machine's, for the record).

usage: python tests/golden/make_scale_goldens.py oracle [--only c2|c4] [--threads T]
       python tests/golden/make_scale_goldens.py ref-run --out DIR
       python tests/golden/make_scale_goldens.py ref-collect --src DIR
       python tests/golden/make_scale_goldens.py vnm-ref [--ref DIR]
"""
import argparse
import hashlib
import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "vnm-graph-reordering_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

OUT_NPZ = os.path.join(HERE, "scale_oracle_goldens.npz")
REF_NPZ = os.path.join(HERE, "scale_ref_c2.npz")
VNM_NPZ = os.path.join(HERE, "scale_vnm_c2.npz")
DEFAULT_REF = os.environ.get("VNM_REF_DIR", "/root/reference")
WORKLOADS = {"c2": ("rmat_c2", 2, 4), "c4": ("rmat_c4", 2, 8)}


def coo_digest(nrows, row, col, val):
    h = hashlib.sha256()
    h.update(np.int64(nrows).tobytes())
    for a, t in ((row, np.int32), (col, np.int32), (val, np.float32)):
        h.update(np.ascontiguousarray(a, t).tobytes())
    return h.hexdigest()


def load(name):
    from vnm_gb300 import synth
    gen, N, M = WORKLOADS[name]
    nr, r, c, v = getattr(synth, gen)(0)
    return nr, r, c, v, N, M


def improve_rate(res):
    """main.cu:57 in float32: (init_cnt - final_cnt) / init_cnt."""
    if res[2] == 0:
        return np.float32(0)
    return np.float32(np.float32(res[2] - res[3]) / np.float32(res[2]))


def pick_best(res4):
    """find_best_2toX (main.cu:72-114) with ties to the lower schedule id."""
    best, best_rate = 0, np.float32(0)
    for s in range(4):
        if res4[s][1] == 0 or res4[s][0] == 0:  # main.cu:85 (nnz == 0 or init_size == 0)
            return 0
        rate = improve_rate(res4[s])
        if rate > best_rate:
            best, best_rate = s, rate
    return best


def _one(job):
    name, sched, threads = job
    import oracle
    oracle.set_threads(threads)
    nr, r, c, v, N, M = load(name)
    t0 = time.time()
    res, _, _, newpos = oracle.nm_run(nr, r, c, v, N, M, sched)
    return name, sched, res, newpos, time.time() - t0


def ref_run(out, timeout=900.0):
    """The reference's own GPU reorder on the c2 matrix, schedule by
    schedule, as find_best_2toX runs them (main.cu:72-114)."""
    import subprocess
    import ref_build
    from vnm_gb300 import synth
    exe = ref_build.ensure("ref_nm_n2_m4")
    os.makedirs(out, exist_ok=True)
    nr, r, c, v, N, M = load("c2")
    mtx = os.path.join(out, "c2.mtx")
    synth.write_mtx(mtx, nr, r, c, v)
    times = {}
    for s in range(4):
        t0 = time.perf_counter()
        p = subprocess.run([exe, mtx, str(s), os.path.join(out, "c2__s%d.txt" % s)], capture_output=True, text=True,
                           timeout=timeout)
        times[s] = time.perf_counter() - t0
        if p.returncode != 0:
            raise SystemExit("reference run failed (schedule %d): %s" % (s, p.stderr[-2000:]))
        print("schedule %d: %.2f s" % (s, times[s]), flush=True)
    with open(os.path.join(out, "seconds.json"), "w") as f:
        import json
        json.dump(times, f)
    os.remove(mtx)


def ref_collect(src):
    import json
    nr, r, c, v, N, M = load("c2")
    res4, pos4 = [], []
    for s in range(4):
        with open(os.path.join(src, "c2__s%d.txt" % s)) as fh:
            head = fh.readline().split()
            body = np.loadtxt(fh, dtype=np.int64, ndmin=2).reshape(-1, 2)
        assert int(head[0]) == nr and int(head[1]) == len(r), head
        newpos = np.full(nr, -1, np.int64)
        newpos[r] = body[:, 0]
        newpos[c] = body[:, 1]
        assert np.array_equal(newpos[r], body[:, 0]) and np.array_equal(newpos[c], body[:, 1])
        res4.append([int(x) for x in head[2:7]])
        pos4.append(newpos)
    with open(os.path.join(src, "seconds.json")) as f:
        sec = json.load(f)
    np.savez_compressed(REF_NPZ, res5x4=np.array(res4, np.int32), newpos4=np.stack(pos4).astype(np.int32),
                        seconds=np.array([sec[str(s)] for s in range(4)]), sha256=np.array(coo_digest(nr, r, c, v)),
                        best=np.int32(pick_best(np.array(res4))))
    print("wrote", REF_NPZ, res4)


def vnm_ref(ref):
    """reordering.py (M=8, V=64, maxiter 10) on the c2 matrix, in a scratch
    working directory as main.cu runs it (temp.mtx in, temp.mtx and
    output.txt out)."""
    import subprocess
    import tempfile
    from scipy.io import mmread
    from vnm_gb300 import synth
    nr, r, c, v, N, M = load("c2")
    with tempfile.TemporaryDirectory() as td:
        synth.write_mtx(os.path.join(td, "temp.mtx"), nr, r, c, v)
        t0 = time.perf_counter()
        p = subprocess.run([sys.executable, os.path.join(ref, "reordering.py"), "--m", "8", "--v", "64", "--maxiter",
                            "10"], cwd=td, capture_output=True, text=True)
        dt = time.perf_counter() - t0
        if p.returncode != 0:
            raise SystemExit(p.stderr[-2000:])
        with open(os.path.join(td, "output.txt")) as f:
            out5 = [int(x) for x in f.read().strip().split(",")]
        mm = mmread(os.path.join(td, "temp.mtx"))
    np.savez_compressed(VNM_NPZ, out5=np.array(out5, np.int32), row=np.asarray(mm.row, np.int32),
                        col=np.asarray(mm.col, np.int32), seconds=np.float64(dt),
                        sha256=np.array(coo_digest(nr, r, c, v)))
    print("wrote", VNM_NPZ, out5, "%.1f s" % dt)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("step", choices=["oracle", "ref-run", "ref-collect", "vnm-ref"])
    ap.add_argument("--ref", default=DEFAULT_REF)
    ap.add_argument("--only", choices=sorted(WORKLOADS), default=None)
    ap.add_argument("--threads", type=int, default=max(1, (os.cpu_count() or 4) // 4))
    ap.add_argument("--out", help="ref-run: the folder the raw outputs go to (one that comes back from the GPU machine)")
    ap.add_argument("--src", help="ref-collect: that folder")
    a = ap.parse_args()
    if a.step == "ref-run":
        if not a.out:
            ap.error("ref-run needs --out")
        return ref_run(a.out)
    if a.step == "ref-collect":
        if not a.src:
            ap.error("ref-collect needs --src")
        return ref_collect(a.src)
    if a.step == "vnm-ref":
        return vnm_ref(a.ref)
    names = [a.only] if a.only else sorted(WORKLOADS)
    old = dict(np.load(OUT_NPZ)) if os.path.exists(OUT_NPZ) else {}
    out = {k: v for k, v in old.items() if k.split("__")[0] not in names}
    jobs = [(n, s, a.threads) for n in names for s in range(4)]
    with mp.get_context("spawn").Pool(min(4, len(jobs))) as pool:
        results = pool.map(_one, jobs)
    for name in names:
        nr, r, c, v, N, M = load(name)
        rows = sorted((x for x in results if x[0] == name), key=lambda x: x[1])
        res4 = np.stack([x[2] for x in rows]).astype(np.int32)
        pos4 = np.stack([x[3] for x in rows]).astype(np.int32)
        out[name + "__res5x4"] = res4
        out[name + "__newpos4"] = pos4
        out[name + "__best"] = np.int32(pick_best(res4))
        out[name + "__nm"] = np.array([N, M], np.int32)
        out[name + "__nrows_nnz"] = np.array([nr, len(r)], np.int64)
        out[name + "__sha256"] = np.array(coo_digest(nr, r, c, v))
        for x in rows:
            print("%s sched %d: res %s in %.0f s" % (name, x[1], x[2].tolist(), x[4]), flush=True)
    np.savez_compressed(OUT_NPZ, **out)
    print("wrote", OUT_NPZ)


if __name__ == "__main__":
    main()
