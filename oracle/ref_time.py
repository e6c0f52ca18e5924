"""Wall time of the reference's own GPU NM reorder on the R-MAT 16384 (2:4)
workload, schedule by schedule, as find_best_2toX runs them (main.cu:72-114:
four full runs in a row, each reading the matrix from its file).

TEST INFRASTRUCTURE ONLY: runs the flattened reference unit that
oracle/ref_build.py makes (oracle/_ref/ref_nm_n2_m4.cu, the reference's
mtx/Mtx.h + reorder/reorder.h with N=2, M=4, around oracle/ref_harness.cu),
compiling it first when its binary is missing.  Needs a GPU.

usage: python oracle/ref_time.py [--scheds 0,1,2,3] [--timeout S] [--out F]
Prints one JSON object: per schedule the wall seconds, the result vector
and whether it finished within the time limit.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(REPO, "vnm-graph-reordering_gb300"))
sys.path.insert(0, HERE)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--scheds", default="0,1,2,3")
    ap.add_argument("--timeout", type=float, default=600.0)
    ap.add_argument("--out", default=None)
    a = ap.parse_args()
    import ref_build
    from vnm_gb300 import synth
    src = os.path.join(HERE, "_ref", "ref_nm_n2_m4.cu")
    exe = src[:-3]
    if not os.path.exists(exe):
        if not os.path.exists(src):
            sys.exit("missing %s: run oracle/ref_build.py flatten where the reference checkout is" % src)
        t0 = time.time()
        ref_build._nvcc(src)
        print("compiled %s in %.1f s" % (exe, time.time() - t0), file=sys.stderr)
    nr, r, c, v = synth.rmat_c2(0)
    out = {"workload": "R-MAT 16384x16384, 131072 edges symmetrised (%d entries), N(0,1), 2:4" % len(r),
           "binary": "reference mtx/Mtx.h + reorder/reorder.h (N=2, M=4) built for sm_103a, -maxrregcount=64",
           "schedules": {}}
    with tempfile.TemporaryDirectory() as td:
        mtx = os.path.join(td, "c2.mtx")
        synth.write_mtx(mtx, nr, r, c, v)
        total = 0.0
        for s in (int(x) for x in a.scheds.split(",")):
            res_path = os.path.join(td, "res%d.txt" % s)
            t0 = time.perf_counter()
            try:
                p = subprocess.run([exe, mtx, str(s), res_path], capture_output=True, text=True, timeout=a.timeout)
                dt = time.perf_counter() - t0
                ok = p.returncode == 0
                res = open(res_path).readline().split()[2:7] if ok else None
                out["schedules"][s] = {"seconds": dt, "finished": ok, "res5": res}
            except subprocess.TimeoutExpired:
                dt = time.perf_counter() - t0
                out["schedules"][s] = {"seconds": dt, "finished": False, "timeout": a.timeout}
            total += dt
        out["total_seconds"] = total
    js = json.dumps(out)
    print(js)
    if a.out:
        with open(a.out, "w") as f:
            f.write(js + "\n")


if __name__ == "__main__":
    main()
