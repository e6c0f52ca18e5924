"""Golden outputs of the reference's own `spmm` command (main.cu:339-352).

The command is built from main.cu itself (oracle/ref_build.py flattens it
with N and M set, oracle/_ref/ref_spmm_n<N>_m<M>) and run on a GPU machine on
the cases of tests/golden_cases.py CLI_CASES: find_best_2toX, the stale
temp.mtx evaluation, the NM / VNM loop, the output .mtx and the 16-field CSV
line, all by the reference's code.  Its VNM stage is `python3
reordering.py`, which needs the reference checkout; that script runs only
where the checkout is.  oracle/vnm_replay.py, placed in the command's working
directory as reordering.py, replays the recorded runs of the real script
(keyed by flags and input bytes) and records what it has not seen yet.  The
steps alternate until a run has no miss; that run is the golden.

  prepare  (where the checkout is) write the inputs, answer the first
           evaluation (the stale temp.mtx, here a copy of the input)
  run      (GPU machine) run the command per case; raw output to --out
  serve    (where the checkout is) run the real reordering.py on the
           requests the last run recorded (--src = that run's --out)
  collect  (anywhere) write tests/golden/cli_ref_goldens.npz from a run
           whose cases all completed without a miss

The working directory of every case starts with temp.mtx = a copy of the
input, so the command's first evaluation (main.cu:207, which reads whatever
temp.mtx is lying around) sees the input matrix.  Run state lives in
oracle/_ref/cli/ (not committed).  The checkout is read from --ref, else
$VNM_REF_DIR, else /root/reference.
"""
import argparse
import glob
import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TESTS = os.path.dirname(HERE)
REPO = os.path.dirname(TESTS)
for p in (os.path.join(REPO, "vnm-graph-reordering_gb300"), os.path.join(REPO, "oracle"), TESTS):
    if p not in sys.path:
        sys.path.insert(0, p)

from golden_cases import CLI_CASES, cli_input  # noqa: E402

STATE = os.path.join(REPO, "oracle", "_ref", "cli")
INPUTS = os.path.join(STATE, "inputs")
CACHE = os.path.join(STATE, "cache")
OUT_NPZ = os.path.join(HERE, "cli_ref_goldens.npz")
DEFAULT_REF = os.environ.get("VNM_REF_DIR", "/root/reference")


def ref_cases():
    return [c for c in CLI_CASES if c[5] > 0]  # maxiter 0: main.cu:331 reads an empty vector


def _goldens():
    return np.load(os.path.join(HERE, "nm_ref_goldens.npz"))


def input_path(name):
    return os.path.join(INPUTS, name + ".mtx")


def serve_one(ref, req_json, req_mtx):
    """Run the real reordering.py on one recorded request; store its outputs
    in the cache under the request's key."""
    import vnm_replay
    with open(req_json) as f:
        q = json.load(f)
    with open(req_mtx, "rb") as f:
        data = f.read()
    key = vnm_replay.request_key(q["evalonly"], q["m"], q["v"], q["maxiter"], data)
    if os.path.exists(os.path.join(CACHE, key + ".out")):
        return key, False
    with tempfile.TemporaryDirectory() as td:
        with open(os.path.join(td, "temp.mtx"), "wb") as f:
            f.write(data)
        cmd = [sys.executable, os.path.join(ref, "reordering.py"), "--m", str(q["m"]), "--v", str(q["v"]),
               "--maxiter", str(q["maxiter"])] + (["--evalonly"] if q["evalonly"] else [])
        r = subprocess.run(cmd, cwd=td, capture_output=True, text=True, timeout=3600)
        if r.returncode != 0:
            raise RuntimeError("reordering.py failed: %s" % r.stderr[-2000:])
        os.makedirs(CACHE, exist_ok=True)
        if not q["evalonly"]:
            shutil.copyfile(os.path.join(td, "temp.mtx"), os.path.join(CACHE, key + ".mtx"))
        shutil.copyfile(os.path.join(td, "output.txt"), os.path.join(CACHE, key + ".out"))
    return key, True


def prepare(ref):
    from vnm_gb300 import synth
    os.makedirs(INPUTS, exist_ok=True)
    g = _goldens()
    for name in sorted({c[1] for c in CLI_CASES}):
        synth.write_mtx(input_path(name), *cli_input(name, g))
    # the first evaluation reads the stale temp.mtx, a copy of the input
    n = 0
    with tempfile.TemporaryDirectory() as td:
        for case, name, N, M, V, it in ref_cases():
            jq, jm = os.path.join(td, case + ".json"), os.path.join(td, case + ".mtx")
            with open(jq, "w") as f:
                json.dump({"evalonly": True, "m": M, "v": V, "maxiter": 10}, f)
            shutil.copyfile(input_path(name), jm)
            n += serve_one(ref, jq, jm)[1]
    print("inputs in %s; %d first evaluations answered" % (INPUTS, n))


def run(out):
    import ref_build
    exes = {}
    for N, M in sorted({(c[2], c[3]) for c in ref_cases()}):
        exes[(N, M)] = ref_build.ensure("ref_spmm_n%d_m%d" % (N, M))
    replay = os.path.join(REPO, "oracle", "vnm_replay.py")

    def one(c):
        case, name, N, M, V, it = c
        wd = os.path.join(out, case)
        if os.path.isdir(wd):
            shutil.rmtree(wd)
        os.makedirs(wd)
        shutil.copyfile(input_path(name), os.path.join(wd, "input.mtx"))
        shutil.copyfile(input_path(name), os.path.join(wd, "temp.mtx"))
        shutil.copyfile(replay, os.path.join(wd, "reordering.py"))
        env = dict(os.environ, VNM_REPLAY_CACHE=CACHE, VNM_REPLAY_PENDING=os.path.join(wd, "pending"),
                   VNM_REPLAY_LOG=os.path.join(wd, "replay.log"))
        cmd = [exes[(N, M)], "--mtxfile", "input.mtx", "--outmtxfile", "out.mtx", "--maxiter", str(it), "--n", "64",
               "--sched", "0", "--v", str(V)]
        r = subprocess.run(cmd, cwd=wd, env=env, capture_output=True, text=True, timeout=900)
        with open(os.path.join(wd, "stdout.txt"), "w") as f:
            f.write(r.stdout)
        with open(os.path.join(wd, "stderr.txt"), "w") as f:
            f.write(r.stderr)
        misses = len(glob.glob(os.path.join(wd, "pending", "*.json")))
        st = {"rc": r.returncode, "misses": misses, "case": case}
        with open(os.path.join(wd, "status.json"), "w") as f:
            json.dump(st, f)
        return st

    with ThreadPoolExecutor(max_workers=4) as ex:
        sts = list(ex.map(one, ref_cases()))
    for st in sts:
        print(json.dumps(st))
    bad = [s for s in sts if s["rc"] != 0]
    return 1 if bad else 0


def serve(src, ref):
    reqs = sorted(glob.glob(os.path.join(src, "*", "pending", "*.json")))
    done = 0
    for q in reqs:
        done += serve_one(ref, q, q[:-5] + ".mtx")[1]
    print("%d requests, %d new answers in %s" % (len(reqs), done, CACHE))


def collect(src):
    data, names = {}, []
    for case, name, N, M, V, it in ref_cases():
        wd = os.path.join(src, case)
        with open(os.path.join(wd, "status.json")) as f:
            st = json.load(f)
        if st["rc"] != 0 or st["misses"] != 0:
            raise SystemExit("case %s is not complete (%s): serve and run again" % (case, st))
        with open(os.path.join(wd, "stdout.txt")) as f:
            line = f.read().strip()
        with open(os.path.join(wd, "out.mtx"), "rb") as f:
            text = f.read()
        with open(input_path(name), "rb") as f:
            data["in_sha__" + case] = np.array(hashlib.sha256(f.read()).hexdigest())
        data["csv__" + case] = np.array(line)
        data["out__" + case] = np.frombuffer(text, np.uint8)
        data["cfg__" + case] = np.array([N, M, V, it], np.int32)
        names.append(case)
    data["cases"] = np.array(names)
    np.savez_compressed(OUT_NPZ, **data)
    print("wrote %s with %d cases" % (OUT_NPZ, len(names)))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("step", choices=["prepare", "run", "serve", "collect"])
    ap.add_argument("--ref", default=DEFAULT_REF)
    ap.add_argument("--out", help="run: the folder the raw outputs go to (one that comes back from the GPU machine)")
    ap.add_argument("--src", help="serve / collect: that folder, back where the checkout is")
    a = ap.parse_args()
    if a.step == "prepare":
        prepare(a.ref)
    elif a.step == "run":
        if not a.out:
            ap.error("run needs --out")
        sys.exit(run(a.out))
    elif a.step == "serve":
        if not a.src:
            ap.error("serve needs --src")
        serve(a.src, a.ref)
    else:
        if not a.src:
            ap.error("collect needs --src")
        collect(a.src)


if __name__ == "__main__":
    main()
