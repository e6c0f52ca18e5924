"""Build recipe for the reference's own NM reorder, used to pin the oracle.

TEST INFRASTRUCTURE ONLY.  Nothing in the product uses the result.

Step 1 (`flatten`, run where the reference checkout is present): for each
(N, M) pair, write one translation unit oracle/_ref/ref_nm_n<N>_m<M>.cu made of
the reference headers util/argparse.h, mtx/Mtx.h (+ util/utility.h, mtx/readMtx.hpp,
mtx/mmio.hpp) and reorder/reorder.h (+ reorder/swappair.h), with the quoted
#includes inlined in place and the two compile-time constants of
mtx/Mtx.h:15-16 set to N and M -- the configuration step the reference's
README prescribes -- followed by oracle/ref_harness.cu.  oracle/_ref/ is not
committed; it is a build directory.

The same step also writes oracle/_ref/ref_spmm_n<N>_m<M>.cu for the (N, M)
pairs of the command's golden cases: main.cu itself (the `spmm` command of
main.cu:339-352 with find_best_2toX and hybrid_reordering) with its quoted
#includes inlined the same way.

Step 2 (`compile`, run on a machine with nvcc; needs a GPU only to *run*):
nvcc each flattened unit for sm_103a against cuSPARSE/cuBLAS, as the
reference's Makefile does for sm_89, with -maxrregcount=64.  The register cap
is needed for M=8: there GetSegSwapScore (reorder/reorder.h:75-131) keeps
two 64-entry gain arrays and ptxas gives it 72 registers on sm_103a (40 on
the Makefile's sm_89).  Launched with 1024 threads (reorder/reorder.h:505-507)
it then exceeds the 65536 registers of an SM, the launch fails, nothing
checks it, and every gain stays at the cudaMemset zero.  With the cap the
kernel launches and computes what its source says, as on sm_89.

The reference checkout is read from --ref, else from $VNM_REF_DIR, else
from /root/reference.

usage: python oracle/ref_build.py flatten [--ref DIR]
       python oracle/ref_build.py compile [--only NAME]
"""
import argparse
import os
import re
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
CONFIGS = [(2, 8), (2, 4), (1, 4), (3, 8)]
SPMM_CONFIGS = [(2, 8), (2, 4)]
DEFAULT_REF = os.environ.get("VNM_REF_DIR", "/root/reference")
INC_RE = re.compile(r'^\s*#\s*include\s+"([^"]+)"')


def _inline(path, seen, out_lines, nm):
    path = os.path.normpath(path)
    if path in seen:
        return
    seen.add(path)
    base = os.path.dirname(path)
    with open(path) as f:
        for line in f:
            m = INC_RE.match(line)
            if m:
                _inline(os.path.join(base, m.group(1)), seen, out_lines, nm)
                continue
            if path.endswith(os.path.join("mtx", "Mtx.h")):
                if re.match(r"^\s*#define\s+N\s+\d+\s*$", line):
                    line = "#define N %d\n" % nm[0]
                elif re.match(r"^\s*#define\s+M\s+\d+\s*$", line):
                    line = "#define M %d\n" % nm[1]
            out_lines.append(line)
    out_lines.append("\n")


def flatten(ref):
    os.makedirs(OUT, exist_ok=True)
    paths = []
    for N, M in CONFIGS:
        lines = ["// generated by oracle/ref_build.py from the reference checkout; not committed\n"]
        seen = set()
        # main.cu includes util/argparse.h first; its `using namespace std;`
        # is what reorder/reorder.h relies on for unordered_map.
        _inline(os.path.join(ref, "util", "argparse.h"), seen, lines, (N, M))
        _inline(os.path.join(ref, "mtx", "Mtx.h"), seen, lines, (N, M))
        _inline(os.path.join(ref, "reorder", "reorder.h"), seen, lines, (N, M))
        with open(os.path.join(HERE, "ref_harness.cu")) as f:
            lines.append(f.read())
        p = os.path.join(OUT, "ref_nm_n%d_m%d.cu" % (N, M))
        with open(p, "w") as f:
            f.writelines(lines)
        paths.append(p)
    for N, M in SPMM_CONFIGS:
        lines = ["// generated by oracle/ref_build.py from the reference checkout; not committed\n"]
        _inline(os.path.join(ref, "main.cu"), set(), lines, (N, M))
        p = os.path.join(OUT, "ref_spmm_n%d_m%d.cu" % (N, M))
        with open(p, "w") as f:
            f.writelines(lines)
        paths.append(p)
    return paths


def _nvcc(src):
    exe = src[:-3]
    cmd = ["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-w", "-maxrregcount=64",
           "-o", exe, src, "-lcusparse", "-lcublas"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s" % (src, r.stderr[-4000:]))
    return exe


def ensure(name):
    """Path of the compiled unit oracle/_ref/<name>, compiling it first when
    its binary is missing or older than its flattened source."""
    exe = os.path.join(OUT, name)
    src = exe + ".cu"
    if not os.path.exists(src):
        raise FileNotFoundError("missing %s: run oracle/ref_build.py flatten where the reference checkout is" % src)
    if not os.path.exists(exe) or os.path.getmtime(exe) < os.path.getmtime(src):
        _nvcc(src)
    return exe


def compile_all(only=None):
    srcs = sorted(os.path.join(OUT, f) for f in os.listdir(OUT) if f.endswith(".cu")) if os.path.isdir(OUT) else []
    if only:
        srcs = [p for p in srcs if os.path.basename(p)[:-3] == only]
    if not srcs:
        return []
    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        return list(ex.map(_nvcc, srcs))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("step", choices=["flatten", "compile"])
    ap.add_argument("--ref", default=DEFAULT_REF)
    ap.add_argument("--only", default=None, help="compile one unit, e.g. ref_nm_n2_m4")
    a = ap.parse_args()
    if a.step == "flatten":
        if not os.path.isdir(a.ref):
            sys.exit("reference checkout not found at %s" % a.ref)
        for p in flatten(a.ref):
            print(p)
    else:
        for p in compile_all(a.only):
            print(p)


if __name__ == "__main__":
    main()
