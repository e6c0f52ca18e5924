"""Build libvnm_gb300.so (CUDA, sm_103a) and the `spmm` drop-in command.

Every .cu/.cpp file under csrc/ is compiled in parallel with nvcc for
sm_103a only, then linked into libvnm_gb300.so next to this file; cli/spmm.cpp
is linked against it into ./spmm (rpath $ORIGIN).  Incremental: a unit is
rebuilt when it or any header under csrc/ or include/ changed.
"""
import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libvnm_gb300.so")
CLI_SRC = os.path.join(HERE, "cli", "spmm.cpp")
CLI = os.path.join(HERE, "spmm")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
                     "-diag-suppress", "177", "-I", os.path.join(REPO, "include")]


def _nvcc():
    for c in ("nvcc", "/usr/local/cuda/bin/nvcc"):
        try:
            subprocess.run([c, "--version"], capture_output=True, check=True)
            return c
        except (OSError, subprocess.CalledProcessError):
            pass
    raise RuntimeError("nvcc not found")


def _headers():
    hs = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh"))
    hs += glob.glob(os.path.join(REPO, "include", "*.h"))
    return max((os.path.getmtime(h) for h in hs), default=0.0)


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, jobs=None):
    nvcc = _nvcc()
    os.makedirs(OBJ, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    hdr_time = _headers()
    todo = []
    objs = []
    for s in srcs:
        o = os.path.join(OBJ, os.path.basename(s) + ".o")
        objs.append(o)
        if not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), hdr_time):
            todo.append((s, o))

    def cc(so):
        s, o = so
        cmd = [nvcc] + NVCC_FLAGS + ["-c", s, "-o", o + ".tmp"]
        if s.endswith(".cpp"):
            cmd = [nvcc] + NVCC_FLAGS + ["-x", "cu", "-c", s, "-o", o + ".tmp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed on %s:\n%s" % (s, r.stderr[-6000:]))
        os.replace(o + ".tmp", o)
        if verbose and r.stderr.strip():
            print(r.stderr)
        return s

    if todo:
        with ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            for s in ex.map(cc, todo):
                if verbose:
                    print("compiled", os.path.relpath(s, REPO))
    if todo or _stale(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s" % r.stderr[-4000:])
        os.replace(tmp, LIB)
    if os.path.exists(CLI_SRC) and _stale(CLI, [CLI_SRC, LIB, os.path.join(REPO, "include", "vnm_gb300.h")]):
        tmp = CLI + ".tmp%d" % os.getpid()
        cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(REPO, "include"), "-o", tmp, CLI_SRC,
               "-L", HERE, "-lvnm_gb300", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("cli build failed:\n%s" % r.stderr[-4000:])
        os.replace(tmp, CLI)
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(LIB)
