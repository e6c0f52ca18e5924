"""ctypes front-end of the CPU oracle (oracle/vnm_oracle.cpp).

TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg use this module as the checker.  The product never imports it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
SRC = os.path.join(HERE, "vnm_oracle.cpp")

_i32p = ctypes.POINTER(ctypes.c_int)
_f32p = ctypes.POINTER(ctypes.c_float)
_f64p = ctypes.POINTER(ctypes.c_double)


def build(force=False):
    """Compile liboracle.so with g++ (OpenMP on)."""
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= max(
            os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "vnm_oracle.h"))):
        return LIB_PATH
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared",
                           "-o", tmp, SRC])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_mtx_read.argtypes = [ctypes.c_char_p, ctypes.c_int, _i32p, _i32p, _i32p,
                                   ctypes.POINTER(_i32p), ctypes.POINTER(_i32p), ctypes.POINTER(_f32p)]
        L.orc_mtx_write.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _i32p, _i32p, _f32p]
        L.orc_nm_run.argtypes = [ctypes.c_int, ctypes.c_int, _i32p, _i32p, _f32p, ctypes.c_int, ctypes.c_int,
                                 ctypes.c_int, ctypes.c_int, _i32p, _i32p]
        L.orc_nm_run_trace.argtypes = [ctypes.c_int, ctypes.c_int, _i32p, _i32p, _f32p, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_int, ctypes.c_int, _i32p,
                                       ctypes.POINTER(_i32p), ctypes.POINTER(_i32p), _i32p]
        L.orc_nm_segment_counts.argtypes = [ctypes.c_int, ctypes.c_int, _i32p, _i32p, _f32p, ctypes.c_int,
                                            ctypes.c_int, _i32p, _i32p]
        L.orc_nm_pair_score.argtypes = [ctypes.c_int, ctypes.c_int, _i32p, _i32p, _f32p, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_int, ctypes.c_int, _i32p]
        L.orc_swap_heap_order.argtypes = [ctypes.c_int, _i32p, _i32p, _i32p]
        L.orc_swap_heap_order.restype = None
        L.orc_vnm_eval.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _i32p, _i32p, ctypes.c_int,
                                   ctypes.c_int, _i32p]
        L.orc_vnm_run.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _i32p, _i32p, ctypes.c_int,
                                  ctypes.c_int, ctypes.c_int, _i32p, _i32p]
        L.orc_roundtrip_nm.argtypes = [ctypes.c_float]
        L.orc_roundtrip_nm.restype = ctypes.c_float
        L.orc_roundtrip_vnm.argtypes = [ctypes.c_float]
        L.orc_roundtrip_vnm.restype = ctypes.c_float
        L.orc_find_best.argtypes = [ctypes.c_int, ctypes.c_int, _i32p, _i32p, _f32p, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_int, _i32p, _f32p]
        L.orc_spmm_cli.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_int, _f64p, _i32p, _i32p, _i32p, ctypes.POINTER(_i32p),
                                   ctypes.POINTER(_i32p), ctypes.POINTER(_f32p)]
        L.orc_spmm_cli_sched.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_int, ctypes.c_int, _f64p, _i32p, _i32p, _i32p,
                                         ctypes.POINTER(_i32p), ctypes.POINTER(_i32p), ctypes.POINTER(_f32p)]
        L.orc_retained_nm.argtypes = [ctypes.c_int, ctypes.c_int, _i32p, _i32p, _f32p, ctypes.c_int, ctypes.c_int]
        L.orc_retained_nm.restype = ctypes.c_int64
        L.orc_retained_vnm.argtypes = [ctypes.c_int, ctypes.c_int, _i32p, _i32p, _f32p, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_int]
        L.orc_retained_vnm.restype = ctypes.c_int64
        L.orc_spmm_f64.argtypes = [ctypes.c_int, ctypes.c_int, _i32p, _i32p, _f64p, _f64p, ctypes.c_int, _f64p]
        L.orc_spmm_f64.restype = None
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_set_threads.restype = None
        L.orc_get_max_threads.restype = ctypes.c_int
        L.orc_free.argtypes = [ctypes.c_void_p]
        L.orc_free.restype = None
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t)


def _check(st, what):
    if st != 0:
        raise RuntimeError("oracle %s failed with status %d" % (what, st))


def _take(ptr, n, dtype):
    if n == 0:
        out = np.zeros(0, dtype=dtype)
    else:
        out = np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)
    lib().orc_free(ctypes.cast(ptr, ctypes.c_void_p))
    return out


def set_threads(n):
    lib().orc_set_threads(int(n))


def max_threads():
    return lib().orc_get_max_threads()


def read_mtx(path, aligned):
    """readMtx + Mtx padding: returns (nrows, ncols, row, col, val)."""
    nr, nc, nz = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    r, c, v = _i32p(), _i32p(), _f32p()
    _check(lib().orc_mtx_read(os.fsencode(path), aligned, nr, nc, nz, r, c, v), "read_mtx")
    n = nz.value
    return nr.value, nc.value, _take(r, n, np.int32), _take(c, n, np.int32), _take(v, n, np.float32)


def write_mtx(path, nrows, ncols, row, col, val):
    row = np.ascontiguousarray(row, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    val = np.ascontiguousarray(val, np.float32)
    _check(lib().orc_mtx_write(os.fsencode(path), nrows, ncols, len(row), _p(row, _i32p), _p(col, _i32p),
                               _p(val, _f32p)), "write_mtx")


def nm_run(nrows, row, col, val, N, M, sched, nm_maxiter=10):
    """One NM job: returns (res5, row', col', newpos)."""
    row = np.array(row, np.int32)
    col = np.array(col, np.int32)
    val = np.ascontiguousarray(val, np.float32)
    res = np.zeros(5, np.int32)
    newpos = np.zeros(nrows, np.int32)
    _check(lib().orc_nm_run(nrows, len(row), _p(row, _i32p), _p(col, _i32p), _p(val, _f32p), N, M, sched,
                            nm_maxiter, _p(res, _i32p), _p(newpos, _i32p)), "nm_run")
    return res, row, col, newpos


def nm_run_trace(nrows, row, col, val, N, M, sched, nm_maxiter=10):
    """Returns (res5, list of per-round swap arrays of shape (k, 2))."""
    row = np.array(row, np.int32)
    col = np.array(col, np.int32)
    val = np.ascontiguousarray(val, np.float32)
    res = np.zeros(5, np.int32)
    pp, rp, nr = _i32p(), _i32p(), ctypes.c_int()
    _check(lib().orc_nm_run_trace(nrows, len(row), _p(row, _i32p), _p(col, _i32p), _p(val, _f32p), N, M, sched,
                                  nm_maxiter, _p(res, _i32p), pp, rp, nr), "nm_run_trace")
    ptr = _take(rp, nr.value + 1, np.int64)
    pairs = _take(pp, int(ptr[-1]) * 2, np.int32).reshape(-1, 2)
    return res, [pairs[ptr[i]:ptr[i + 1]] for i in range(nr.value)]


def nm_segment_counts(nrows, row, col, val, N, M):
    row = np.ascontiguousarray(row, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    val = np.ascontiguousarray(val, np.float32)
    nseg = nrows // M
    inv = np.zeros(nseg, np.int32)
    az = np.zeros(nseg, np.int32)
    _check(lib().orc_nm_segment_counts(nrows, len(row), _p(row, _i32p), _p(col, _i32p), _p(val, _f32p), N, M,
                                       _p(inv, _i32p), _p(az, _i32p)), "segment_counts")
    return inv, az


def nm_pair_score(nrows, row, col, val, N, M, s1, s2):
    row = np.ascontiguousarray(row, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    val = np.ascontiguousarray(val, np.float32)
    sc = np.zeros(2 * M * M, np.int32)
    _check(lib().orc_nm_pair_score(nrows, len(row), _p(row, _i32p), _p(col, _i32p), _p(val, _f32p), N, M, s1, s2,
                                   _p(sc, _i32p)), "pair_score")
    return sc


def swap_heap_order(lg, rg):
    lg = np.ascontiguousarray(lg, np.int32)
    rg = np.ascontiguousarray(rg, np.int32)
    order = np.zeros(len(lg), np.int32)
    lib().orc_swap_heap_order(len(lg), _p(lg, _i32p), _p(rg, _i32p), _p(order, _i32p))
    return order


def vnm_eval(m, n, row, col, M, V):
    row = np.ascontiguousarray(row, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    out = np.zeros(2, np.int32)
    _check(lib().orc_vnm_eval(m, n, len(row), _p(row, _i32p), _p(col, _i32p), M, V, _p(out, _i32p)), "vnm_eval")
    return out


def vnm_run(m, n, row, col, M, V, maxiter=10):
    """reordering.py loop: returns (out5, row', col', newpos)."""
    row = np.array(row, np.int32)
    col = np.array(col, np.int32)
    out = np.zeros(5, np.int32)
    mp = (m + M - 1) // M * M
    newpos = np.zeros(mp, np.int32)
    _check(lib().orc_vnm_run(m, n, len(row), _p(row, _i32p), _p(col, _i32p), M, V, maxiter, _p(out, _i32p),
                             _p(newpos, _i32p)), "vnm_run")
    return out, row, col, newpos


def roundtrip_nm(v):
    return lib().orc_roundtrip_nm(float(v))


def roundtrip_vnm(v):
    return lib().orc_roundtrip_vnm(float(v))


def find_best(nrows, row, col, val, N, M, nscheds=4):
    row = np.ascontiguousarray(row, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    val = np.ascontiguousarray(val, np.float32)
    best = ctypes.c_int()
    out = np.zeros(48, np.float32)
    _check(lib().orc_find_best(nrows, len(row), _p(row, _i32p), _p(col, _i32p), _p(val, _f32p), N, M, nscheds,
                               best, _p(out, _f32p)), "find_best")
    return best.value, out.reshape(4, 12)


def spmm_cli(mtxfile, N, M, V, maxiter, init_mb_path=None, sched=None):
    """Whole `spmm` command; returns (csv16, best, nrows, row, col, val).
    `sched` fixes the schedule instead of find_best_2toX's choice (the
    reference breaks its ties by wall time, main.cu:90-99)."""
    csv = np.zeros(16, np.float64)
    best, onr, onz = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    r, c, v = _i32p(), _i32p(), _f32p()
    _check(lib().orc_spmm_cli_sched(os.fsencode(mtxfile), os.fsencode(init_mb_path) if init_mb_path else None, N, M,
                                    V, maxiter, -1 if sched is None else int(sched), _p(csv, _f64p), best, onr, onz,
                                    r, c, v), "spmm_cli")
    n = onz.value
    return csv, best.value, onr.value, _take(r, n, np.int32), _take(c, n, np.int32), _take(v, n, np.float32)


def retained_nm(nrows, row, col, val, N, M):
    row = np.ascontiguousarray(row, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    val = np.ascontiguousarray(val, np.float32)
    return lib().orc_retained_nm(nrows, len(row), _p(row, _i32p), _p(col, _i32p), _p(val, _f32p), N, M)


def retained_vnm(nrows, row, col, val, N, M, V):
    row = np.ascontiguousarray(row, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    val = np.ascontiguousarray(val, np.float32)
    return lib().orc_retained_vnm(nrows, len(row), _p(row, _i32p), _p(col, _i32p), _p(val, _f32p), N, M, V)


def spmm_f64(nrows, row, col, val, B):
    row = np.ascontiguousarray(row, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    val = np.ascontiguousarray(val, np.float64)
    B = np.ascontiguousarray(B, np.float64)
    n = B.shape[1]
    C = np.zeros((nrows, n), np.float64)
    lib().orc_spmm_f64(nrows, len(row), _p(row, _i32p), _p(col, _i32p), _p(val, _f64p), _p(B, _f64p), n,
                       _p(C, _f64p))
    return C


def rowwise_rel_err(C, ref):
    """Largest per-row relative error max_i ||C_i - ref_i||_inf / ||ref_i||_inf.

    Rows whose reference is exactly zero (no nonzero in the row) count with
    a denominator of 1e-30, so any nonzero output there fails the bound.
    Unlike max |C - ref| / max |ref| over the whole matrix, a low-degree row
    cannot hide behind the hub rows that set the global maximum."""
    C = np.asarray(C, np.float64)
    ref = np.asarray(ref, np.float64)
    num = np.abs(C - ref).max(axis=1) if C.size else np.zeros(len(C))
    den = np.maximum(np.abs(ref).max(axis=1) if ref.size else np.zeros(len(ref)), 1e-30)
    return float((num / den).max()) if len(num) else 0.0
