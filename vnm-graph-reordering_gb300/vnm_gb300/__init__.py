"""Python binding of libvnm_gb300 (ctypes over the C ABI in include/vnm_gb300.h).

This module is a thin host-side mirror of the library's C entry points; all
work happens in the CUDA library.  It refuses to run without the library:
there is no CPU fallback.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
LIB_PATH = os.path.join(PKG, "libvnm_gb300.so")

MEM_HOST = 0
MEM_DEVICE = 1

_i32p = ctypes.POINTER(ctypes.c_int)
_i64p = ctypes.POINTER(ctypes.c_int64)
_f32p = ctypes.POINTER(ctypes.c_float)
_vp = ctypes.c_void_p


class VnmError(RuntimeError):
    def __init__(self, status, what):
        self.status = status
        super().__init__("%s failed: %s (status %d)" % (what, status_string(status), status))


_lib = None


def build():
    import importlib.util
    spec = importlib.util.spec_from_file_location("vnm_gb300_build", os.path.join(PKG, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build()


def lib():
    """Load libvnm_gb300.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libvnm_gb300.so is missing at %s: build it first (python __graft_entry__.py build "
                           "or vnm-graph-reordering_gb300/build.py)" % LIB_PATH)
    L = ctypes.CDLL(LIB_PATH)
    L.vnm_status_string.restype = ctypes.c_char_p
    L.vnm_status_string.argtypes = [ctypes.c_int]
    L.vnm_version.restype = ctypes.c_char_p
    L.vnm_create.argtypes = [ctypes.POINTER(_vp), ctypes.c_int]
    L.vnm_destroy.argtypes = [_vp]
    L.vnm_last_kernel_ms.argtypes = [_vp]
    L.vnm_last_kernel_ms.restype = ctypes.c_float
    L.vnm_last_launch_count.argtypes = [_vp]
    L.vnm_last_main_kernel_ms.argtypes = [_vp]
    L.vnm_last_main_kernel_ms.restype = ctypes.c_float
    L.vnm_last_stats.argtypes = [_vp, ctypes.POINTER(ctypes.c_longlong), ctypes.c_int]
    L.vnm_nm_reorder.argtypes = [_vp, ctypes.c_int, ctypes.c_int, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int,
                                 ctypes.c_int, ctypes.c_int, ctypes.c_int, _i32p, _i32p]
    L.vnm_nm_search.argtypes = [_vp, ctypes.c_int, ctypes.c_int, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int,
                                ctypes.c_int, ctypes.c_int, _i32p, _i32p, _i32p]
    L.vnm_nm_reorder_batch.argtypes = [_vp, ctypes.c_int, _i32p, _i64p, _i32p, _i32p, _f32p, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_int, ctypes.c_int, _i32p, _i32p]
    L.vnm_nm_set_trace.argtypes = [_vp, ctypes.c_int]
    L.vnm_nm_set_phase_timing.argtypes = [_vp, ctypes.c_int]
    L.vnm_nm_get_trace.argtypes = [_vp, _i32p, ctypes.c_int, _i32p, _i32p, ctypes.c_int, _i32p]
    L.vnm_permute_coo.argtypes = [_vp, ctypes.c_int, ctypes.c_int, _vp, _vp, ctypes.c_int, _vp]
    L.vnm_nm_segment_counts.argtypes = [_vp, ctypes.c_int, ctypes.c_int, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int, _i32p, _i32p]
    L.vnm_nm_pair_score.argtypes = [_vp, ctypes.c_int, ctypes.c_int, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_int, ctypes.c_int, ctypes.c_int, _i32p]
    L.vnm_swap_heap_order.argtypes = [ctypes.c_int, _i32p, _i32p, _i32p]
    L.vnm_vnm_eval.argtypes = [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp, _vp, ctypes.c_int, ctypes.c_int,
                               ctypes.c_int, _i32p]
    L.vnm_vnm_reorder.argtypes = [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp, _vp, ctypes.c_int,
                                  ctypes.c_int, ctypes.c_int, ctypes.c_int, _i32p, _i32p]
    _lib = L
    return L


def status_string(s):
    return lib().vnm_status_string(int(s)).decode()


def version():
    return lib().vnm_version().decode()


def _check(st, what):
    if st != 0:
        raise VnmError(st, what)


def _ptr(a, dtype):
    if a is None:
        return None
    return ctypes.c_void_p(a.ctypes.data)


def _host(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def swap_heap_order(lg, rg):
    lg = _host(lg, np.int32)
    rg = _host(rg, np.int32)
    out = np.zeros(len(lg), np.int32)
    _check(lib().vnm_swap_heap_order(len(lg), lg.ctypes.data_as(_i32p), rg.ctypes.data_as(_i32p),
                                     out.ctypes.data_as(_i32p)), "vnm_swap_heap_order")
    return out


class Context:
    """One CUDA context handle (own stream and scratch) of the library."""

    def __init__(self, device=0):
        h = ctypes.c_void_p()
        _check(lib().vnm_create(ctypes.byref(h), int(device)), "vnm_create")
        self.h = h

    def close(self):
        if self.h:
            lib().vnm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def last_kernel_ms(self):
        return lib().vnm_last_kernel_ms(self.h)

    @property
    def last_launch_count(self):
        return lib().vnm_last_launch_count(self.h)

    @property
    def last_main_kernel_ms(self):
        return lib().vnm_last_main_kernel_ms(self.h)

    def last_stats(self):
        out = (ctypes.c_longlong * 28)()
        _check(lib().vnm_last_stats(self.h, out, 28), "vnm_last_stats")
        keys = ("rounds", "gathered", "touched", "nseg", "jobs", "pattern_nnz", "blocks_per_job", "table_rounds")
        d = dict(zip(keys, list(out)[:8]))
        d["phase_us"] = dict(zip(("select", "choose", "gather", "process", "heap_entries", "heaps_and_walk", "apply"),
                                 [x * 1.024 for x in list(out)[8:15]]))
        d["global_rounds"] = out[15]
        d["kernel_us"] = out[16] * 1.024
        d["job_start_spread_us"] = out[17]
        d["jobs_span_us"] = out[18]
        d["clusters_fit"] = out[19]
        d["leader_own_us"] = {"process": out[20] * 1.024, "apply": out[21] * 1.024}
        d["inside_us"] = dict(zip(("walk", "walk_waits", "process_warp0", "apply_warp0", "process_warp0_masks",
                                   "process_warp0_pairs"), [x * 1.024 for x in list(out)[22:28]]))
        return d

    # ---- array plumbing: numpy arrays (host) or torch CUDA tensors (device)
    @staticmethod
    def _arrays(row, col, val):
        if hasattr(row, "is_cuda") and row.is_cuda:
            import torch
            assert row.dtype == torch.int32 and col.dtype == torch.int32 and val.dtype == torch.float32
            return (ctypes.c_void_p(row.data_ptr()), ctypes.c_void_p(col.data_ptr()),
                    ctypes.c_void_p(val.data_ptr()), MEM_DEVICE, int(row.numel()), (row, col, val))
        r = _host(row, np.int32)
        c = _host(col, np.int32)
        v = _host(val, np.float32)
        return _ptr(r, np.int32), _ptr(c, np.int32), _ptr(v, np.float32), MEM_HOST, len(r), (r, c, v)

    def nm_reorder(self, nrows, row, col, val, N, M, sched, nm_maxiter=10, want_newpos=True):
        """One NM job; returns (res5, newpos or None)."""
        pr, pc, pv, mem, nnz, keep = self._arrays(row, col, val)
        res = np.zeros(5, np.int32)
        newpos = np.zeros(nrows, np.int32) if want_newpos else None
        _check(lib().vnm_nm_reorder(self.h, nrows, nnz, pr, pc, pv, mem, N, M, sched, nm_maxiter,
                                    res.ctypes.data_as(_i32p),
                                    newpos.ctypes.data_as(_i32p) if newpos is not None else None),
               "vnm_nm_reorder")
        return res, newpos

    def nm_search(self, nrows, row, col, val, N, M, nm_maxiter=10, want_newpos=True):
        """find_best_2toX over schedules 0..3: returns (best, res5x4, newpos)."""
        pr, pc, pv, mem, nnz, keep = self._arrays(row, col, val)
        res = np.zeros(20, np.int32)
        best = ctypes.c_int()
        newpos = np.zeros(nrows, np.int32) if want_newpos else None
        _check(lib().vnm_nm_search(self.h, nrows, nnz, pr, pc, pv, mem, N, M, nm_maxiter, ctypes.byref(best),
                                   res.ctypes.data_as(_i32p),
                                   newpos.ctypes.data_as(_i32p) if newpos is not None else None), "vnm_nm_search")
        return best.value, res.reshape(4, 5), newpos

    def set_trace(self, on):
        _check(lib().vnm_nm_set_trace(self.h, 1 if on else 0), "vnm_nm_set_trace")

    def set_phase_timing(self, on):
        """Per-phase timers of the round kernel (last_stats' phase_us,
        leader_own_us, inside_us); off by default, as they cost time."""
        _check(lib().vnm_nm_set_phase_timing(self.h, 1 if on else 0), "vnm_nm_set_phase_timing")

    def get_trace(self):
        """Swaps of the last traced job: list of per-round (k, 2) arrays."""
        np_, nr = ctypes.c_int(), ctypes.c_int()
        _check(lib().vnm_nm_get_trace(self.h, None, 0, ctypes.byref(np_), None, 0, ctypes.byref(nr)), "trace")
        pairs = np.zeros(2 * max(np_.value, 1), np.int32)
        ends = np.zeros(max(nr.value, 1), np.int32)
        _check(lib().vnm_nm_get_trace(self.h, pairs.ctypes.data_as(_i32p), np_.value, ctypes.byref(np_),
                                      ends.ctypes.data_as(_i32p), nr.value, ctypes.byref(nr)), "trace")
        pairs = pairs[:2 * np_.value].reshape(-1, 2)
        out, start = [], 0
        for e in ends[:nr.value].tolist():
            out.append(pairs[start:e])
            start = e
        return out

    def permute_coo(self, nrows, row, col, newpos, out=None):
        """Relabel a COO by newpos.  CUDA tensors are relabelled in place; host
        arrays are copied first, into `out` = (row_out, col_out) when given
        (int32 host arrays of the same length, e.g. pinned), else into new
        arrays."""
        if hasattr(row, "is_cuda") and row.is_cuda:
            _check(lib().vnm_permute_coo(self.h, nrows, int(row.numel()), ctypes.c_void_p(row.data_ptr()),
                                         ctypes.c_void_p(col.data_ptr()), MEM_DEVICE,
                                         ctypes.c_void_p(newpos.data_ptr())), "vnm_permute_coo")
            return row, col
        if out is not None:
            r, c = out
            if r.dtype != np.int32 or c.dtype != np.int32 or len(r) != len(row) or len(c) != len(col) \
                    or not r.flags["C_CONTIGUOUS"] or not c.flags["C_CONTIGUOUS"]:
                raise ValueError("out must be two C-contiguous int32 arrays as long as the COO")
            np.copyto(r, row, casting="same_kind")
            np.copyto(c, col, casting="same_kind")
        else:
            r = np.array(row, np.int32)
            c = np.array(col, np.int32)
        p = _host(newpos, np.int32)
        _check(lib().vnm_permute_coo(self.h, nrows, len(r), _ptr(r, None), _ptr(c, None), MEM_HOST,
                                     _ptr(p, None)), "vnm_permute_coo")
        return r, c

    def nm_segment_counts(self, nrows, row, col, val, N, M):
        pr, pc, pv, mem, nnz, keep = self._arrays(row, col, val)
        inv = np.zeros(nrows // M, np.int32)
        az = np.zeros(nrows // M, np.int32)
        _check(lib().vnm_nm_segment_counts(self.h, nrows, nnz, pr, pc, pv, mem, N, M, inv.ctypes.data_as(_i32p),
                                           az.ctypes.data_as(_i32p)), "vnm_nm_segment_counts")
        return inv, az

    def nm_pair_score(self, nrows, row, col, val, N, M, s1, s2):
        pr, pc, pv, mem, nnz, keep = self._arrays(row, col, val)
        sc = np.zeros(2 * M * M, np.int32)
        _check(lib().vnm_nm_pair_score(self.h, nrows, nnz, pr, pc, pv, mem, N, M, s1, s2,
                                       sc.ctypes.data_as(_i32p)), "vnm_nm_pair_score")
        return sc

    # ---- VNM stage (reordering.py)
    def vnm_eval(self, m, n, row, col, M, V):
        r = _host(row, np.int32)
        c = _host(col, np.int32)
        out = np.zeros(2, np.int32)
        _check(lib().vnm_vnm_eval(self.h, m, n, len(r), _ptr(r, None), _ptr(c, None), MEM_HOST, M, V,
                                  out.ctypes.data_as(_i32p)), "vnm_vnm_eval")
        return out

    def vnm_reorder(self, m, n, row, col, M, V, maxiter=10):
        """reordering.py's loop: returns (out5, row', col', newpos)."""
        r = np.array(row, np.int32)
        c = np.array(col, np.int32)
        out = np.zeros(5, np.int32)
        mp = (m + M - 1) // M * M
        newpos = np.zeros(mp, np.int32)
        _check(lib().vnm_vnm_reorder(self.h, m, n, len(r), _ptr(r, None), _ptr(c, None), MEM_HOST, M, V, maxiter,
                                     out.ctypes.data_as(_i32p), newpos.ctypes.data_as(_i32p)), "vnm_vnm_reorder")
        return out, r, c, newpos

    # ---- batches
    @staticmethod
    def pack_batch(mats):
        """The arrays of vnm_nm_reorder_batch for [(nrows, row, col, val), ...]:
        (nrows, nnz_offset, row, col, val), each matrix's entries in turn."""
        nmat = len(mats)
        nrows = np.array([m[0] for m in mats], np.int32)
        off = np.zeros(nmat + 1, np.int64)
        off[1:] = np.cumsum([len(m[1]) for m in mats])
        row = np.ascontiguousarray(np.concatenate([m[1] for m in mats]) if nmat else np.zeros(0), np.int32)
        col = np.ascontiguousarray(np.concatenate([m[2] for m in mats]) if nmat else np.zeros(0), np.int32)
        val = np.ascontiguousarray(np.concatenate([m[3] for m in mats]) if nmat else np.zeros(0), np.float32)
        return nrows, off, row, col, val

    def nm_reorder_batch(self, mats, N, M, sched, nm_maxiter=10, want_newpos=True):
        """Reorder many matrices [(nrows, row, col, val), ...] (or the arrays
        of pack_batch) in one launch.  Returns (res5 [nmat, 5], list of
        newpos arrays or None)."""
        nrows, off, row, col, val = mats if isinstance(mats, tuple) else self.pack_batch(mats)
        nmat = len(nrows)
        res = np.zeros(5 * max(nmat, 1), np.int32)
        tot = int(nrows.sum()) if nmat else 0
        newpos = np.zeros(max(tot, 1), np.int32) if want_newpos else None
        _check(lib().vnm_nm_reorder_batch(self.h, nmat, nrows.ctypes.data_as(_i32p), off.ctypes.data_as(_i64p),
                                          row.ctypes.data_as(_i32p), col.ctypes.data_as(_i32p),
                                          val.ctypes.data_as(_f32p), N, M, sched, nm_maxiter,
                                          res.ctypes.data_as(_i32p),
                                          newpos.ctypes.data_as(_i32p) if newpos is not None else None),
               "vnm_nm_reorder_batch")
        outs = None
        if want_newpos:
            ro = np.concatenate([[0], np.cumsum(nrows)])
            outs = [newpos[ro[b]:ro[b + 1]].copy() for b in range(nmat)]
        return res[:5 * nmat].reshape(nmat, 5), outs


class SpmmMatrix:
    """A matrix compressed into the V:N:M layout of the SpMM kernel."""

    def __init__(self, ctx, nrows, row, col, val, M, V, dtype="bf16"):
        L = lib()
        if not hasattr(L, "_spmm_typed"):
            L.vnm_spmm_compress.argtypes = [_vp, ctypes.c_int, ctypes.c_int, _vp, _vp, _vp, ctypes.c_int,
                                            ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(_vp)]
            L.vnm_spmm_info.argtypes = [_vp, ctypes.POINTER(ctypes.c_longlong), ctypes.c_int]
            L.vnm_spmm_run.argtypes = [_vp, _vp, _vp, ctypes.c_int, _vp, ctypes.c_int]
            L.vnm_spmm_free.argtypes = [_vp]
            L.vnm_spmm_run_async.argtypes = [_vp, _vp, _vp, ctypes.c_int, _vp, _vp]
            L.vnm_spmm_check.argtypes = [_vp, _vp, _i32p]
            L._spmm_typed = True
        self.ctx = ctx
        self.nrows = nrows
        self.dtype = dtype
        pr, pc, pv, mem, nnz, keep = ctx._arrays(row, col, val)
        h = ctypes.c_void_p()
        _check(L.vnm_spmm_compress(ctx.h, nrows, nnz, pr, pc, pv, mem, M, V, 1 if dtype == "bf16" else 0,
                                   ctypes.byref(h)), "vnm_spmm_compress")
        self.h = h

    def info(self):
        out = (ctypes.c_longlong * 13)()
        _check(lib().vnm_spmm_info(self.h, out, 13), "vnm_spmm_info")
        keys = ("nnz", "blocks", "valid_blocks", "slices", "slices_padded", "ksteps", "tiles", "a_bytes",
                "residual_nnz", "residual_tasks", "tensor_tiles", "dense_min", "split_chunks")
        return dict(zip(keys, list(out)))

    def run(self, B, C=None):
        """B: torch CUDA tensor (nrows x n, bf16/f16) or host array of the 16-bit
        words; returns C (nrows x n fp32) on B's side.  C may be given: a CUDA
        tensor, or for host B a C-contiguous float32 host array (pinned memory
        makes the device-to-host copy direct)."""
        if hasattr(B, "is_cuda") and B.is_cuda:
            import torch
            n = B.shape[1]
            if C is None:
                C = torch.empty((self.nrows, n), dtype=torch.float32, device=B.device)
            _check(lib().vnm_spmm_run(self.ctx.h, self.h, ctypes.c_void_p(B.data_ptr()), n,
                                      ctypes.c_void_p(C.data_ptr()), MEM_DEVICE), "vnm_spmm_run")
            return C
        B = np.ascontiguousarray(B)
        n = B.shape[1]
        if C is None:
            C = np.empty((self.nrows, n), np.float32)
        elif C.shape != (self.nrows, n) or C.dtype != np.float32 or not C.flags["C_CONTIGUOUS"]:
            raise ValueError("C must be a C-contiguous float32 array of shape (nrows, n)")
        _check(lib().vnm_spmm_run(self.ctx.h, self.h, ctypes.c_void_p(B.ctypes.data), n,
                                  ctypes.c_void_p(C.ctypes.data), MEM_HOST), "vnm_spmm_run")
        return C

    def run_async(self, B, C=None, stream=None):
        """C = A B enqueued on a CUDA stream (torch's current stream of B's
        device by default) without waiting; B and C are CUDA tensors.  The
        first call for an operand shape and n times the kernel widths once."""
        import torch
        n = B.shape[1]
        if C is None:
            C = torch.empty((self.nrows, n), dtype=torch.float32, device=B.device)
        if stream is None:
            stream = torch.cuda.current_stream(B.device)
        _check(lib().vnm_spmm_run_async(self.ctx.h, self.h, ctypes.c_void_p(B.data_ptr()), n,
                                        ctypes.c_void_p(C.data_ptr()), ctypes.c_void_p(stream.cuda_stream)),
               "vnm_spmm_run_async")
        return C

    def check(self, stream=None):
        """Wait for the stream; raise if an asynchronous product failed in a kernel."""
        import torch
        if stream is None:
            stream = torch.cuda.current_stream()
        failed = ctypes.c_int()
        _check(lib().vnm_spmm_check(self.h, ctypes.c_void_p(stream.cuda_stream), ctypes.byref(failed)),
               "vnm_spmm_check")
        if failed.value:
            raise VnmError(6, "vnm_spmm_run_async")

    def close(self):
        if self.h:
            lib().vnm_spmm_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# Learned-proposal reorder
# ---------------------------------------------------------------------------
LEARNED_MLP, LEARNED_EXHAUSTIVE, LEARNED_RANDOM = 0, 1, 2
MLP_FEATURES, MLP_HIDDEN = 32, 128
OBJ_INVALID, OBJ_RETAINED = 0, 1


class _LearnedParams(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int), ("objective", ctypes.c_int), ("targets", ctypes.c_int),
                ("topk", ctypes.c_int), ("max_rounds", ctypes.c_int), ("patience", ctypes.c_int), ("seed", ctypes.c_uint),
                ("dump_every", ctypes.c_int), ("dump_cap", ctypes.c_int), ("dump_features", _f32p),
                ("dump_gains", _f32p), ("stop_gain", ctypes.c_longlong)]


class _LearnedResult(ctypes.Structure):
    _fields_ = [("init_invalid", ctypes.c_longlong), ("final_invalid", ctypes.c_longlong),
                ("init_retained", ctypes.c_longlong), ("final_retained", ctypes.c_longlong),
                ("gain", ctypes.c_longlong), ("exact_scored", ctypes.c_longlong), ("rounds", ctypes.c_int),
                ("swaps", ctypes.c_int), ("ndump", ctypes.c_int), ("reserved", ctypes.c_int)]


def _learned_lib():
    L = lib()
    if not hasattr(L, "_learned_typed"):
        L.vnm_mlp_param_count.restype = ctypes.c_int
        L.vnm_mlp_create.argtypes = [_vp, ctypes.c_uint, ctypes.POINTER(_vp)]
        L.vnm_mlp_free.argtypes = [_vp]
        L.vnm_mlp_get.argtypes = [_vp, _f32p]
        L.vnm_mlp_set.argtypes = [_vp, _f32p]
        L.vnm_mlp_forward.argtypes = [_vp, _vp, _f32p, ctypes.c_int, _f32p]
        L.vnm_mlp_grad.argtypes = [_vp, _vp, _f32p, _f32p, ctypes.c_int, _f32p, _f32p]
        L.vnm_mlp_train.argtypes = [_vp, _vp, _f32p, _f32p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_float, _f32p]
        L.vnm_nm_learned.argtypes = [_vp, ctypes.c_int, ctypes.c_int, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_int, _vp, ctypes.POINTER(_LearnedParams),
                                     ctypes.POINTER(_LearnedResult), _i32p]
        L._learned_typed = True
    return L


class Mlp:
    """The swap-proposal network (FP32 master weights and Adam state on the
    device of `ctx`).  Parameters as one flat float32 vector:
    W1[128][32], b1[128], W2[128][128], b2[128], w3[128], b3."""

    def __init__(self, ctx, seed=0):
        L = _learned_lib()
        self.ctx = ctx
        h = ctypes.c_void_p()
        _check(L.vnm_mlp_create(ctx.h, int(seed), ctypes.byref(h)), "vnm_mlp_create")
        self.h = h

    @staticmethod
    def param_count():
        return _learned_lib().vnm_mlp_param_count()

    def get(self):
        p = np.zeros(self.param_count(), np.float32)
        _check(_learned_lib().vnm_mlp_get(self.h, p.ctypes.data_as(_f32p)), "vnm_mlp_get")
        return p

    def set(self, p):
        p = _host(p, np.float32)
        assert p.size == self.param_count()
        _check(_learned_lib().vnm_mlp_set(self.h, p.ctypes.data_as(_f32p)), "vnm_mlp_set")

    def forward(self, X):
        X = _host(X, np.float32).reshape(-1, MLP_FEATURES)
        Y = np.zeros(len(X), np.float32)
        _check(_learned_lib().vnm_mlp_forward(self.ctx.h, self.h, X.ctypes.data_as(_f32p), len(X),
                                              Y.ctypes.data_as(_f32p)), "vnm_mlp_forward")
        return Y

    def grad(self, X, t):
        X = _host(X, np.float32).reshape(-1, MLP_FEATURES)
        t = _host(t, np.float32)
        g = np.zeros(self.param_count(), np.float32)
        loss = ctypes.c_float()
        _check(_learned_lib().vnm_mlp_grad(self.ctx.h, self.h, X.ctypes.data_as(_f32p), t.ctypes.data_as(_f32p),
                                           len(X), g.ctypes.data_as(_f32p), ctypes.byref(loss)), "vnm_mlp_grad")
        return g, loss.value

    def train(self, X, t, batch=1024, epochs=1, lr=1e-3):
        X = _host(X, np.float32).reshape(-1, MLP_FEATURES)
        t = _host(t, np.float32)
        loss = ctypes.c_float()
        _check(_learned_lib().vnm_mlp_train(self.ctx.h, self.h, X.ctypes.data_as(_f32p), t.ctypes.data_as(_f32p),
                                            len(X), int(batch), int(epochs), float(lr), ctypes.byref(loss)),
               "vnm_mlp_train")
        return loss.value

    def close(self):
        if self.h:
            _learned_lib().vnm_mlp_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def nm_learned(ctx, nrows, row, col, val, N, M, mode=LEARNED_MLP, net=None, objective=OBJ_RETAINED, targets=16,
               topk=8, max_rounds=64, patience=2, seed=0, dump_every=0, dump_cap=0, stop_gain=0, want_newpos=True):
    """Learned-proposal (or exhaustive / random-proposal) reorder.  Returns
    (result dict, newpos or None, (features, gains) or None)."""
    L = _learned_lib()
    pr, pc, pv, mem, nnz, keep = ctx._arrays(row, col, val)
    p = _LearnedParams()
    p.mode, p.objective, p.targets, p.topk = int(mode), int(objective), int(targets), int(topk)
    p.max_rounds, p.patience, p.seed = int(max_rounds), int(patience), int(seed) & 0xffffffff
    p.stop_gain = int(stop_gain)
    dx = dy = None
    if dump_every > 0 and dump_cap > 0:
        dx = np.zeros((dump_cap, MLP_FEATURES), np.float32)
        dy = np.zeros(dump_cap, np.float32)
        p.dump_every, p.dump_cap = int(dump_every), int(dump_cap)
        p.dump_features, p.dump_gains = dx.ctypes.data_as(_f32p), dy.ctypes.data_as(_f32p)
    r = _LearnedResult()
    newpos = np.zeros(nrows, np.int32) if want_newpos else None
    _check(L.vnm_nm_learned(ctx.h, nrows, nnz, pr, pc, pv, mem, N, M, net.h if net is not None else None,
                            ctypes.byref(p), ctypes.byref(r),
                            newpos.ctypes.data_as(_i32p) if newpos is not None else None), "vnm_nm_learned")
    res = {k: getattr(r, k) for k, _ in _LearnedResult._fields_ if k != "reserved"}
    dump = (dx[:r.ndump], dy[:r.ndump]) if dx is not None else None
    return res, newpos, dump


# ---------------------------------------------------------------------------
# Matrix Market files (host code of the library; no GPU needed)
# ---------------------------------------------------------------------------
def _io_lib():
    L = lib()
    if not hasattr(L, "_io_typed"):
        L.vnm_mtx_read.argtypes = [ctypes.c_char_p, ctypes.c_int, _i32p, _i32p, _i32p, ctypes.POINTER(_i32p),
                                   ctypes.POINTER(_i32p), ctypes.POINTER(_f32p)]
        L.vnm_mtx_write.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _i32p, _i32p, _f32p]
        L.vnm_host_free.argtypes = [ctypes.c_void_p]
        L._io_typed = True
    return L


def read_mtx(path, aligned=1):
    """readMtx + the row padding of Mtx::init_from_file: (nrows, ncols, row,
    col, val), sorted by (row, col), repeats removed, symmetric mirrored."""
    L = _io_lib()
    nr, nc, nz = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    r, c, v = _i32p(), _i32p(), _f32p()
    _check(L.vnm_mtx_read(os.fsencode(path), int(aligned), nr, nc, nz, ctypes.byref(r), ctypes.byref(c),
                          ctypes.byref(v)), "vnm_mtx_read")
    n = nz.value
    out = []
    for p, t in ((r, np.int32), (c, np.int32), (v, np.float32)):
        out.append(np.ctypeslib.as_array(p, shape=(n,)).astype(t, copy=True) if n else np.zeros(0, t))
        L.vnm_host_free(ctypes.cast(p, ctypes.c_void_p))
    return (nr.value, nc.value) + tuple(out)


def write_mtx(path, nrows, ncols, row, col, val):
    """Mtx::write_to_file: "real general" banner, "%d %d %.2f" lines, 1-based."""
    L = _io_lib()
    r, c, v = _host(row, np.int32), _host(col, np.int32), _host(val, np.float32)
    _check(L.vnm_mtx_write(os.fsencode(path), int(nrows), int(ncols), len(r), r.ctypes.data_as(_i32p),
                           c.ctypes.data_as(_i32p), v.ctypes.data_as(_f32p)), "vnm_mtx_write")
