"""The allocation-free NM entry point, checked against vnm_nm_reorder.

vnm_nm_reorder_noalloc serves callers that cannot call cudaMalloc (their
device memory is owned by their own allocator, or their loop may not
allocate): it takes its scratch from a fixed device array instead.  This
test calls it through the C ABI with device buffers the test owns, twice in
a row on different inputs (the array keeps the previous call's contents),
and requires results identical to the allocating entry point's.  It lives in
its own file, collected last, so that a stop at the first failure has run
every other test before it.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(lib, nr, tr, tc, tv, N, M, sched, torch):
    res = torch.zeros(5, dtype=torch.int32, device="cuda")
    newpos = torch.full((nr,), -1, dtype=torch.int32, device="cuda")
    fn = lib.vnm_nm_reorder_noalloc
    fn.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                   ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    stream = torch.cuda.current_stream().cuda_stream
    st = fn(nr, int(tr.numel()), tr.data_ptr(), tc.data_ptr(), tv.data_ptr(), N, M, sched, 10, res.data_ptr(),
            newpos.data_ptr(), ctypes.c_void_p(stream))
    assert st == 0, "vnm_nm_reorder_noalloc returned %d" % st
    return res.cpu().numpy(), newpos.cpu().numpy()


def test_noalloc_matches_allocating_entry_point_twice():
    torch = pytest.importorskip("torch")
    import vnm_gb300
    from vnm_gb300 import synth
    lib = vnm_gb300.lib()
    cases = [(synth.rmat(12, 16384, 31, "normal"), 2, 4, 3),   # 4096 rows, 2:4
             (synth.uniform(512, 0.02, 0), 2, 8, 1)]          # smaller second call on the same scratch
    with vnm_gb300.Context(0) as ctx:
        for (nr, r, c, v), N, M, sched in cases:
            tr = torch.from_numpy(r).cuda()
            tc = torch.from_numpy(c).cuda()
            tv = torch.from_numpy(v).cuda()
            got_res, got_pos = _noalloc(lib, nr, tr, tc, tv, N, M, sched, torch)
            want_res, want_pos = ctx.nm_reorder(nr, r, c, v, N, M, sched)
            assert np.array_equal(got_res, want_res), (got_res, want_res)
            assert np.array_equal(got_pos, want_pos)


def test_noalloc_rejects_sizes_above_its_limit():
    torch = pytest.importorskip("torch")
    import vnm_gb300
    lib = vnm_gb300.lib()
    nr = 32768 + 8
    z = torch.zeros(1, dtype=torch.int32, device="cuda")
    v = torch.ones(1, dtype=torch.float32, device="cuda")
    res = torch.zeros(5, dtype=torch.int32, device="cuda")
    pos = torch.zeros(nr, dtype=torch.int32, device="cuda")
    fn = lib.vnm_nm_reorder_noalloc
    fn.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                   ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    st = fn(nr, 1, z.data_ptr(), z.data_ptr(), v.data_ptr(), 2, 4, 0, 10, res.data_ptr(), pos.data_ptr(), None)
    assert st == 10  # VNM_ERR_LIMIT
