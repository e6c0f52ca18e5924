"""Parity of the CUDA NM reorder (through the C ABI) with the oracle and with
the reference's own results (tests/golden/nm_ref_goldens.npz).

Bit-exact throughout: the path is integer-only."""
import numpy as np
import pytest

import oracle
from golden_cases import nm_cases, nm_input

pytestmark = pytest.mark.gpu


def _keys(goldens):
    return sorted({key for _, key, _, _, _ in nm_cases(goldens)})


def test_segment_counts_match_oracle(ctx, goldens):
    for key in _keys(goldens):
        nr, r, c, v = nm_input(goldens, key)
        N, M = int(key.split("__n")[1].split("_")[0]), int(key.split("_m")[-1])
        inv, az = ctx.nm_segment_counts(nr, r, c, v, N, M)
        oinv, oaz = oracle.nm_segment_counts(nr, r, c, v, N, M)
        assert np.array_equal(inv, oinv), key
        assert np.array_equal(az, oaz), key


def test_pair_scores_match_oracle(ctx, goldens):
    rng = np.random.default_rng(0)
    for key in _keys(goldens):
        nr, r, c, v = nm_input(goldens, key)
        N, M = int(key.split("__n")[1].split("_")[0]), int(key.split("_m")[-1])
        nseg = nr // M
        pairs = [(0, 0), (0, nseg - 1)] + [tuple(rng.integers(0, nseg, 2)) for _ in range(6)]
        for s1, s2 in pairs:
            got = ctx.nm_pair_score(nr, r, c, v, N, M, int(s1), int(s2))
            want = oracle.nm_pair_score(nr, r, c, v, N, M, int(s1), int(s2))
            assert np.array_equal(got, want), (key, s1, s2)


def test_reorder_matches_oracle_every_case(ctx, goldens):
    bad = []
    for case, key, N, M, s in nm_cases(goldens):
        nr, r, c, v = nm_input(goldens, key)
        res, newpos = ctx.nm_reorder(nr, r, c, v, N, M, s)
        ores, _, _, opos = oracle.nm_run(nr, r, c, v, N, M, s)
        if not (np.array_equal(res, ores) and np.array_equal(newpos, opos)):
            bad.append((case, res.tolist(), ores.tolist()))
    assert not bad, bad[:5]


def test_phase_timers_change_nothing_but_the_stats(ctx, goldens):
    """The round kernel's phase timers are off by default (their stats read
    0); on, they fill the stats, and the results are the same either way."""
    nr, r, c, v = nm_input(goldens, "rmat_2048__n2_m4")
    best0, res0, pos0 = ctx.nm_search(nr, r, c, v, 2, 4)
    st = ctx.last_stats()
    assert sum(st["phase_us"].values()) == 0 and st["inside_us"]["walk"] == 0
    assert st["rounds"] > 0 and st["kernel_us"] > 0
    ctx.set_phase_timing(True)
    try:
        best1, res1, pos1 = ctx.nm_search(nr, r, c, v, 2, 4)
        st = ctx.last_stats()
    finally:
        ctx.set_phase_timing(False)
    assert all(st["phase_us"][k] > 0 for k in ("gather", "process", "heaps_and_walk", "apply"))
    assert st["inside_us"]["walk"] > 0
    assert best0 == best1 and np.array_equal(res0, res1) and np.array_equal(pos0, pos1)


def test_reorder_trace_matches_oracle(ctx, goldens):
    ctx.set_trace(True)
    try:
        for key in ("rmat_1024__n2_m8", "rmat_2048__n2_m4", "lund_b__n2_m8", "c1_512__n1_m4"):
            nr, r, c, v = nm_input(goldens, key)
            N, M = int(key.split("__n")[1].split("_")[0]), int(key.split("_m")[-1])
            for s in range(4):
                res, _ = ctx.nm_reorder(nr, r, c, v, N, M, s)
                tr = ctx.get_trace()
                ores, otr = oracle.nm_run_trace(nr, r, c, v, N, M, s)
                assert len(tr) == len(otr), (key, s)
                for k, (a, b) in enumerate(zip(tr, otr)):
                    assert np.array_equal(a, b), (key, s, "round", k)
    finally:
        ctx.set_trace(False)


def test_reorder_matches_reference_goldens(ctx, goldens):
    """Against the numbers the reference's own GPU code produced."""
    bad = []
    for case, key, N, M, s in nm_cases(goldens):
        nr, r, c, v = nm_input(goldens, key)
        res, newpos = ctx.nm_reorder(nr, r, c, v, N, M, s)
        pos = goldens["pos__" + case]
        m = pos >= 0
        if not (np.array_equal(res, goldens["res__" + case]) and np.array_equal(newpos[m], pos[m])):
            bad.append(case)
    assert not bad, "%d of the reference cases differ, e.g. %s" % (len(bad), bad[:4])


def test_search_picks_like_find_best(ctx, goldens):
    for key in ("c1_512__n2_m8", "rmat_1024__n2_m4", "u256_d05__n1_m4", "GD01_c__n2_m8"):
        nr, r, c, v = nm_input(goldens, key)
        N, M = int(key.split("__n")[1].split("_")[0]), int(key.split("_m")[-1])
        best, res, newpos = ctx.nm_search(nr, r, c, v, N, M)
        obest, _ = oracle.find_best(nr, r, c, v, N, M)
        assert best == obest, key
        for s in range(4):
            ores, _, _, _ = oracle.nm_run(nr, r, c, v, N, M, s)
            assert np.array_equal(res[s], ores), (key, s)
        ores, _, _, opos = oracle.nm_run(nr, r, c, v, N, M, best)
        assert np.array_equal(newpos, opos), key


def test_device_pointers_and_permute(ctx, goldens):
    import torch
    nr, r, c, v = nm_input(goldens, "rmat_2048__n2_m4")
    tr = torch.from_numpy(r.astype(np.int32)).cuda()
    tc = torch.from_numpy(c.astype(np.int32)).cuda()
    tv = torch.from_numpy(v.astype(np.float32)).cuda()
    res, newpos = ctx.nm_reorder(nr, tr, tc, tv, 2, 4, 1)
    ores, orow, ocol, opos = oracle.nm_run(nr, r, c, v, 2, 4, 1)
    assert np.array_equal(res, ores) and np.array_equal(newpos, opos)
    pr, pc = ctx.permute_coo(nr, tr, tc, torch.from_numpy(newpos).cuda())
    assert np.array_equal(pr.cpu().numpy(), orow) and np.array_equal(pc.cpu().numpy(), ocol)
    hr, hc = ctx.permute_coo(nr, r, c, newpos)
    assert np.array_equal(hr, orow) and np.array_equal(hc, ocol)


def test_errors_are_reported(ctx):
    import vnm_gb300
    r = np.array([1, 0], np.int32)  # not sorted
    c = np.array([0, 1], np.int32)
    v = np.ones(2, np.float32)
    with pytest.raises(vnm_gb300.VnmError) as e:
        ctx.nm_reorder(8, r, c, v, 2, 4, 0)
    assert e.value.status == 3
    with pytest.raises(vnm_gb300.VnmError) as e:
        ctx.nm_reorder(8, np.array([0], np.int32), np.array([9], np.int32), v[:1], 2, 4, 0)
    assert e.value.status == 4
    with pytest.raises(vnm_gb300.VnmError):
        ctx.nm_reorder(6, r[:0], c[:0], v[:0], 2, 4, 0)  # nrows not a multiple of M
    res, newpos = ctx.nm_reorder(8, r[:0], c[:0], v[:0], 2, 4, 0)  # empty matrix
    assert res.tolist() == [0, 0, 0, 0, 0] and newpos.tolist() == list(range(8))


@pytest.mark.parametrize("table", ["1", "0"])
@pytest.mark.parametrize("M", [4, 8])
def test_cluster_sizes_agree(ctx, M, table):
    """Each job runs on a thread-block cluster whose size depends on the
    matrix; each block owns the rows whose group (row & 15 rotated by a hash
    of the higher bits) is in its share of the 16 and keeps their records
    in its shared-memory table or, with
    VNM_NM_ROW_TABLE=0, in global memory; every size and both places give
    the oracle's result bit for bit."""
    import os
    from vnm_gb300 import synth
    n, r, c, v = synth.rmat(12, 4096 * 8, 17 + M, "normal")
    ores, _, _, opos = oracle.nm_run(n, r, c, v, 2, M, 1)
    old = {k: os.environ.get(k) for k in ("VNM_NM_CLUSTER", "VNM_NM_ROW_TABLE")}
    try:
        os.environ["VNM_NM_ROW_TABLE"] = table
        for cs in ("1", "2", "4", "8", "16"):
            os.environ["VNM_NM_CLUSTER"] = cs
            res, newpos = ctx.nm_reorder(n, r, c, v, 2, M, 1)
            assert np.array_equal(res, ores), cs
            assert np.array_equal(newpos, opos), cs
            st = ctx.last_stats()
            assert st["blocks_per_job"] == int(cs)
            if table == "1":
                assert st["table_rounds"] > 0, st
            else:
                assert st["table_rounds"] == 0 and st["global_rounds"] == res[4] * int(cs), st
    finally:
        for k, v0 in old.items():
            if v0 is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v0


def _large_gain_matrix():
    # segments 0..3 at 2:4 each with 3000 rows holding three of their nodes
    rng = np.random.default_rng(5)
    n = 8192
    rs, cs = [rng.integers(0, n, 20000)], [rng.integers(0, n, 20000)]
    for s in range(4):
        hub_rows = rng.choice(np.arange(16, n), 3000, replace=False)
        rs.append(np.repeat(hub_rows, 3))
        cs.append(np.tile([4 * s, 4 * s + 1, 4 * s + 2], 3000))
    r, c = np.concatenate(rs), np.concatenate(cs)
    key = np.unique(r.astype(np.int64) * n + c)
    r, c = (key // n).astype(np.int32), (key % n).astype(np.int32)
    return n, r, c, rng.uniform(0.5, 1.0, len(r)).astype(np.float32)


def test_large_gains_match_oracle(ctx):
    """Swap gains beyond +-2047 (four segments with 3000 rows holding three
    of their nodes, 2:4): the swap heaps order such keys by rank instead of
    packing them directly; the result is still the oracle's, for every
    schedule."""
    n, r, c, v = _large_gain_matrix()
    for sched in range(4):
        ores, _, _, opos = oracle.nm_run(n, r, c, v, 2, 4, sched)
        res, newpos = ctx.nm_reorder(n, r, c, v, 2, 4, sched)
        assert np.array_equal(res, ores), sched
        assert np.array_equal(newpos, opos), sched


@pytest.mark.parametrize("M", [2, 3, 5, 6, 7])
def test_other_group_sizes_match_oracle(ctx, M):
    """Group sizes besides 4 and 8 (the reference takes M from mtx/Mtx.h):
    every schedule against the oracle, on a cluster and on one block."""
    import os
    from vnm_gb300 import synth
    nr, r, c, v = synth.uniform(128 * M, 0.04, 30 + M)
    N = max(1, M // 2)
    old = os.environ.get("VNM_NM_CLUSTER")
    try:
        for cs in ("8", "1"):
            os.environ["VNM_NM_CLUSTER"] = cs
            for sched in range(4):
                ores, _, _, opos = oracle.nm_run(nr, r, c, v, N, M, sched)
                res, newpos = ctx.nm_reorder(nr, r, c, v, N, M, sched)
                assert np.array_equal(res, ores), (cs, sched)
                assert np.array_equal(newpos, opos), (cs, sched)
    finally:
        if old is None:
            os.environ.pop("VNM_NM_CLUSTER", None)
        else:
            os.environ["VNM_NM_CLUSTER"] = old


def test_uneven_rows_mix_table_and_global_records(ctx):
    """With clusters of 16 blocks, block b owns the rows of group b
    (row_group).  Here the only invalid segment touches 4608 rows that all
    fall in group 0: block 0's entries are more than 3/4 of its table, so it
    keeps its records in global memory while the other blocks use their
    tables in the same rounds, and the result is still the oracle's."""
    import os
    R = 81920
    hi = np.arange(4608, dtype=np.uint64)
    rot = ((hi * np.uint64(2654435761)) & np.uint64(0xffffffff)) >> np.uint64(28)  # row_group's rotation
    rows = (hi * np.uint64(16) + ((np.uint64(16) - rot) & np.uint64(15))).astype(np.int64)  # one group-0 row per 16
    r = np.concatenate([np.repeat(rows, 3), rows])
    c = np.concatenate([np.tile([0, 1, 2], len(rows)), np.full(len(rows), 5)])  # three nodes of segment 0, one of 1
    key = np.unique(r * R + c)
    r, c = (key // R).astype(np.int32), (key % R).astype(np.int32)
    v = np.ones(len(r), np.float32)
    ores, _, _, opos = oracle.nm_run(R, r, c, v, 2, 4, 0)
    old = {k: os.environ.get(k) for k in ("VNM_NM_CLUSTER", "VNM_NM_ROW_TABLE")}
    try:
        os.environ["VNM_NM_CLUSTER"] = "16"
        os.environ.pop("VNM_NM_ROW_TABLE", None)
        res, newpos = ctx.nm_reorder(R, r, c, v, 2, 4, 0)
        st = ctx.last_stats()
        assert st["blocks_per_job"] == 16
        assert st["global_rounds"] > 0 and st["table_rounds"] > 0, st
        assert np.array_equal(res, ores) and np.array_equal(newpos, opos)
    finally:
        for k, v0 in old.items():
            if v0 is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v0
