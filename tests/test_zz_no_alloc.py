"""The allocation-free bank entry point, csmv_bank_run_noalloc, against the engine's own.

Some callers of this library cannot allocate device memory once they are running - a host that
hands the library a fixed budget, or a process whose device memory belongs to another allocator
- so csmv_bank_run_noalloc keeps its scratch in a fixed device array and takes only inputs and
outputs. This test calls it through the C ABI and checks, on two calls in a row, that it gives
exactly what csmv_bank_create + csmv_bank_run_device give on the same inputs: final account
values, per-transaction outcomes and read-only sums (integer results, so the tolerance is
zero). One CTA with one client warp makes both runs deterministic. The file is named to be
collected last.
"""
import ctypes as C

import numpy as np
import pytest

import csmv_gb300 as cg
from gpu_util import c1_workload

pytestmark = pytest.mark.gpu
MAX_ACCOUNTS = MAX_TXN = 65536  # CSMV_NOALLOC_MAX_ACCOUNTS / CSMV_NOALLOC_MAX_TXN


def _noalloc():
    L = cg.lib()
    fn = L.csmv_bank_run_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_int32, C.c_void_p, C.c_uint32, C.c_void_p, C.POINTER(cg.BankStream),
                   C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p,
                   C.POINTER(cg.Stats)]
    return fn


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda()


def _engine(torch, w, s, init):
    d = [_dev(torch, x) for x in (s.op, s.off, s.addr)]
    ds = cg.BankStream(w.n_txn, d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(),
                       int(s.addr.shape[0]))
    with cg.Bank(n_accounts=w.n_accounts, version_depth=4, ctas=1, client_warps=1,
                 max_txn=w.n_txn, validate=cg.VALIDATE_STAMP, batch=cg.BATCH_CTA,
                 writeback=cg.WRITEBACK_CLIENT, prevalidate=1) as bank:
        bank.load(init)
        st = bank.run_device(ds)
        torch.cuda.synchronize()
        _, outcome, result = bank.log(w.n_txn, st.final_ts)
        return bank.values(), outcome, result, st


def _call(torch, fn, w, s, init, aborts=None, **kw):
    d = [_dev(torch, x) for x in (s.op, s.off, s.addr)]
    ds = cg.BankStream(w.n_txn, d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(),
                       int(s.addr.shape[0]))
    if aborts is not None:
        ds.txn_aborts = aborts.data_ptr()
    d_init = _dev(torch, init)
    vals = torch.full((w.n_accounts,), -7, dtype=torch.int32, device="cuda")
    outc = torch.full((w.n_txn,), -7, dtype=torch.int32, device="cuda")
    res = torch.full((w.n_txn,), -7, dtype=torch.int32, device="cuda")
    st = cg.Stats()
    rc = fn(0, None, w.n_accounts, d_init.data_ptr(), C.byref(ds), kw.get("client_warps", 1),
            kw.get("ctas", 1), vals.data_ptr(), outc.data_ptr(), res.data_ptr(), C.byref(st))
    torch.cuda.synchronize()
    return rc, vals.cpu().numpy(), outc.cpu().numpy().view(np.uint32), res.cpu().numpy(), st


@pytest.mark.parametrize("n_accounts,n_txn", [(600, 32 * 200), (MAX_ACCOUNTS, MAX_TXN)])
def test_noalloc_matches_engine_on_two_calls_in_a_row(n_accounts, n_txn):
    torch = pytest.importorskip("torch")
    fn = _noalloc()
    w = c1_workload(n_txn=n_txn, n_accounts=n_accounts, seed=21, pr_read_pct=20)
    s = cg.generate(w)
    init = np.random.default_rng(3).integers(0, 2000, n_accounts).astype(np.int32)
    want_vals, want_outc, want_res, want_st = _engine(torch, w, s, init)
    for _ in range(2):
        rc, vals, outc, res, st = _call(torch, fn, w, s, init)
        assert rc == 0, cg.lib().csmv_last_error()
        np.testing.assert_array_equal(vals, want_vals)
        np.testing.assert_array_equal(outc, want_outc)
        np.testing.assert_array_equal(res, want_res)
        assert (st.commits_update, st.commits_readonly, st.commits_nowrite, st.final_ts) == (
            want_st.commits_update, want_st.commits_readonly, want_st.commits_nowrite,
            want_st.final_ts)
        assert int(vals.astype(np.int64).sum()) == int(init.astype(np.int64).sum())


def test_noalloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    fn = _noalloc()
    w = c1_workload(n_txn=64, n_accounts=MAX_ACCOUNTS + 1)
    s = cg.generate(w)
    rc, *_ = _call(torch, fn, w, s, np.zeros(w.n_accounts, np.int32))
    assert rc == 5 and b"scratch limit" in cg.lib().csmv_last_error()
    w = c1_workload(n_txn=MAX_TXN + 32, n_accounts=100)
    s = cg.generate(w)
    rc, *_ = _call(torch, fn, w, s, np.zeros(100, np.int32))
    assert rc == 5 and b"scratch limit" in cg.lib().csmv_last_error()


def test_noalloc_full_grid_keeps_the_invariants_on_two_calls_in_a_row():
    """The default launch shape (every co-resident CTA, 15 client warps each) on a contended bank:
    many warps overlap, timestamps interleave across CTAs and the completion-bitmap ring turns
    over. No commit log leaves the fixed scratch, so the checks are the invariants: every
    transaction commits once, the balance is conserved, each outcome is a distinct commit
    timestamp within the run or a snapshot, and the per-transaction failed-attempt counts passed
    through add up to the aborts reported."""
    torch = pytest.importorskip("torch")
    fn = _noalloc()
    w = c1_workload(n_txn=MAX_TXN, n_accounts=4096, seed=23, pr_read_pct=20,
                    dist=cg.DIST_ZIPF, zipf_theta=0.9, up_reads=4)
    s = cg.generate(w)
    init = np.full(w.n_accounts, 1000, np.int32)
    for _ in range(2):
        ab = torch.zeros(w.n_txn, dtype=torch.int32, device="cuda")
        rc, vals, outc, res, st = _call(torch, fn, w, s, init, aborts=ab, ctas=0, client_warps=15)
        assert rc == 0, cg.lib().csmv_last_error()
        assert st.commits_update + st.commits_readonly + st.commits_nowrite == w.n_txn
        assert int(vals.astype(np.int64).sum()) == int(init.astype(np.int64).sum())
        snap = (outc & np.uint32(cg.SNAP_FLAG)) != 0
        ts = outc[~snap]
        assert ts.size == st.commits_update and len(np.unique(ts)) == ts.size
        assert ts.min() >= 1 and ts.max() <= st.final_ts
        assert ((outc[snap] & np.uint32(0x7FFFFFFF)) <= st.final_ts).all()
        assert int(ab.sum()) == st.aborts


def test_noalloc_reports_a_full_timestamp_log_as_capacity():
    """Four accounts, every transfer reading all four and writing two, unconditionally, on every
    SM: two warps can hold disjoint pairs of locks at once and each then fails to validate the
    other pair's reads, so nearly every timestamp drawn ends as a hole and the run needs more
    timestamps than the fixed scratch's log holds; the call must stop and say so
    (CSMV_ERR_CAPACITY, with a message naming the limit)."""
    torch = pytest.importorskip("torch")
    fn = _noalloc()
    w = c1_workload(n_txn=MAX_TXN, n_accounts=4, seed=5, pr_read_pct=0, up_reads=4,
                    kind=cg.KIND_TRANSFER_ALWAYS)
    s = cg.generate(w)
    rc, _, _, _, st = _call(torch, fn, w, s, np.full(4, 1000, np.int32), ctas=0, client_warps=15)
    if rc == 0:
        pytest.skip(f"the run fit in the log ({st.final_ts} timestamps)")
    assert rc == 5, cg.lib().csmv_last_error()
    assert b"commit timestamps" in cg.lib().csmv_last_error()
