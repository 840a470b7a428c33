"""Shared helpers of the GPU tests: run a stream through the C ABI and check it with the oracle."""
import numpy as np

import csmv_gb300 as cg
import oracle as orc


def c1_workload(n_txn=8 * 128 * 256, seed=1, **kw):
    """4096 accounts at 1000, 90% transfers of 1..10 between 2 distinct uniform accounts (skip
    if insufficient), 10% read-only sums of 8 uniform accounts."""
    d = dict(seed=seed, pr_read_pct=10, ro_reads=8, up_reads=2, kind=cg.KIND_TRANSFER, amt_lo=1,
             amt_hi=10, dist=cg.DIST_UNIFORM)
    d.update(kw)
    n_acc = d.pop("n_accounts", 4096)
    return cg.bank_workload(n_acc, n_txn, **d)


def run_checked(w, *, init_value=1000, check=True, stream=None, txn_aborts=None, split_round=0,
                deferred_warps=0, lane_start=None, **cfg):
    """Run workload w (or a given stream over its accounts) on a fresh bank; returns (stats,
    stream, bank outputs); asserts exactness."""
    s = cg.generate(w) if stream is None else stream
    cfg.setdefault("max_txn", w.n_txn)
    depth = cfg.setdefault("version_depth", 4)
    with cg.Bank(n_accounts=w.n_accounts, init_value=init_value, **cfg) as bank:
        bank.load()
        st = bank.run(s, txn_aborts=txn_aborts, split_round=split_round,
                      deferred_warps=deferred_warps, lane_start=lane_start)
        log_txn, outcome, result = bank.log(w.n_txn, st.final_ts)
        groups = bank.groups(st.final_ts)
        slots = bank.versions()
    assert st.error == 0
    assert st.commits == w.n_txn, (st.commits, w.n_txn)
    if cfg.get("validate", cg.VALIDATE_STAMP) == cg.VALIDATE_STAMP:
        # timestamps of transactions that failed validation after taking one are holes
        assert st.commits_update <= st.final_ts
        logged = np.count_nonzero(log_txn != 0xFFFFFFFF)  # chained links may commit no writes
        assert st.commits_update <= logged <= st.commits_update + st.commits_nowrite
    else:
        assert st.commits_update == st.final_ts  # the reference's dense commit order
    if check:
        init = np.full(w.n_accounts, init_value, np.int32)
        err = orc.check(s.op, s.off, s.addr, w.n_accounts, init, depth, st.final_ts, log_txn,
                        outcome, result, slots, groups=groups)
        assert err is None, err
    return st, s, (log_txn, outcome, result, slots)


def memcd_run_checked(cache, req, *, check=True, tick=None):
    """One cache batch through the C ABI, checked against the oracle's serial replay from the
    table as it was before the batch. Returns (found, val_out, stats)."""
    table0 = cache.table() if check else None
    found, val_out, st = cache.run(req, tick=tick)
    t = cache.tick - 1 if tick is None else tick
    assert st.error == 0
    n_set = int(np.count_nonzero(req.kind == cg.MEMCD_SET))
    assert st.commits_update == n_set and st.commits_readonly == req.n_req - n_set
    if check:
        log_txn, outcome, base = cache.log(req.n_req)
        tags, recs = cache.table()
        orc.memcd_check(req.kind, req.key, req.val, t, cache.cfg.n_sets, table0, base, log_txn,
                        outcome, found, val_out, tags, recs)
    return found, val_out, st


def defer_plan(s, risky):
    """Permutation putting the update transactions flagged risky into a deferred queue at the
    end of the stream (rounds stay uniform in kind). Returns (permuted stream, split_round)."""
    n = s.n_txn
    rr = np.repeat((s.op[::32] & 3) == 0, 32)
    idx = np.arange(n)
    upd = idx[~rr]
    rk = risky[upd]
    safe_u, risky_u = upd[~rk], upd[rk]
    pad = (-len(risky_u)) % 32
    main = np.concatenate([idx[rr], safe_u[pad:]])
    perm = np.concatenate([main, risky_u, safe_u[:pad]])
    return cg.Stream(np.ascontiguousarray(s.op[perm]), np.ascontiguousarray(s.off[perm]),
                     s.addr), len(main) // 32


def to_device(torch, s):
    """Device copy of a host stream: (BankStream with device pointers, tensors to keep alive)."""
    d = [torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda() for a in (s.op, s.off, s.addr)]
    return cg.BankStream(s.n_txn, d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(),
                         int(s.addr.shape[0])), d


def concat_groups(parts):
    """Group-end bitmaps of consecutive runs joined into one over the runs' timestamps:
    parts = [(bitmap words, timestamps the run used), ...]."""
    bits = [np.unpackbits(np.ascontiguousarray(w, np.uint32).view(np.uint8),
                          bitorder="little")[:n] for w, n in parts]
    allb = np.concatenate(bits) if bits else np.zeros(0, np.uint8)
    pad = np.zeros((-len(allb)) % 32, np.uint8)
    return np.packbits(np.concatenate([allb, pad]), bitorder="little").view(np.uint32)


def zipf_bank_workload(n_txn, seed=2026):
    """The contended bank: 2^20 accounts at 1000, Zipf(0.99) account choice, transfers reading 4
    and writing 2 accounts (skipped when funds are short), 20 % read-only rounds summing 32."""
    return cg.bank_workload(1 << 20, n_txn, seed=seed, pr_read_pct=20, ro_reads=32, up_reads=4,
                            kind=cg.KIND_TRANSFER, amt_lo=1, amt_hi=10, dist=cg.DIST_ZIPF,
                            zipf_theta=0.99)


def sub_stream(s, lo, hi):
    """Transactions [lo, hi) of a host stream (addresses shared)."""
    return cg.Stream(np.ascontiguousarray(s.op[lo:hi]), np.ascontiguousarray(s.off[lo:hi]), s.addr)
