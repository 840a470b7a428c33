"""GPU tests of the learned conflict scheduler (csmv_sched_*): its plans are permutations that
keep rounds uniform in kind, a scheduled chunk replays exactly (the engine still validates every
transaction), and on a shifting-hotspot bank the trained network lowers the abort rate against
the same engine running the stream in its given order."""
import numpy as np
import pytest

import csmv_gb300 as cg
import oracle as orc
from gpu_util import c1_workload, concat_groups, to_device, zipf_bank_workload

pytestmark = pytest.mark.gpu
HOLE = 0xFFFFFFFF


@pytest.mark.parametrize("threshold,defer", [(0.0, 2.0), (0.0, 0.3), (0.05, 2.0)])
def test_scheduled_chunk_is_a_permutation_and_replays_exactly(threshold, defer):
    torch = pytest.importorskip("torch")
    n_acc, n = 1 << 14, 1 << 15
    w = c1_workload(n_txn=n, n_accounts=n_acc, dist=cg.DIST_HOTSPOT, hot_frac=0.01,
                    hot_prob=0.4, seed=8)
    s = cg.generate(w)
    ds, keep = to_device(torch, s)
    with cg.Bank(n_accounts=n_acc, max_txn=n, ctas=16, client_warps=4) as bank, \
            cg.Scheduler(n_accounts=n_acc, max_txn=n, threshold=threshold, defer_threshold=defer,
                         deferred_warps=8, train_steps=3, plan=0) as sched:
        bank.load()
        r1 = sched.probe(bank, ds)
        f1 = r1.probe.final_ts
        np_ = r1.n_probe
        log1, out1, res1 = bank.log(np_, f1)
        r2 = sched.plan_run(bank, ds)
        f2 = r2.planned.final_ts
        perm, probe_rounds, split = sched.plan(n)
        log2, out2, res2 = bank.log(n - np_, f2 - f1)
        slots = bank.versions()
    assert probe_rounds * 32 == np_ and len(perm) == n - np_
    assert sorted(perm.tolist()) == list(range(np_, n))
    kinds = (s.op[perm] & 3).reshape(-1, 32)
    assert ((kinds == 0) == (kinds[:, :1] == 0)).all()  # rounds stay uniform in kind
    if defer < 1.0:
        assert r2.n_deferred_rounds > 0 and split > 0
    op_c = np.concatenate([s.op[:np_], s.op[perm]])
    off_c = np.concatenate([s.off[:np_], s.off[perm]])
    log_c = np.concatenate([log1, np.where(log2 != HOLE, log2 + np_, HOLE)]).astype(np.uint32)
    err = orc.check(op_c, off_c, s.addr, n_acc, np.full(n_acc, 1000, np.int32), 4, f2, log_c,
                    np.concatenate([out1, out2]), np.concatenate([res1, res2]), slots)
    assert err is None, err
    assert r1.probe.commits + r2.planned.commits == n


def _hotspot_chunks(n_acc, chunk, n_chunks, hot_prob, seed=3):
    w = cg.bank_workload(n_acc, chunk * n_chunks, seed=seed, pr_read_pct=10, ro_reads=8,
                         up_reads=2, dist=cg.DIST_HOTSPOT, hot_frac=0.01, hot_prob=hot_prob,
                         shift_every=1 << 20)
    s = cg.generate(w)
    return s, [(i * chunk, (i + 1) * chunk) for i in range(n_chunks)]


def test_trained_scheduler_lowers_abort_rate_on_shifting_hotspot():
    """1 M accounts, a 1 % hot set drawing 30 % of the accesses that moves every 2^20
    transactions; eight chunks of 2^18. Plain: the engine runs each chunk in stream order.
    Learned: the scheduler probes, trains and plans each chunk. The learned abort rate must be
    at least 30 % lower, with every transaction committed and the balance conserved."""
    torch = pytest.importorskip("torch")
    n_acc, chunk, n_chunks = 1 << 20, 1 << 18, 8
    s, bounds = _hotspot_chunks(n_acc, chunk, n_chunks, 0.3)
    res = {}
    for arm in ("plain", "learned"):
        commits = aborts = 0
        ms = 0.0
        with cg.Bank(n_accounts=n_acc, max_txn=chunk, ctas=152, client_warps=2, version_depth=8,
                     log_commits=0) as bank:
            bank.load()
            sched = cg.Scheduler(n_accounts=n_acc, max_txn=chunk, plan=0) \
                if arm == "learned" else None
            for lo, hi in bounds:
                c = cg.Stream(np.ascontiguousarray(s.op[lo:hi]), np.ascontiguousarray(s.off[lo:hi]),
                              s.addr)
                ds, keep = to_device(torch, c)
                if sched is None:
                    st = bank.run_device(ds)
                    commits, aborts, ms = commits + st.commits, aborts + st.aborts, ms + st.kernel_ms
                else:
                    r = sched.run(bank, ds)
                    commits += r.commits
                    aborts += r.aborts
                    ms += r.kernel_ms + r.plan_ms + r.train_ms
            vals = bank.values()
            if sched is not None:
                sched.close()
        assert commits == chunk * n_chunks
        assert int(vals.astype(np.int64).sum()) == 1000 * n_acc
        res[arm] = (aborts / (aborts + commits), commits / ms / 1e3)
    print("abort rate / Mtx/s:", res)
    assert res["learned"][0] <= 0.7 * res["plain"][0], res


@pytest.mark.parametrize("lane", [1, 2])
def test_serial_lane_plan_replays_exactly(lane):
    """With serial_lane set, transfers scored above defer_threshold run on the serial lane (1) or
    the dataflow lane (2) after the concurrent part; probe, concurrent and deferred runs replay
    exactly together."""
    torch = pytest.importorskip("torch")
    n_acc, n = 1 << 14, 1 << 15
    w = c1_workload(n_txn=n, n_accounts=n_acc, dist=cg.DIST_ZIPF, zipf_theta=0.99, seed=9,
                    up_reads=4, pr_read_pct=20)
    s = cg.generate(w)
    ds, keep = to_device(torch, s)
    with cg.Bank(n_accounts=n_acc, max_txn=n, ctas=16, client_warps=4) as bank, \
            cg.Scheduler(n_accounts=n_acc, max_txn=n, threshold=0.0, defer_threshold=0.0,
                         serial_lane=lane, train_steps=2, plan=0) as sched:
        bank.load()
        r1 = sched.probe(bank, ds)
        f1, np_ = r1.probe.final_ts, r1.n_probe
        log1, out1, res1 = bank.log(np_, f1)
        r2 = sched.plan_run(bank, ds)
        perm, _, split = sched.plan(n)
        f2 = r2.planned.final_ts if r2.planned.commits else f1
        n2 = 32 * split
        log2, out2, res2 = bank.log(n2, f2 - f1) if n2 else (np.zeros(0, np.uint32),) * 3
        r3 = sched.serial_run(bank, ds)
        f3 = r3.serial.final_ts
        log3, out3, res3 = bank.log(len(perm) - n2, f3 - f2)
        slots = bank.versions()
    assert r3.n_serial == len(perm) - n2 > 0 and r3.serial.aborts == 0
    op_c = np.concatenate([s.op[:np_], s.op[perm]])
    off_c = np.concatenate([s.off[:np_], s.off[perm]])
    sh = lambda lg, k: np.where(lg != HOLE, lg + k, HOLE).astype(np.uint32)
    log_c = np.concatenate([log1, sh(log2, np_), sh(log3, np_ + n2)]).astype(np.uint32)
    err = orc.check(op_c, off_c, s.addr, n_acc, np.full(n_acc, 1000, np.int32), 4, f3, log_c,
                    np.concatenate([out1, out2[:n2], out3]).astype(np.uint32),
                    np.concatenate([res1, res2[:n2], res3]).astype(np.int32), slots)
    assert err is None, err


def _scheduled_chunk_checked(bank, sched, s, ds, n, n_acc, depth):
    """Probe and planned runs of one chunk, replayed together with their commit groups."""
    r1 = sched.probe(bank, ds)
    f1, np_ = r1.probe.final_ts, r1.n_probe
    log1, out1, res1 = bank.log(np_, f1)
    g1 = bank.groups(f1)
    r2 = sched.plan_run(bank, ds)
    f2 = r2.planned.final_ts
    perm, _, split = sched.plan(n)
    log2, out2, res2 = bank.log(n - np_, f2 - f1)
    g2 = bank.groups(f2 - f1)
    slots = bank.versions()
    assert split == 0 and sorted(perm.tolist()) == list(range(np_, n))
    kinds = (s.op[perm] & 3).reshape(-1, 32)
    assert ((kinds == 0) == (kinds[:, :1] == 0)).all()  # rounds stay uniform in kind
    op_c = np.concatenate([s.op[:np_], s.op[perm]])
    off_c = np.concatenate([s.off[:np_], s.off[perm]])
    log_c = np.concatenate([log1, np.where(log2 != HOLE, log2 + np_, HOLE)]).astype(np.uint32)
    err = orc.check(op_c, off_c, s.addr, n_acc, np.full(n_acc, 1000, np.int32), depth, f2, log_c,
                    np.concatenate([out1, out2]), np.concatenate([res1, res2]), slots,
                    groups=concat_groups([(g1, f1), (g2, f2 - f1)]))
    assert err is None, err
    assert r1.probe.commits + r2.planned.commits == n
    return r1, r2


@pytest.mark.parametrize("score,key_written", [(0, 0), (1, 0), (0, 1)])
def test_grouped_plan_replays_exactly(score, key_written):
    """Grouped plan (plan 1) in front of group commit on a small contended bank, with the network
    (score 0) or the raw sketch-count score (score 1) flagging transfers, and rounds keyed by the
    hottest accounts touched or (key_written) written."""
    torch = pytest.importorskip("torch")
    n_acc, n = 1 << 14, 1 << 15
    w = c1_workload(n_txn=n, n_accounts=n_acc, dist=cg.DIST_ZIPF, zipf_theta=0.99, seed=10,
                    up_reads=4, pr_read_pct=20)
    s = cg.generate(w)
    ds, keep = to_device(torch, s)
    with cg.Bank(n_accounts=n_acc, max_txn=n, ctas=16, client_warps=4, prevalidate=3) as bank, \
            cg.Scheduler(n_accounts=n_acc, max_txn=n, plan=1, score=score, threshold=0.05,
                         train_steps=2, key_written=key_written) as sched:
        bank.load()
        r1, r2 = _scheduled_chunk_checked(bank, sched, s, ds, n, n_acc, 4)
    assert r2.n_flagged > 0


def test_grouped_plan_at_the_bench_shape_replays_exactly():
    """The benchmark's configuration, checked end to end: one 2^20-transaction Zipf(0.99) batch
    on 2^20 accounts (read 4 / write 2, 20 % read-only scans of 32), 152 CTAs of two client warps,
    8 versions per account, group commit. The scheduler probes 2 % of the rounds in stream order,
    trains, and runs its grouped plan; the engine locks, timestamps and validates every
    transaction. Probe and planned runs replay exactly together (groups included), the plain
    engine's run of the same batch does too, and the lock waits it reports label conflicts."""
    torch = pytest.importorskip("torch")
    n_acc, n, depth = 1 << 20, 1 << 20, 8
    s = cg.generate(zipf_bank_workload(n))
    ds, keep = to_device(torch, s)
    cfg = dict(n_accounts=n_acc, max_txn=n, ctas=152, client_warps=2, version_depth=depth,
               prevalidate=3)
    with cg.Bank(**cfg) as bank, \
            cg.Scheduler(n_accounts=n_acc, max_txn=n, plan=1, probe_rounds_pct=2) as sched:
        bank.load()
        r1, r2 = _scheduled_chunk_checked(bank, sched, s, ds, n, n_acc, depth)
    assert r2.n_flagged > 0 and r2.planned.error == 0
    waits = np.zeros(n, np.uint32)
    with cg.Bank(**cfg) as bank:
        bank.load()
        st = bank.run(s, txn_waits=waits)
        log_txn, outcome, result = bank.log(n, st.final_ts)
        err = orc.check(s.op, s.off, s.addr, n_acc, np.full(n_acc, 1000, np.int32), depth,
                        st.final_ts, log_txn, outcome, result, bank.versions(),
                        groups=bank.groups(st.final_ts))
    assert err is None, err
    upd = (s.op & 3) != 0
    assert 0 < waits[upd].mean() < 1 and not waits[~upd].any()


@pytest.mark.parametrize("arm", ["network", "sketch_score", "no_backoff"])
def test_grouped_plan_ablation_on_shifting_hotspot(arm):
    """Ablation of the learned arm on the shifting hotspot (1 M accounts, a 1 % hot set drawing
    30 % of the accesses, moving every 2^20 transactions; four chunks of 2^18): the grouped plan
    on group commit with the network's score, with the raw sketch-count score instead, or with
    the network and no backoff. Each arm commits everything, conserves the balance, and keeps
    its abort rate at least 30 % below the reference's commit method on the same chunks in
    stream order (the rates of all arms are printed for the record)."""
    torch = pytest.importorskip("torch")
    n_acc, chunk, n_chunks = 1 << 20, 1 << 18, 4
    s, bounds = _hotspot_chunks(n_acc, chunk, n_chunks, 0.3)
    over = {"network": {}, "sketch_score": {"score": 1}, "no_backoff": {"backoff_ns": 0}}[arm]
    res = {}
    for name in ("plain", arm):
        commits = aborts = 0
        cfg = dict(prevalidate=1) if name == "plain" else dict(prevalidate=3)
        with cg.Bank(n_accounts=n_acc, max_txn=chunk, ctas=152, client_warps=2, version_depth=8,
                     log_commits=0, **cfg) as bank:
            bank.load()
            sched = None if name == "plain" else cg.Scheduler(
                n_accounts=n_acc, max_txn=chunk, plan=1, probe_every=1, **over)
            for lo, hi in bounds:
                c = cg.Stream(np.ascontiguousarray(s.op[lo:hi]), np.ascontiguousarray(s.off[lo:hi]),
                              s.addr)
                ds, keep = to_device(torch, c)
                if sched is None:
                    st = bank.run_device(ds)
                    commits, aborts = commits + st.commits, aborts + st.aborts
                else:
                    r = sched.run(bank, ds)
                    commits, aborts = commits + r.commits, aborts + r.aborts
            vals = bank.values()
            if sched is not None:
                sched.close()
        assert commits == chunk * n_chunks
        assert int(vals.astype(np.int64).sum()) == 1000 * n_acc
        res[name] = aborts / (aborts + commits)
    print("abort rates:", res)
    assert res[arm] <= 0.7 * res["plain"], res
