"""GPU parity tests of the bank commit path, through the C ABI, against the CPU oracle.

Exactness bar (integer path, bit-exact): every run's commit log replayed serially in commit-ts
order reproduces the device's final version slots bit for bit, every read-only and no-write
transaction saw the state at its snapshot, commit timestamps are unique and dense, the total
balance is conserved. With one client warp the run is deterministic and must equal the oracle's
model of the engine exactly (log, outcomes, versions, abort counts)."""
import subprocess

import numpy as np
import pytest

import csmv_gb300 as cg
import oracle as orc
from gpu_util import c1_workload, defer_plan, run_checked, sub_stream, to_device

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prevalidate", [1, 0, 2, 3])
@pytest.mark.parametrize("validate", [cg.VALIDATE_STAMP, cg.VALIDATE_RING, cg.VALIDATE_RING_LANE])
def test_one_client_warp_equals_oracle_model(prevalidate, validate):
    if prevalidate >= 2 and validate != cg.VALIDATE_STAMP:
        pytest.skip("intra-warp chaining and group commit are stamp-protocol modes")
    w = c1_workload(n_txn=32 * 96, n_accounts=40, pr_read_pct=20, up_reads=3, seed=11)
    st, s, (log_txn, outcome, result, slots) = run_checked(
        w, ctas=1, client_warps=1, prevalidate=prevalidate, validate=validate, batch=cg.BATCH_WARP,
        init_value=100)
    init = np.full(40, 100, np.int32)
    mslots, mlog, mout, mres, ms = orc.sim_1warp(s.op, s.off, s.addr, 40, init, 4, prevalidate,
                                                 locks=validate == cg.VALIDATE_STAMP)
    np.testing.assert_array_equal(log_txn, mlog)
    np.testing.assert_array_equal(outcome, mout)
    np.testing.assert_array_equal(result, mres)
    np.testing.assert_array_equal(slots, mslots)
    assert (st.commits_update, st.commits_readonly, st.commits_nowrite) == (
        ms.commits_update, ms.commits_readonly, ms.commits_nowrite)
    assert (st.aborts_prevalid, st.aborts_read_write, st.aborts_write_write, st.rounds) == (
        ms.aborts_prevalid, ms.aborts_read_write, ms.aborts_write_write, ms.rounds)
    assert st.aborts_data_age == 0 and st.aborts_record_age == 0


VARIANTS = {
    "stamp-cta-client": dict(validate=cg.VALIDATE_STAMP, batch=cg.BATCH_CTA),
    "stamp-warp-client": dict(validate=cg.VALIDATE_STAMP, batch=cg.BATCH_WARP),
    "stamp-cta-server": dict(validate=cg.VALIDATE_STAMP, batch=cg.BATCH_CTA, writeback=cg.WRITEBACK_SERVER),
    "stamp-lane-server": dict(validate=cg.VALIDATE_STAMP, batch=cg.BATCH_LANE, writeback=cg.WRITEBACK_SERVER),
    "ring-cta-client": dict(validate=cg.VALIDATE_RING, batch=cg.BATCH_CTA),
    "ring-warp-server": dict(validate=cg.VALIDATE_RING, batch=cg.BATCH_WARP, writeback=cg.WRITEBACK_SERVER),
    "ringlane-warp-client": dict(validate=cg.VALIDATE_RING_LANE, batch=cg.BATCH_WARP),
    "stamp-cta-noprevalid": dict(validate=cg.VALIDATE_STAMP, batch=cg.BATCH_CTA, prevalidate=0),
    "stamp-cta-chain": dict(validate=cg.VALIDATE_STAMP, batch=cg.BATCH_CTA, prevalidate=2),
    "stamp-cluster2": dict(validate=cg.VALIDATE_STAMP, batch=cg.BATCH_CLUSTER, cluster_size=2),
    "stamp-cta-group": dict(validate=cg.VALIDATE_STAMP, batch=cg.BATCH_CTA, prevalidate=3),
    "stamp-cta-group-r4": dict(validate=cg.VALIDATE_STAMP, batch=cg.BATCH_CTA, prevalidate=3,
                               max_reads=4),
    "stamp-cta-r4": dict(validate=cg.VALIDATE_STAMP, batch=cg.BATCH_CTA, max_reads=4),
    "stamp-warp-group": dict(validate=cg.VALIDATE_STAMP, batch=cg.BATCH_WARP, prevalidate=3),
    "stamp-cluster2-group": dict(validate=cg.VALIDATE_STAMP, batch=cg.BATCH_CLUSTER,
                                 cluster_size=2, prevalidate=3),
    "stamp-cluster8": dict(validate=cg.VALIDATE_STAMP, batch=cg.BATCH_CLUSTER, cluster_size=8),
}


@pytest.mark.parametrize("variant", list(VARIANTS))
def test_c1_plain_bank_exact(variant):
    """4096 accounts, 8 blocks x 128 client threads, 256 transactions each, depth 4."""
    st, _, _ = run_checked(c1_workload(), ctas=8, client_warps=4, **VARIANTS[variant])
    assert st.commits_readonly > 0 and st.commits_update > 0


@pytest.mark.parametrize("validate,prevalidate", [(cg.VALIDATE_STAMP, 1), (cg.VALIDATE_STAMP, 2),
                                                  (cg.VALIDATE_STAMP, 3), (cg.VALIDATE_RING, 1)])
@pytest.mark.parametrize("depth", [2, 4, 16])
def test_high_contention_exact(depth, validate, prevalidate):
    """16 accounts, 32 client warps: most attempts conflict; the ring form runs with a 64-record
    ring (RecordAge), depth 2 keeps only two versions (DataAge on read-only scans)."""
    w = c1_workload(n_txn=32 * 600, n_accounts=16, pr_read_pct=30, ro_reads=8, up_reads=3, seed=3)
    st, _, _ = run_checked(w, ctas=4, client_warps=8, version_depth=depth, ring_size=64,
                           validate=validate, prevalidate=prevalidate)
    if prevalidate != 3:  # group commit waits for write locks instead of aborting on them
        assert st.aborts > 0


def test_transfer_wider_than_max_reads_is_refused():
    """A transfer reading more accounts than the kernel holds (max_reads = 4) fails the run as
    malformed instead of being cut short."""
    w = c1_workload(n_txn=32 * 64, n_accounts=512, up_reads=6, seed=6)
    with pytest.raises(cg.CsmvError) as e:
        run_checked(w, ctas=4, client_warps=2, prevalidate=3, max_reads=4)
    assert e.value.status == 1


def test_two_accounts_extreme():
    w = c1_workload(n_txn=32 * 40, n_accounts=2, pr_read_pct=0, up_reads=2, seed=5)
    run_checked(w, ctas=2, client_warps=2, init_value=50)


def test_single_round():
    run_checked(c1_workload(n_txn=32, n_accounts=100), ctas=1, client_warps=1)


@pytest.mark.parametrize("prevalidate,max_reads", [(3, 8), (3, 4), (2, 8), (1, 8)])
def test_zipf_contended_exact(prevalidate, max_reads):
    """1M accounts, Zipf 0.99, read 4 / write 2, 20% read-only scans of 32, one CTA per SM."""
    w = cg.bank_workload(1 << 20, 1 << 16, seed=9, pr_read_pct=20, ro_reads=32, up_reads=4,
                         kind=cg.KIND_TRANSFER, amt_lo=1, amt_hi=10, dist=cg.DIST_ZIPF,
                         zipf_theta=0.99)
    st, _, _ = run_checked(w, ctas=152, client_warps=2, version_depth=8, prevalidate=prevalidate,
                           max_reads=max_reads)
    if prevalidate != 3:  # group commit waits for write locks instead of aborting on them
        assert st.aborts > 0


@pytest.mark.parametrize("prevalidate", [2, 3])
def test_hotspot_full_gpu_exact(prevalidate):
    w = cg.bank_workload(1 << 20, 1 << 18, seed=4, pr_read_pct=10, ro_reads=8, up_reads=4,
                         dist=cg.DIST_HOTSPOT, hot_frac=0.01, hot_prob=0.9, shift_every=1 << 16)
    run_checked(w, ctas=0, client_warps=15, prevalidate=prevalidate)


def test_runs_continue_the_commit_order():
    w = c1_workload(n_txn=32 * 256)
    s = cg.generate(w)
    with cg.Bank(n_accounts=4096, max_txn=w.n_txn, ctas=8, client_warps=4) as bank:
        bank.load()
        st1 = bank.run(s)
        v1 = bank.values()
        st2 = bank.run(s)
        log2, out2, res2 = bank.log(w.n_txn, st2.final_ts - st1.final_ts)
        v2 = bank.values()
    assert v1.sum() == v2.sum() == 4096 * 1000
    assert st2.final_ts > st1.final_ts
    # replay run 2 from the state after run 1, timestamps shifted to start at 1
    f1 = np.uint32(st1.final_ts)
    out = out2.copy()
    snap = (out & np.uint32(cg.SNAP_FLAG)) != 0
    out[~snap] -= f1
    out[snap] = ((out[snap] & np.uint32(0x7FFFFFFF)) - f1) | np.uint32(cg.SNAP_FLAG)
    err = orc.check(s.op, s.off, s.addr, 4096, v1, 4, st2.final_ts - st1.final_ts, log2, out, res2)
    assert err is None, err
    assert np.array_equal(v2, _replay_values(s, v1, log2))


def _replay_values(s, init, log):
    import ctypes as C

    vals = init.copy()
    L = orc.lib()
    wa, wv, r = np.zeros(2, np.uint32), np.zeros(2, np.int32), C.c_int32()
    for t in log:
        if t == 0xFFFFFFFF:  # timestamp of a transaction that failed validation
            continue
        nr = (int(s.op[t]) >> 2) & 63
        a = s.addr[s.off[t]:s.off[t] + nr].copy()
        v = vals[a].astype(np.int32)
        nw = L.orc_bank_exec(C.c_uint32(int(s.op[t])), orc.p(a), orc.p(v), orc.p(wa), orc.p(wv), C.byref(r))
        for k in range(nw):
            vals[wa[k]] = wv[k]
    return vals


def test_run_device_matches_run():
    torch = pytest.importorskip("torch")
    w = c1_workload(n_txn=32 * 512)
    s = cg.generate(w)
    dop = torch.from_numpy(s.op.view(np.int32)).cuda()
    doff = torch.from_numpy(s.off.view(np.int32)).cuda()
    daddr = torch.from_numpy(s.addr.view(np.int32)).cuda()
    ds = cg.BankStream(w.n_txn, dop.data_ptr(), doff.data_ptr(), daddr.data_ptr(), s.addr.shape[0])
    with cg.Bank(n_accounts=4096, max_txn=w.n_txn, ctas=8, client_warps=4) as bank:
        bank.load()
        st = bank.run_device(ds)
        torch.cuda.synchronize()
        log_txn, outcome, result = bank.log(w.n_txn, st.final_ts)
        slots = bank.versions()
    assert st.commits == w.n_txn
    err = orc.check(s.op, s.off, s.addr, 4096, np.full(4096, 1000, np.int32), 4, st.final_ts,
                    log_txn, outcome, result, slots)
    assert err is None, err


def test_driver_reference_command_line():
    from csmv_gb300 import build as b

    out = subprocess.run([str(b.BIN / "csmv_bank"), "4096", "128", "8", "128", "10", "8", "1", "0"],
                         capture_output=True, text=True, timeout=300,
                         env={"CSMV_TX_PER_THREAD": "64", "PATH": "/usr/bin:/bin"})
    assert out.returncode == 0, out.stderr
    assert "Consistency fail" not in out.stdout
    fields = out.stdout.strip().split("\t")
    assert len(fields) == 6 + 17 + 4
    assert float(fields[1]) > 0 and 0.0 <= float(fields[0]) < 100.0


def test_driver_trace_files_replay_exactly(tmp_path):
    """CSMV_TRACE_OUT writes the driver's stream and commit log; the files replay exactly in
    the oracle, and CSMV_TRACE_IN runs the same stream again from its file."""
    from csmv_gb300 import build as b

    prefix = tmp_path / "run"
    env = {"CSMV_TX_PER_THREAD": "32", "PATH": "/usr/bin:/bin", "CSMV_TRACE_OUT": str(prefix)}
    args = [str(b.BIN / "csmv_bank"), "2048", "128", "4", "128", "10", "8", "2", "0"]
    out = subprocess.run(args, capture_output=True, text=True, timeout=300, env=env)
    assert out.returncode == 0, out.stderr
    s = cg.load_stream(f"{prefix}.stream")
    base, log_txn, outcome, result = cg.load_log(f"{prefix}.log")
    assert base == 0 and s.n_txn == 128 * 4 * 32 and outcome.shape[0] == s.n_txn
    err = orc.check(s.op, s.off, s.addr, 2048, np.full(2048, 100, np.int32), 4, log_txn.shape[0],
                    log_txn, outcome, result)
    assert err is None, err
    env2 = {"PATH": "/usr/bin:/bin", "CSMV_TRACE_IN": f"{prefix}.stream"}
    out2 = subprocess.run(args, capture_output=True, text=True, timeout=300, env=env2)
    assert out2.returncode == 0, out2.stderr
    assert "Consistency fail" not in out2.stdout


def test_bank_run_from_a_stream_file_and_log_file(tmp_path):
    """A stream saved and loaded back runs on the GPU; its commit log, saved and loaded back,
    replays exactly."""
    w = c1_workload(n_txn=32 * 512, n_accounts=1024, dist=cg.DIST_ZIPF, up_reads=4, seed=31)
    cg.save_stream(tmp_path / "s.stream", cg.generate(w))
    s = cg.load_stream(tmp_path / "s.stream")
    with cg.Bank(n_accounts=1024, max_txn=s.n_txn) as bank:
        bank.load()
        st = bank.run(s)
        lt, oc, rs = bank.log(s.n_txn, st.final_ts)
        slots = bank.versions()
    cg.save_log(tmp_path / "s.log", 0, lt, oc, rs)
    base, lt2, oc2, rs2 = cg.load_log(tmp_path / "s.log")
    err = orc.check(s.op, s.off, s.addr, 1024, np.full(1024, 1000, np.int32), 4, st.final_ts,
                    lt2, oc2, rs2, slots)
    assert err is None, err


@pytest.mark.parametrize("deferred_warps", [1, 7, 64])
def test_deferred_queue_and_per_transaction_aborts_exact(deferred_warps):
    """A stream whose hot-account transfers sit in a deferred queue served by a few warps runs
    exactly (serial replay), and the per-transaction failed-attempt counts add up to the
    aborts the statistics report."""
    w = c1_workload(n_txn=32 * 1024, n_accounts=8192, dist=cg.DIST_HOTSPOT, hot_frac=0.01,
                    hot_prob=0.5, seed=4)
    s = cg.generate(w)
    hot = np.zeros(w.n_accounts, bool)
    cnt = np.bincount(s.addr, minlength=w.n_accounts)
    hot[cnt > 8 * cnt.mean()] = True
    risky = hot[s.addr[s.off]] | hot[s.addr[s.off + 1]]
    ps, split = defer_plan(s, risky)
    assert 0 < split < w.n_txn // 32
    ab = np.zeros(w.n_txn, np.uint32)
    st, _, _ = run_checked(w, stream=ps, txn_aborts=ab, split_round=split,
                           deferred_warps=deferred_warps, ctas=16, client_warps=4)
    assert int(ab.sum()) == st.aborts
    ab0 = np.zeros(w.n_txn, np.uint32)
    st0, _, _ = run_checked(w, txn_aborts=ab0, ctas=16, client_warps=4)
    assert int(ab0.sum()) == st0.aborts and st0.aborts > 0


@pytest.mark.parametrize("prevalidate", [1, 3])
def test_deferred_queue_lanes_exact(prevalidate):
    """The deferred queue cut into lanes (lane_start): each of the first warps serves its own
    lane of rounds in order - here one lane per hot account of a Zipf bank, as a scheduler's
    hot lanes are, plus an empty lane - and the run replays exactly."""
    w = c1_workload(n_txn=32 * 2048, n_accounts=1 << 14, dist=cg.DIST_ZIPF, zipf_theta=0.99,
                    up_reads=4, pr_read_pct=20, seed=5)
    s = cg.generate(w)
    R = w.n_txn // 32
    ro = (s.op.reshape(R, 32)[:, 0] & 3) == 0
    first = s.addr[s.off].reshape(R, 32)[:, 0]  # a round's lane: its first transfer's debit
    lanes = [np.flatnonzero(~ro & (first == a)) for a in (0, 1, 2)]
    laned = np.concatenate(lanes)
    rest = np.setdiff1d(np.arange(R), laned)
    order = np.concatenate([rest] + lanes + [np.zeros(0, np.int64)])
    perm = (order[:, None] * 32 + np.arange(32)).ravel()
    ps = cg.Stream(np.ascontiguousarray(s.op[perm]), np.ascontiguousarray(s.off[perm]), s.addr)
    split = len(rest)
    bounds = np.cumsum([split] + [len(x) for x in lanes] + [0]).astype(np.uint32)
    assert 0 < split < R and len(laned) > 0
    run_checked(w, stream=ps, split_round=split, deferred_warps=4, lane_start=bounds, ctas=16,
                client_warps=4, version_depth=8, prevalidate=prevalidate)


@pytest.mark.parametrize("dist", [cg.DIST_UNIFORM, cg.DIST_ZIPF])
def test_serial_lane_equals_stream_order_execution(dist):
    """The serial lane commits every transaction in stream order: its final balances, read-only
    sums and commit log equal a serial execution of the stream, and the replay check holds."""
    torch = pytest.importorskip("torch")
    n_acc, n = 2048, 32 * 600
    w = c1_workload(n_txn=n, n_accounts=n_acc, dist=dist, zipf_theta=0.99, up_reads=4,
                    pr_read_pct=20, seed=12)
    s = cg.generate(w)
    ds, keep = to_device(torch, s)
    with cg.Bank(n_accounts=n_acc, max_txn=n, version_depth=4) as bank:
        bank.load()
        st = bank.run_serial_device(ds)
        log_txn, outcome, result = bank.log(n, st.final_ts)
        slots = bank.versions()
        vals = bank.values()
    init = np.full(n_acc, 1000, np.int32)
    assert st.commits == n and st.aborts == 0
    err = orc.check(s.op, s.off, s.addr, n_acc, init, 4, st.final_ts, log_txn, outcome, result,
                    slots)
    assert err is None, err
    ref, _ = orc.serial(s.op, s.off, s.addr, n_acc, init)
    np.testing.assert_array_equal(vals, ref)
    writers = np.flatnonzero((outcome & cg.SNAP_FLAG) == 0)
    assert (np.diff(writers) > 0).all() and (log_txn == writers).all()  # stream order


FLOW_CASES = {
    "zipf-depth4": dict(n_acc=2048, n=32 * 600, dist=cg.DIST_ZIPF, depth=4, up_reads=4, ro=20),
    "uniform-depth8": dict(n_acc=1 << 16, n=1 << 15, dist=cg.DIST_UNIFORM, depth=8, up_reads=4,
                           ro=20),
    "hot16-depth2": dict(n_acc=16, n=32 * 200, dist=cg.DIST_UNIFORM, depth=2, up_reads=3, ro=30),
    "zipf-depth16-transfers": dict(n_acc=1 << 14, n=1 << 14, dist=cg.DIST_ZIPF, depth=16,
                                   up_reads=4, ro=0),
    "two-accounts-always": dict(n_acc=2, n=32 * 40, dist=cg.DIST_UNIFORM, depth=4, up_reads=2,
                                ro=0, kind=cg.KIND_TRANSFER_ALWAYS),
    "zipf-self-transfers": dict(n_acc=512, n=32 * 300, dist=cg.DIST_ZIPF, depth=4, up_reads=3,
                                ro=10, self_every=5),
    "zipf-1-warp": dict(n_acc=1024, n=32 * 400, dist=cg.DIST_ZIPF, depth=4, up_reads=4, ro=20,
                        flow_warps=1),
    "zipf-16-warps": dict(n_acc=1 << 15, n=1 << 16, dist=cg.DIST_ZIPF, depth=8, up_reads=4,
                          ro=20, flow_warps=16),
    "zipf-eight-reads": dict(n_acc=4096, n=32 * 300, dist=cg.DIST_ZIPF, depth=4, up_reads=8,
                             ro=10),
}


@pytest.mark.parametrize("case", list(FLOW_CASES))
def test_flow_lane_equals_serial_lane(case):
    """The dataflow lane leaves exactly what the serial lane leaves - versions in the same slots,
    commit log, outcomes, results, statistics - and its run replays exactly."""
    torch = pytest.importorskip("torch")
    c = FLOW_CASES[case]
    n_acc, n, depth = c["n_acc"], c["n"], c["depth"]
    w = c1_workload(n_txn=n, n_accounts=n_acc, dist=c["dist"], zipf_theta=0.99,
                    up_reads=c["up_reads"], pr_read_pct=c["ro"], seed=21,
                    kind=c.get("kind", cg.KIND_TRANSFER))
    s = cg.generate(w)
    if "self_every" in c:  # some transfers name one account twice: it is written once
        t = np.flatnonzero((s.op & 3) != 0)[:: c["self_every"]]
        s.addr[s.off[t] + 1] = s.addr[s.off[t]]
    ds, keep = to_device(torch, s)
    res = []
    for lane in ("serial", "flow"):
        with cg.Bank(n_accounts=n_acc, max_txn=n, version_depth=depth,
                     flow_warps=c.get("flow_warps", 0)) as bank:
            bank.load()
            st = bank.run_serial_device(ds) if lane == "serial" else bank.run_flow_device(ds)
            res.append((st, bank.log(n, st.final_ts), bank.versions(), bank.values()))
    (s1, l1, v1, b1), (s2, l2, v2, b2) = res
    assert s2.error == 0 and s2.commits == n and s2.aborts == 0
    for f in ("commits_update", "commits_readonly", "commits_nowrite", "final_ts", "rounds",
              "sections"):
        assert getattr(s1, f) == getattr(s2, f), f
    for a, b in zip(l1, l2):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(v1, v2)
    np.testing.assert_array_equal(b1, b2)
    init = np.full(n_acc, 1000, np.int32)
    ref, _ = orc.serial(s.op, s.off, s.addr, n_acc, init)
    np.testing.assert_array_equal(b2, ref)
    if "self_every" not in c:  # a self-transfer keeps only its credit: the total is not invariant
        err = orc.check(s.op, s.off, s.addr, n_acc, init, depth, s2.final_ts, *l2, v2)
        assert err is None, err


def test_flow_lane_interleaves_with_engine_and_serial_lane():
    """Concurrent run, dataflow run, serial-lane run, dataflow run on one bank: the commit order
    carries across them and the concatenated log replays exactly."""
    torch = pytest.importorskip("torch")
    n_acc, n = 4096, 32 * 512
    w = c1_workload(n_txn=4 * n, n_accounts=n_acc, seed=17, dist=cg.DIST_ZIPF, zipf_theta=0.9,
                    up_reads=4)
    s = cg.generate(w)
    parts = [sub_stream(s, i * n, (i + 1) * n) for i in range(4)]
    logs, outs, ress = [], [], []
    with cg.Bank(n_accounts=n_acc, max_txn=n, ctas=8, client_warps=4) as bank:
        bank.load()
        prev = 0
        for i, part in enumerate(parts):
            ds, keep = to_device(torch, part)
            run = [bank.run_device, bank.run_flow_device, bank.run_serial_device,
                   bank.run_flow_device][i]
            st = run(ds)
            lt, oc, rs = bank.log(n, st.final_ts - prev)
            logs.append(np.where(lt != 0xFFFFFFFF, lt + i * n, lt).astype(np.uint32))
            outs.append(oc)
            ress.append(rs)
            prev = st.final_ts
        slots = bank.versions()
    err = orc.check(s.op, s.off, s.addr, n_acc, np.full(n_acc, 1000, np.int32), 4, prev,
                    np.concatenate(logs), np.concatenate(outs), np.concatenate(ress), slots)
    assert err is None, err


def test_flow_lane_rejects_a_bad_account_and_applies_nothing():
    """An account id past the bank fails the call (CSMV_ERR_INVALID_ARG); the checks run before
    any access, so the bank is left as it was and the next run is exact."""
    torch = pytest.importorskip("torch")
    n_acc, n = 1024, 32 * 64
    w = c1_workload(n_txn=2 * n, n_accounts=n_acc, seed=23, pr_read_pct=0)
    s = cg.generate(w)
    bad = cg.Stream(s.op[:n].copy(), s.off[:n].copy(), s.addr.copy())
    bad.addr[bad.off[n // 2] + 1] = n_acc + 5
    with cg.Bank(n_accounts=n_acc, max_txn=n) as bank:
        bank.load()
        before = bank.versions()
        dbad, keep = to_device(torch, bad)
        with pytest.raises(cg.CsmvError):
            bank.run_flow_device(dbad)
        np.testing.assert_array_equal(bank.versions(), before)
        ds, keep2 = to_device(torch, sub_stream(s, n, 2 * n))
        st = bank.run_flow_device(ds)
        log_txn, outcome, result = bank.log(n, st.final_ts)
        slots = bank.versions()
    tail = sub_stream(s, n, 2 * n)
    err = orc.check(tail.op, tail.off, tail.addr, n_acc, np.full(n_acc, 1000, np.int32), 4,
                    st.final_ts, log_txn, outcome, result, slots)
    assert err is None, err


def test_engine_and_serial_lane_runs_interleave_exactly():
    """Concurrent run, serial-lane run, concurrent run on one bank: the commit order carries
    across them and the concatenated log replays exactly."""
    torch = pytest.importorskip("torch")
    n_acc, n = 4096, 32 * 512
    w = c1_workload(n_txn=3 * n, n_accounts=n_acc, seed=13)
    s = cg.generate(w)
    parts = [sub_stream(s, i * n, (i + 1) * n) for i in range(3)]
    logs, outs, ress = [], [], []
    with cg.Bank(n_accounts=n_acc, max_txn=n, ctas=8, client_warps=4) as bank:
        bank.load()
        prev = 0
        for i, part in enumerate(parts):
            ds, keep = to_device(torch, part)
            st = bank.run_serial_device(ds) if i == 1 else bank.run_device(ds)
            lt, oc, rs = bank.log(n, st.final_ts - prev)
            logs.append(np.where(lt != 0xFFFFFFFF, lt + i * n, lt).astype(np.uint32))
            outs.append(oc)
            ress.append(rs)
            prev = st.final_ts
        slots = bank.versions()
    err = orc.check(s.op, s.off, s.addr, n_acc, np.full(n_acc, 1000, np.int32), 4, prev,
                    np.concatenate(logs), np.concatenate(outs), np.concatenate(ress), slots)
    assert err is None, err
