"""CPU tests of the oracle: its restatements against brute force, its replay checker against
serial executions and planted mistakes, and its generator against the product's."""
import ctypes as C

import numpy as np
import pytest

import csmv_gb300 as cg
import oracle as orc
from oracle import p

L = orc.lib()


def packed_init(depth, init):
    s = np.full(depth, np.uint64(0xFFFFFFFF) << np.uint64(32), np.uint64)
    s[0] = np.uint64(np.uint32(init))
    return s


def ref_layout_init(maxv, init):
    ver = np.zeros(maxv, np.uint32)
    val = np.zeros(maxv, np.int32)
    val[1] = init
    return [1, 0, ver, val]  # head, tail (bank/csmv_sh/API.cu:310-315)


def ref_layout_write(st, maxv, ts, v):
    h, t = C.c_uint16(st[0]), C.c_uint16(st[1])
    L.orc_ref_writeback(C.byref(h), C.byref(t), p(st[2]), p(st[3]), maxv, C.c_uint32(ts), C.c_int32(v))
    st[0], st[1] = h.value, t.value


def ref_layout_read(st, maxv, snap):
    out = C.c_int32()
    ab = L.orc_ref_read(C.c_uint16(st[0]), C.c_uint16(st[1]), p(st[2]), p(st[3]), maxv,
                        C.c_uint32(snap), C.byref(out))
    return None if ab else out.value


def packed_read(slots, snap):
    out = C.c_int32()
    ab = L.orc_packed_read(p(slots), len(slots), C.c_uint32(snap), C.byref(out))
    return None if ab else out.value


@pytest.mark.parametrize("depth", [2, 4, 10])
def test_packed_layout_reads_like_reference_layout(depth):
    rng = np.random.default_rng(depth)
    for trial in range(200):
        st = ref_layout_init(depth, 1000)
        slots = packed_init(depth, 1000)
        ts = 0
        for _ in range(rng.integers(0, 3 * depth)):
            ts += int(rng.integers(1, 5))
            v = int(rng.integers(-10**6, 10**6))
            ref_layout_write(st, depth, ts, v)
            L.orc_packed_writeback(p(slots), depth, C.c_uint32(ts), C.c_int32(v))
        for snap in range(0, ts + 3):
            assert ref_layout_read(st, depth, snap) == packed_read(slots, snap), (trial, snap)


def test_packed_victim_prefers_empty_then_oldest():
    s = packed_init(4, 5)
    assert L.orc_packed_victim(p(s), 4) == 1
    for ts in (3, 7, 9):
        L.orc_packed_writeback(p(s), 4, C.c_uint32(ts), C.c_int32(ts))
    assert L.orc_packed_victim(p(s), 4) == 0  # ts 0 is the oldest
    L.orc_packed_writeback(p(s), 4, C.c_uint32(11), C.c_int32(11))
    assert sorted(int(x >> np.uint64(32)) for x in s) == [3, 7, 9, 11]


def brute_prevalidate(rs, ws, active):
    commit = 0
    for l in range(32):
        if not (active >> l) & 1:
            continue
        conflict = any((active >> i) & 1 and (commit >> i) & 1 and set(ws[i]) & set(rs[l])
                       for i in range(l))
        if not conflict:
            commit |= 1 << l
    return commit


def pack_sets(sets, stride):
    a = np.zeros((32, stride), np.uint32)
    n = np.zeros(32, np.uint32)
    for l, s in enumerate(sets):
        a[l, :len(s)] = s
        n[l] = len(s)
    return a, n


@pytest.mark.parametrize("n_addr", [4, 16, 64])
def test_prevalidate_is_lane_order_greedy(n_addr):
    rng = np.random.default_rng(n_addr)
    for _ in range(300):
        rs = [list(rng.integers(0, n_addr, rng.integers(1, 5))) for _ in range(32)]
        ws = [list(r[:2]) for r in rs]
        active = int(rng.integers(0, 1 << 32))
        ra, rn = pack_sets(rs, 8)
        wa, wn = pack_sets(ws, 2)
        got = L.orc_prevalidate(p(ra), p(rn), 8, p(wa), p(wn), 2, C.c_uint32(active), None)
        assert got == brute_prevalidate(rs, ws, active)


def test_batched_ts_offsets():
    out = np.zeros(32, np.uint32)
    L.orc_batched_ts(C.c_uint32(0b1011_0000_0000_0000_0000_0000_0000_0101), C.c_uint32(100), p(out))
    assert out[0] == 101 and out[2] == 102 and out[28] == 103 and out[29] == 104 and out[31] == 105
    assert out[1] == 0 and out[30] == 0


def history_records(rng, n, n_addr):
    recs = (orc.Record * n)()
    for i in range(n):
        recs[i].txn = i + 1
        recs[i].n_writes = 2
        recs[i].ws[0], recs[i].ws[1] = (int(x) for x in rng.integers(0, n_addr, 2))
    return recs


def test_window_validate_matches_brute_force():
    rng = np.random.default_rng(3)
    recs = history_records(rng, 400, 50)
    for _ in range(500):
        snap = int(rng.integers(0, 400))
        front = int(rng.integers(snap, 401))
        rs = rng.integers(0, 50, 3).astype(np.uint32)
        got = L.orc_window_validate(recs, C.c_uint32(snap), C.c_uint32(front), C.c_uint32(1 << 20),
                                    p(rs), 3, 1)
        hit = any(set(recs[t - 1].ws[:2]) & set(rs.tolist()) for t in range(snap + 1, front + 1))
        assert got == (2 if hit else 0)
        # RecordAge once the ring is shorter than the window
        got = L.orc_window_validate(recs, C.c_uint32(snap), C.c_uint32(front), C.c_uint32(8),
                                    p(rs), 3, 1)
        if snap + 8 <= front:
            assert got == 1


def small_workload(**kw):
    d = dict(seed=5, n_accounts=64, n_txn=32 * 40, pr_read_pct=20, ro_reads=8, up_reads=3,
             kind=1, amt_lo=1, amt_hi=10, dist=0, zipf_theta=0.99, hot_frac=0.05, hot_prob=0.9,
             shift_every=256)
    d.update(kw)
    return orc.Workload(**d)


@pytest.mark.parametrize("dist", [0, 1, 2])
def test_generator_matches_product(dist):
    w = small_workload(dist=dist, n_accounts=5000, n_txn=32 * 200)
    o = orc.generate(w)
    s = cg.generate(cg.BankWorkload(*[getattr(w, f) for f, _ in orc.Workload._fields_]))
    for a, b in zip(o, (s.op, s.off, s.addr)):
        np.testing.assert_array_equal(a, b)


def test_zipf_head_frequency():
    n, theta = 100000, 0.99
    w = small_workload(dist=1, n_accounts=n, n_txn=32 * 2000, pr_read_pct=100, ro_reads=32)
    _, _, addr = orc.generate(w)
    h = sum(k ** -theta for k in range(1, n + 1))
    f0 = np.mean(addr == 0)
    assert abs(f0 - 1 / h) < 0.1 / h, (f0, 1 / h)
    assert np.mean(addr == 1) < f0


def serial_log(op, off, addr, n_acc, init, depth):
    """A commit log of the serial execution in stream order (what an exact run may produce)."""
    vals = np.array(init, np.int32)
    slots = np.concatenate([packed_init(depth, v) for v in vals])
    log, outcome, result = [], np.zeros(len(op), np.uint32), np.zeros(len(op), np.int32)
    wa, wv, r = np.zeros(2, np.uint32), np.zeros(2, np.int32), C.c_int32()
    for t in range(len(op)):
        nr = (int(op[t]) >> 2) & 63
        a = addr[off[t]:off[t] + nr].copy()
        v = vals[a].astype(np.int32)
        nw = L.orc_bank_exec(C.c_uint32(int(op[t])), p(a), p(v), p(wa), p(wv), C.byref(r))
        if nw == 0:
            outcome[t] = len(log) | orc.SNAP_FLAG
            result[t] = r.value
            continue
        log.append(t)
        ts = len(log)
        outcome[t] = ts
        for k in range(nw):
            vals[wa[k]] = wv[k]
            L.orc_packed_writeback(p(slots[wa[k] * depth:]), depth, C.c_uint32(ts), C.c_int32(int(wv[k])))
    return np.array(log, np.uint32), outcome, result, slots


def test_check_accepts_serial_execution():
    w = small_workload()
    op, off, addr = orc.generate(w)
    init = np.full(64, 100, np.int32)
    log, outcome, result, slots = serial_log(op, off, addr, 64, init, 4)
    assert orc.check(op, off, addr, 64, init, 4, len(log), log, outcome, result, slots) is None


def test_check_rejects_planted_mistakes():
    w = small_workload()
    op, off, addr = orc.generate(w)
    init = np.full(64, 100, np.int32)
    log, outcome, result, slots = serial_log(op, off, addr, 64, init, 4)
    args = (op, off, addr, 64, init, 4, len(log))
    # a read-only result that no snapshot had
    ro = np.flatnonzero(((op & 3) == 0))[0]
    bad = result.copy()
    bad[ro] += 1
    assert "read-only" in orc.check(*args, log, outcome, bad, slots)
    # two adjacent commits swapped where the later one's amount depends on an account the
    # earlier wrote (its extra read): the swapped order computes different transfers, except when
    # the amounts happen to coincide mod amod, so most (not all) such swaps must be caught
    det = tot = 0
    for i in range(len(log) - 1):
        a, b = log[i], log[i + 1]
        if not set(addr[off[a]:off[a] + 2].tolist()) & set(addr[off[b] + 2:off[b] + 3].tolist()):
            continue
        sw = log.copy()
        sw[i], sw[i + 1] = sw[i + 1], sw[i]
        out2 = outcome.copy()
        out2[sw[i]], out2[sw[i + 1]] = i + 1, i + 2
        tot += 1
        det += orc.check(*args, sw, out2, result, slots) is not None
    assert tot >= 10 and det >= 0.8 * tot, (det, tot)
    # a commit missing from the log
    assert orc.check(op, off, addr, 64, init, 4, len(log) - 1, log[:-1], outcome, result, slots) is not None
    # a corrupted version slot
    s2 = slots.copy()
    s2[5] ^= np.uint64(1)
    assert "slot" in orc.check(*args, log, outcome, result, s2)
    # a transaction committed twice
    dup = log.copy()
    dup[1] = dup[0]
    assert orc.check(*args, dup, outcome, result, slots) is not None


@pytest.mark.parametrize("locks", [True, False])
@pytest.mark.parametrize("prevalidate", [1, 0, 2])
def test_one_warp_model_is_exact(prevalidate, locks):
    w = small_workload(n_txn=32 * 64, n_accounts=40)
    op, off, addr = orc.generate(w)
    init = np.full(40, 100, np.int32)
    slots, log, outcome, result, st = orc.sim_1warp(op, off, addr, 40, init, 4, prevalidate, locks)
    assert st.commits_update + st.commits_readonly + st.commits_nowrite == len(op)
    # a chain (prevalidate 2) installs one version per account: its round is a commit group
    g = round_groups(op, log[:st.final_ts]) if prevalidate == 2 else None
    assert orc.check(op, off, addr, 40, init, 4, st.final_ts, log, outcome, result, slots,
                     groups=g) is None
    if prevalidate == 2:  # the chain commits every transaction on its first attempt
        assert st.aborts_prevalid + st.aborts_read_write + st.aborts_write_write == 0
        assert st.rounds == len(op) // 32
    else:
        assert (st.aborts_prevalid if prevalidate else st.aborts_read_write) > 0


def round_groups(op, log):
    """Group-end bitmap of a one-warp group-commit log: each round's timestamps form a group."""
    n = len(log)
    ends = np.zeros(((n + 31) // 32) * 32, bool)
    rnd = np.asarray(log) // 32
    ends[:n] = np.append(rnd[1:] != rnd[:-1], True)
    return np.packbits(ends.reshape(-1, 32)[:, ::-1], axis=1).view(">u4").astype(np.uint32).ravel()


def test_group_commit_model_installs_one_version_per_account_and_group():
    """The one-warp model of group commit (prevalidate 3) replays exactly when the checker knows
    the commit groups; without them the replay installs every write and the version slots
    differ, so the group bitmap is what the comparison rests on."""
    w = small_workload(n_txn=32 * 64, n_accounts=40)
    op, off, addr = orc.generate(w)
    init = np.full(40, 100, np.int32)
    slots, log, outcome, result, st = orc.sim_1warp(op, off, addr, 40, init, 4, 3, True)
    assert st.commits_update + st.commits_readonly + st.commits_nowrite == len(op)
    assert st.rounds == len(op) // 32
    g = round_groups(op, log)
    assert orc.check(op, off, addr, 40, init, 4, st.final_ts, log, outcome, result, slots,
                     groups=g) is None
    assert "slot" in orc.check(op, off, addr, 40, init, 4, st.final_ts, log, outcome, result,
                               slots)


def test_check_rejects_a_snapshot_inside_a_commit_group():
    w = small_workload(n_txn=32 * 64, n_accounts=40)
    op, off, addr = orc.generate(w)
    init = np.full(40, 100, np.int32)
    slots, log, outcome, result, st = orc.sim_1warp(op, off, addr, 40, init, 4, 3, True)
    g = round_groups(op, log)
    ro = np.flatnonzero((op & 3) == 0)
    inner = [ts for ts in range(1, st.final_ts) if not (g[(ts - 1) >> 5] >> ((ts - 1) & 31)) & 1]
    out2 = outcome.copy()
    out2[ro[-1]] = inner[len(inner) // 2] | orc.SNAP_FLAG
    err = orc.check(op, off, addr, 40, init, 4, st.final_ts, log, out2, result, slots, groups=g)
    assert err is not None and "inside a commit group" in err


def test_cpu_baselines_agree_on_commutative_stream():
    # unconditional transfers with two reads commute: any serialisation ends in the same state
    w = small_workload(kind=2, up_reads=2, n_accounts=1000, n_txn=32 * 3000)
    op, off, addr = orc.generate(w)
    init = np.full(1000, 100, np.int32)
    v1, _ = orc.serial(op, off, addr, 1000, init)
    v2, _ = orc.locked(op, off, addr, 1000, init, 4)
    np.testing.assert_array_equal(v1, v2)
    assert v1.sum() == init.sum()
