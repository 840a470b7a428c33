"""Pin the oracle to the reference: each restatement against the reference's own function,
compiled for the host from the reference sources (oracle/ref_build.sh -> oracle/_ref/).
Skipped where the reference tree is absent; tests/test_golden.py replays the same comparisons
from committed vectors everywhere."""
import ctypes as C

import numpy as np
import pytest

import oracle as orc
from oracle import p

R = orc.ref()
L = orc.lib()
pytestmark = pytest.mark.skipif(R is None, reason="reference tree not present (oracle/_ref not built)")


def test_rand_r_lcg():
    for seed in (0, 1, 12345, 2**40 + 7):
        a, b = C.c_uint64(seed), C.c_uint64(seed)
        for _ in range(2000):
            assert L.orc_rand_r(C.byref(a)) == R.ref_rand_r(C.byref(b))
            assert a.value == b.value


def random_item(rng, maxv=10):
    """A reachable reference version list: the initial state plus k rotations."""
    head, tail = C.c_uint16(1), C.c_uint16(0)
    ver = np.zeros(maxv, np.uint32)
    val = np.zeros(maxv, np.int32)
    val[1] = 1000
    ts = 0
    for _ in range(int(rng.integers(0, 25))):
        ts += int(rng.integers(1, 6))
        R.ref_sh_writeback(C.byref(head), C.byref(tail), p(ver), p(val), C.c_uint32(ts),
                           C.c_int32(int(rng.integers(-999, 999))))
    return head.value, tail.value, ver, val, ts


def test_read_rule_matches_reference():
    rng = np.random.default_rng(1)
    for _ in range(400):
        h, t, ver, val, last = random_item(rng)
        for snap in range(0, last + 2):
            for ro in (0, 1):
                o1, o2 = C.c_int32(), C.c_int32()
                a1 = R.ref_sh_read(h, t, p(ver), p(val), C.c_uint32(snap), ro, C.byref(o1))
                a2 = L.orc_ref_read(h, t, p(ver), p(val), 10, C.c_uint32(snap), C.byref(o2))
                assert a1 == a2
                if not a1:
                    assert o1.value == o2.value


def test_writeback_rotation_matches_reference():
    rng = np.random.default_rng(2)
    for _ in range(200):
        hr, tr = C.c_uint16(1), C.c_uint16(0)
        ho, to = C.c_uint16(1), C.c_uint16(0)
        vr, xr = np.zeros(10, np.uint32), np.zeros(10, np.int32)
        vo, xo = vr.copy(), xr.copy()
        ts = 0
        for _ in range(30):
            ts += 1
            v = int(rng.integers(-5000, 5000))
            R.ref_sh_writeback(C.byref(hr), C.byref(tr), p(vr), p(xr), C.c_uint32(ts), C.c_int32(v))
            L.orc_ref_writeback(C.byref(ho), C.byref(to), p(vo), p(xo), 10, C.c_uint32(ts), C.c_int32(v))
            assert (hr.value, tr.value) == (ho.value, to.value)
            np.testing.assert_array_equal(vr, vo)
            np.testing.assert_array_equal(xr, xo)


def make_ring(rng, ring, n_commits, n_addr):
    """Records as the reference's plain insert leaves them after n_commits commits."""
    recs = (orc.Record * ring)()
    for c in range(1, n_commits + 1):
        r = recs[c % ring]
        r.txn = c
        r.n_writes = int(rng.integers(0, 3))
        r.ws[0], r.ws[1] = (int(x) for x in rng.integers(0, n_addr, 2))
    return recs


@pytest.mark.parametrize("which", ["plain", "batched"])
def test_validate_matches_reference(which):
    rng = np.random.default_rng(4 if which == "plain" else 5)
    ring = R.ref_sh_ring_size() if which == "plain" else R.ref_bt_ring_size()
    ref_fn = R.ref_sh_validate if which == "plain" else R.ref_bt_validate
    orc_fn = L.orc_ref_validate if which == "plain" else L.orc_batched_validate
    for trial in range(300):
        n_commits = int(rng.integers(1, 3 * ring))
        recs = make_ring(rng, ring, n_commits, 40)
        hp = n_commits % ring
        if n_commits >= ring:
            tp = (hp + 1) % ring  # the oldest record once the ring has wrapped
        else:
            tp = 0
        ts = int(rng.integers(max(0, n_commits - ring - 5), n_commits + 1))
        oldhp = tp if rng.random() < 0.5 else int((hp - rng.integers(0, 50)) % ring)
        rs = rng.integers(0, 40, int(rng.integers(1, 6))).astype(np.uint32)
        a = ref_fn(recs, hp, tp, oldhp, ts, p(rs), len(rs))
        b = orc_fn(recs, ring, hp, tp, oldhp, ts, p(rs), len(rs))
        assert a == b, (trial, n_commits, hp, tp, oldhp, ts)


def test_plain_add_to_record_matches_reference():
    """One transaction at a time: the reference's TXAddToRecord takes ts = ring[hp].ts + 1 at
    slot hp+1 - the commit order the oracle's window rule and the GB300 engine use."""
    rng = np.random.default_rng(6)
    ring = R.ref_sh_ring_size()
    recs = (orc.Record * ring)()
    tp, rhp, whp = C.c_int(0), C.c_int(0), C.c_int(0)
    history = []
    for step in range(3000):
        rs = rng.integers(0, 30, 2).astype(np.uint32)
        ws = rs[:2].copy()
        snap = max(0, len(history) - int(rng.integers(0, 12)))
        ts = R.ref_sh_add_to_record(recs, C.byref(tp), C.byref(rhp), C.byref(whp), snap, p(rs), 2,
                                    p(ws), 2)
        by_ts = (orc.Record * max(1, len(history)))(*history) if history else (orc.Record * 1)()
        mine = L.orc_window_validate(by_ts, C.c_uint32(snap), C.c_uint32(len(history)),
                                     C.c_uint32(ring), p(rs), 2, 1)
        if ts:
            assert mine == 0, step
            assert ts == len(history) + 1
            r = orc.Record()
            r.txn, r.n_writes = ts, 2
            r.ws[0], r.ws[1] = int(ws[0]), int(ws[1])
            history.append(r)
        else:
            assert mine != 0, step


def pack(sets, stride):
    a = np.zeros((32, stride), np.uint32)
    n = np.zeros(32, np.uint32)
    for l, s in enumerate(sets):
        a[l, :len(s)] = s
        n[l] = len(s)
    return a, n


@pytest.mark.parametrize("n_addr", [3, 10, 100])
def test_prevalidation_matches_reference_warp(n_addr):
    rng = np.random.default_rng(n_addr)
    for _ in range(60):
        rs = [list(rng.integers(0, n_addr, rng.integers(1, 5))) for _ in range(32)]
        ws = [list(r[:rng.integers(0, 3)]) for r in rs]
        ra, rn = pack(rs, 8)
        wa, wn = pack(ws, 2)
        a = R.ref_bt_prevalidate(p(ra), p(rn), 8, p(wa), p(wn), 2)
        b = L.orc_prevalidate(p(ra), p(rn), 8, p(wa), p(wn), 2, C.c_uint32(0xFFFFFFFF), None)
        assert a == b
