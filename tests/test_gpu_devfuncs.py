"""GPU parity of the public device functions (include/csmv_tx.cuh) against the oracle and the
reference vectors: version read rule, TXPreValidation, TXWriteBack slot choice, bounded waits."""
import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

import oracle as orc
from csmv_gb300 import build as b
from oracle import p

pytestmark = pytest.mark.gpu
L = orc.lib()
G = json.loads((Path(__file__).parent / "golden" / "ref_vectors.json").read_text())


@pytest.fixture(scope="module")
def dt():
    d = C.CDLL(str(b.DEVTEST_LIB))
    for n in ("csmv_devtest_read", "csmv_devtest_prevalidate", "csmv_devtest_writeback",
              "csmv_devtest_bounded_wait"):
        getattr(d, n).restype = C.c_int
    d.csmv_devtest_read.argtypes = [C.c_void_p, C.c_int, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]
    d.csmv_devtest_prevalidate.argtypes = [C.c_void_p] * 5 + [C.c_uint32, C.c_void_p]
    d.csmv_devtest_writeback.argtypes = [C.c_void_p, C.c_int, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]
    d.csmv_devtest_bounded_wait.argtypes = [C.c_uint32, C.c_void_p, C.c_void_p]
    return d


def random_histories(rng, n, depth):
    """Per item: a write sequence with increasing ts, applied by the oracle's packed rule."""
    start = [0]
    ts_all, val_all = [], []
    slots = np.tile(np.full(depth, np.uint64(0xFFFFFFFF) << np.uint64(32), np.uint64), n)
    for i in range(n):
        slots[i * depth] = np.uint64(int(rng.integers(-1000, 1000)) & 0xFFFFFFFF)
        ts = 0
        for _ in range(int(rng.integers(0, 3 * depth))):
            ts += int(rng.integers(1, 4))
            ts_all.append(ts)
            val_all.append(int(rng.integers(-10**6, 10**6)))
        start.append(len(ts_all))
    return slots, np.array(start, np.uint32), np.array(ts_all + [0], np.uint32), np.array(val_all + [0], np.int32)


@pytest.mark.parametrize("depth", [2, 4, 8, 16])
def test_writeback_and_read_rule(dt, depth):
    rng = np.random.default_rng(depth)
    n = 5000
    slots, start, ts, val = random_histories(rng, n, depth)
    dev = slots.copy()
    assert dt.csmv_devtest_writeback(p(dev), depth, n, p(start), p(ts), p(val)) == 0
    host = slots.copy()
    for i in range(n):
        for k in range(start[i], start[i + 1]):
            L.orc_packed_writeback(p(host[i * depth:]), depth, C.c_uint32(int(ts[k])), C.c_int32(int(val[k])))
    np.testing.assert_array_equal(dev, host)
    for _ in range(4):
        snaps = rng.integers(0, 3 * depth * 3, n).astype(np.uint32)
        out = np.zeros(n, np.int32)
        ab = np.zeros(n, np.uint8)
        assert dt.csmv_devtest_read(p(dev), depth, n, p(snaps), p(out), p(ab)) == 0
        for i in range(n):
            o = C.c_int32()
            a = L.orc_packed_read(p(host[i * depth:]), depth, C.c_uint32(int(snaps[i])), C.byref(o))
            assert ab[i] == a and (a or out[i] == o.value), i


def test_read_rule_reference_vectors(dt):
    """The device read on the packed layout gives the reference's TXRead answers."""
    depth = 16  # holds the reference's 10 versions (and its ts-0 dummy) without eviction
    cases = G["writeback"]
    for case, rd in zip(cases, G["read"]):
        if len(case["writes"]) > 8:
            continue  # the reference evicted versions a 16-deep list still holds
        slots = np.full(depth, np.uint64(0xFFFFFFFF) << np.uint64(32), np.uint64)
        slots[0] = np.uint64(1000)
        for t, v in case["writes"]:
            L.orc_packed_writeback(p(slots), depth, C.c_uint32(t), C.c_int32(v))
        snaps = np.array([r[0] for r in rd["reads"]], np.uint32)
        k = len(snaps)
        dev = np.tile(slots, k)
        out = np.zeros(k, np.int32)
        ab = np.zeros(k, np.uint8)
        assert dt.csmv_devtest_read(p(dev), depth, k, p(snaps), p(out), p(ab)) == 0
        for j, (snap, want_ab, want) in enumerate(rd["reads"]):
            assert ab[j] == want_ab and (want_ab or out[j] == want)


def _pack(sets, stride):
    a = np.zeros((32, stride), np.uint32)
    n = np.zeros(32, np.uint32)
    for l, s in enumerate(sets):
        a[l, :len(s)] = s
        n[l] = len(s)
    return a, n


def test_prevalidation_matches_oracle_and_reference_vectors(dt):
    rng = np.random.default_rng(7)
    warps = []
    for case in G["prevalidate"]:
        warps.append((case["rs"], case["ws"], 0xFFFFFFFF, case["commit"]))
    for _ in range(2000):
        na = int(rng.choice([3, 10, 64, 1000]))
        rs = [rng.integers(0, na, int(rng.integers(1, 9))).tolist() for _ in range(32)]
        ws = [r[:int(rng.integers(0, 3))] for r in rs]
        warps.append((rs, ws, int(rng.integers(0, 1 << 32)), None))
    nw = len(warps)
    RS = np.zeros((nw, 32, 8), np.uint32)
    NR = np.zeros((nw, 32), np.uint32)
    WS = np.zeros((nw, 32, 2), np.uint32)
    NW = np.zeros((nw, 32), np.uint32)
    ACT = np.zeros(nw, np.uint32)
    for i, (rs, ws, act, _) in enumerate(warps):
        RS[i], NR[i] = _pack(rs, 8)
        WS[i], NW[i] = _pack(ws, 2)
        ACT[i] = act
    out = np.zeros(nw, np.uint32)
    assert dt.csmv_devtest_prevalidate(p(RS), p(NR), p(WS), p(NW), p(ACT), nw, p(out)) == 0
    for i, (_, _, act, want) in enumerate(warps):
        o = L.orc_prevalidate(p(RS[i]), p(NR[i]), 8, p(WS[i]), p(NW[i]), 2, C.c_uint32(act), None)
        assert out[i] == o, i
        if want is not None:
            assert out[i] == want, i


def test_bounded_wait_returns_error_instead_of_hanging(dt):
    err, done = C.c_uint32(), C.c_uint32()
    assert dt.csmv_devtest_bounded_wait(12, C.byref(err), C.byref(done)) == 0
    assert err.value == 1 and done.value == 2
