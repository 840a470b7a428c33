"""The oracle against the committed reference vectors (tests/golden/ref_vectors.json, generated
from the reference's own functions by tests/golden/make_golden.py). Runs without the reference."""
import ctypes as C
import json
from pathlib import Path

import numpy as np

import oracle as orc
from oracle import p

G = json.loads((Path(__file__).parent / "golden" / "ref_vectors.json").read_text())
L = orc.lib()


def test_rand_r_vectors():
    for case in G["rand_r"]:
        s = C.c_uint64(case["seed"])
        assert [int(L.orc_rand_r(C.byref(s))) for _ in case["values"]] == case["values"]


def test_writeback_vectors():
    for case in G["writeback"]:
        h, t = C.c_uint16(1), C.c_uint16(0)
        ver, val = np.zeros(10, np.uint32), np.zeros(10, np.int32)
        val[1] = 1000
        for ts, v in case["writes"]:
            L.orc_ref_writeback(C.byref(h), C.byref(t), p(ver), p(val), 10, C.c_uint32(ts), C.c_int32(v))
        assert (h.value, t.value) == (case["head"], case["tail"])
        assert ver.tolist() == case["version"] and val.tolist() == case["value"]


def test_read_vectors_reference_and_packed_layout():
    for case, wb in zip(G["read"], G["writeback"]):
        ver = np.array(case["version"], np.uint32)
        val = np.array(case["value"], np.int32)
        slots = np.full(10, np.uint64(0xFFFFFFFF) << np.uint64(32), np.uint64)
        slots[0] = np.uint64(1000)
        for ts, v in wb["writes"]:
            L.orc_packed_writeback(p(slots), 10, C.c_uint32(ts), C.c_int32(v))
        for snap, ab, v in case["reads"]:
            o = C.c_int32()
            assert L.orc_ref_read(case["head"], case["tail"], p(ver), p(val), 10, C.c_uint32(snap), C.byref(o)) == ab
            if not ab:
                assert o.value == v
            o2 = C.c_int32()
            assert L.orc_packed_read(p(slots), 10, C.c_uint32(snap), C.byref(o2)) == ab
            if not ab:
                assert o2.value == v


def _records(case):
    recs = (orc.Record * case["ring"])()
    for slot, (txn, n, w0, w1) in case["records"].items():
        r = recs[int(slot)]
        r.txn, r.n_writes = txn, n
        r.ws[0], r.ws[1] = w0, w1
    return recs


def test_validate_vectors():
    for key, fn in (("validate_plain", L.orc_ref_validate), ("validate_batched", L.orc_batched_validate)):
        for case in G[key]:
            recs = _records(case)
            for ts, oldhp, rs, want in case["cases"]:
                # the vectors keep the 60 newest records: only compare scans that stay inside them
                span = (case["hp"] - oldhp) % case["ring"]
                newest = recs[case["hp"]].txn
                if span > 58 and newest - ts > 58:
                    continue
                rsa = np.array(rs, np.uint32)
                assert fn(recs, case["ring"], case["hp"], case["tp"], oldhp, ts, p(rsa), len(rs)) == want


def test_prevalidate_vectors():
    for case in G["prevalidate"]:
        ra = np.zeros((32, 8), np.uint32)
        rn = np.zeros(32, np.uint32)
        wa = np.zeros((32, 2), np.uint32)
        wn = np.zeros(32, np.uint32)
        for l in range(32):
            ra[l, :len(case["rs"][l])] = case["rs"][l]
            rn[l] = len(case["rs"][l])
            wa[l, :len(case["ws"][l])] = case["ws"][l]
            wn[l] = len(case["ws"][l])
        got = L.orc_prevalidate(p(ra), p(rn), 8, p(wa), p(wn), 2, C.c_uint32(0xFFFFFFFF), None)
        assert got == case["commit"]
