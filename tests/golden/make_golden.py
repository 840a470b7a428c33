"""Generate tests/golden/ref_vectors.json from the reference's own functions compiled for the host
(oracle/_ref/libcsmv_ref.so, built by oracle/ref_build.sh from the reference tree).

Run from the repo root:  python tests/golden/make_golden.py
The vectors pin the oracle where the reference tree is absent (tests/test_golden.py).
"""
import ctypes as C
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "oracle"))
import oracle as orc  # noqa: E402
from oracle import p  # noqa: E402


def main():
    orc.build()
    R = orc.ref()
    if R is None:
        raise SystemExit("reference tree not present: cannot generate golden vectors")
    rng = np.random.default_rng(20261203)
    out = {"source": "reference functions compiled for the host by oracle/ref_build.sh",
           "rand_r": [], "read": [], "writeback": [], "validate_plain": [],
           "validate_batched": [], "prevalidate": []}
    for seed in (1, 7, 1000003):
        s = C.c_uint64(seed)
        out["rand_r"].append({"seed": seed, "values": [int(R.ref_rand_r(C.byref(s))) for _ in range(64)]})
    for _ in range(60):  # version lists and reads
        head, tail = C.c_uint16(1), C.c_uint16(0)
        ver, val = np.zeros(10, np.uint32), np.zeros(10, np.int32)
        val[1] = 1000
        ts, writes = 0, []
        for _ in range(int(rng.integers(0, 20))):
            ts += int(rng.integers(1, 4))
            v = int(rng.integers(-999, 999))
            writes.append([ts, v])
            R.ref_sh_writeback(C.byref(head), C.byref(tail), p(ver), p(val), C.c_uint32(ts), C.c_int32(v))
        out["writeback"].append({"writes": writes, "head": head.value, "tail": tail.value,
                                 "version": ver.tolist(), "value": val.tolist()})
        reads = []
        for snap in range(0, ts + 2):
            o = C.c_int32()
            ab = R.ref_sh_read(head.value, tail.value, p(ver), p(val), C.c_uint32(snap), 0, C.byref(o))
            reads.append([snap, int(ab), int(o.value) if not ab else 0])
        out["read"].append({"head": head.value, "tail": tail.value, "version": ver.tolist(),
                            "value": val.tolist(), "reads": reads})
    for key, ring, fn in (("validate_plain", R.ref_sh_ring_size(), R.ref_sh_validate),
                          ("validate_batched", R.ref_bt_ring_size(), R.ref_bt_validate)):
        for _ in range(40):
            n_commits = int(rng.integers(1, 2 * ring))
            recs = (orc.Record * ring)()
            for c in range(1, n_commits + 1):
                r = recs[c % ring]
                r.txn, r.n_writes = c, int(rng.integers(0, 3))
                r.ws[0], r.ws[1] = (int(x) for x in rng.integers(0, 30, 2))
            hp = n_commits % ring
            tp = (hp + 1) % ring if n_commits >= ring else 0
            cases = []
            for _ in range(10):
                ts = int(rng.integers(max(0, n_commits - ring - 3), n_commits + 1))
                oldhp = tp if rng.random() < 0.5 else int((hp - rng.integers(0, 40)) % ring)
                rs = rng.integers(0, 30, int(rng.integers(1, 5))).astype(np.uint32)
                cases.append([ts, oldhp, rs.tolist(), int(fn(recs, hp, tp, oldhp, ts, p(rs), len(rs)))])
            recs_used = {}  # only the records a scan can reach, as {slot: [txn, n, w0, w1]}
            for d in range(0, 60):
                i = (hp - d) % ring
                recs_used[i] = [recs[i].txn, recs[i].n_writes, recs[i].ws[0], recs[i].ws[1]]
            recs_used[tp] = [recs[tp].txn, recs[tp].n_writes, recs[tp].ws[0], recs[tp].ws[1]]
            out[key].append({"ring": ring, "hp": hp, "tp": tp, "records": recs_used, "cases": cases})
    for n_addr in (3, 8, 40):
        for _ in range(30):
            rs = [rng.integers(0, n_addr, int(rng.integers(1, 5))).tolist() for _ in range(32)]
            ws = [r[:int(rng.integers(0, 3))] for r in rs]
            ra = np.zeros((32, 8), np.uint32)
            rn = np.zeros(32, np.uint32)
            wa = np.zeros((32, 2), np.uint32)
            wn = np.zeros(32, np.uint32)
            for l in range(32):
                ra[l, :len(rs[l])] = rs[l]
                rn[l] = len(rs[l])
                wa[l, :len(ws[l])] = ws[l]
                wn[l] = len(ws[l])
            m = int(R.ref_bt_prevalidate(p(ra), p(rn), 8, p(wa), p(wn), 2))
            out["prevalidate"].append({"rs": rs, "ws": ws, "commit": m})
    path = Path(__file__).resolve().parent / "ref_vectors.json"
    path.write_text(json.dumps(out, separators=(",", ":")))
    print(f"wrote {path} ({path.stat().st_size} bytes)")


if __name__ == "__main__":
    main()
