"""CPU model of the dataflow lane's method (csrc/flow_kernels.cuh), step by step with the same
index arithmetic: elements, the stable radix sort's per-tile / per-warp ranks, producers from
the max-scan of write positions, execution in dependency order, ranks, and installs that walk
back from each account's tail. It must equal a one-transaction-at-a-time execution in stream
order with victim-order installs (what the serial lane leaves), and pass the replay checker -
over several runs on one bank, as the engine and the lanes interleave."""
import numpy as np
import pytest

import csmv_gb300 as cg
import oracle as orc

EMPTY = 0xFFFFFFFF
WRITE = 64  # element codes >= 64 are writes (slot = code - 64)


def u32(x):
    return x & 0xFFFFFFFF


def i32(x):
    x = u32(x)
    return x - (1 << 32) if x >= 1 << 31 else x


def radix_sort(key, val, bits, tile=4096, warps=8):
    """flow_radix_hist_kernel + scan + flow_radix_scatter_kernel, pass by pass."""
    k, v, n = key.copy(), val.copy(), len(key)
    tiles = (n + tile - 1) // tile
    per = tile // warps
    for shift in range(0, bits, 8):
        d = (k >> shift) & 255
        counts = np.zeros((256, tiles), np.int64)
        for t in range(tiles):
            counts[:, t] = np.bincount(d[t * tile:(t + 1) * tile], minlength=256)
        flat = counts.reshape(-1)
        offs = np.concatenate([[0], np.cumsum(flat)[:-1]]).reshape(256, tiles)
        ko = np.full(n, -1, np.int64)
        vo = np.full(n, -1, np.int64)
        for t in range(tiles):
            wc = np.zeros((warps, 256), np.int64)
            for w in range(warps):
                lo, hi = t * tile + w * per, min(t * tile + (w + 1) * per, n)
                if lo < hi:
                    wc[w] = np.bincount(d[lo:hi], minlength=256)
            run = offs[:, t].copy()
            for w in range(warps):
                tmp = wc[w].copy()
                wc[w] = run
                run = run + tmp
            for w in range(warps):
                for c in range(0, per, 32):
                    idx = np.arange(t * tile + w * per + c, t * tile + w * per + c + 32)
                    idx = idx[idx < n]
                    dd = d[idx]
                    for li, ix in enumerate(idx):
                        pos = wc[w, dd[li]] + np.count_nonzero(dd[:li] == dd[li])
                        assert 0 <= pos < n and ko[pos] == -1
                        ko[pos], vo[pos] = k[ix], v[ix]
                    for dg in np.unique(dd):
                        wc[w, dg] += np.count_nonzero(dd == dg)
        assert (ko >= 0).all()
        k, v = ko.astype(np.uint32), vo.astype(np.uint32)
    return k, v


def latest(row):
    best, val = None, 0
    for s in row:
        t = int(s) >> 32
        if t != EMPTY and (best is None or t > best):
            best, val = t, i32(int(s))
    return val


def victim_rank_slot(row, want):
    keys = [u32((int(s) >> 32) + 1) for s in row]
    return sorted(range(len(row)), key=lambda d: (keys[d], d))[want]


def transfer(op, vals):
    kind, amt0, amod = op & 3, (op >> 8) & 4095, (op >> 20) & 4095
    amt = 1 + u32(amt0 - 1 + sum(u32(x) for x in vals[2:])) % amod
    hw = kind == 2 or vals[0] >= amt
    return hw, (i32(vals[0] - amt) if hw else vals[0]), (i32(vals[1] + amt) if hw else vals[1])


def flow_model(op, off, addr, n_items, slots, depth, base0, exact_sort):
    n, slots = len(op), slots.copy()
    nr = (op >> 2) & 63
    ro = (op & 3) == 0
    ne = [int(nr[i]) + (0 if ro[i] else (1 if addr[off[i]] == addr[off[i] + 1] else 2))
          for i in range(n)]
    eoff = np.concatenate([[0], np.cumsum(ne)]).astype(np.int64)
    E = int(eoff[n])
    key, val = np.zeros(E, np.uint32), np.zeros(E, np.uint32)
    for i in range(n):
        e = eoff[i]
        for k in range(nr[i]):
            key[e + k], val[e + k] = addr[off[i] + k], (i << 7) | k
        if ne[i] > nr[i]:
            a0, a1 = addr[off[i]], addr[off[i] + 1]
            if a0 == a1:
                key[e + nr[i]], val[e + nr[i]] = a1, (i << 7) | (WRITE + 1)
            else:
                key[e + nr[i]], val[e + nr[i]] = a0, (i << 7) | WRITE
                key[e + nr[i] + 1], val[e + nr[i] + 1] = a1, (i << 7) | (WRITE + 1)
    order = np.argsort(key, kind="stable")
    sk, sv = key[order], val[order]
    if exact_sort:
        rk, rv = radix_sort(key, val, max(1, (n_items - 1).bit_length()))
        assert (rk == sk).all() and (rv == sv).all()
    wmark = np.where((sv & 127) >= WRITE, np.arange(E) + 1, 0)
    wpos = np.concatenate([[0], np.maximum.accumulate(wmark)[:-1]]) if E else wmark
    code = lambda v: int(v >> 7) * 2 + (int(v & 127) - WRITE)
    src, tails = {}, []
    for p in range(E):
        x, v, q1 = int(sk[p]), int(sv[p]), int(wpos[p])
        prev = q1 != 0 and sk[q1 - 1] == x
        if (v & 127) < WRITE:
            src[eoff[v >> 7] + (v & 127)] = (("p", code(sv[q1 - 1])) if prev else
                                             ("v", latest(slots[x * depth:(x + 1) * depth])))
        if (p + 1 == E or sk[p + 1] != x) and ((v & 127) >= WRITE or prev):
            tails.append((x, code(v if (v & 127) >= WRITE else sv[q1 - 1])))
    assert len(tails) <= 2 * n
    out, wflag, cnt, result = {}, np.zeros(n + 1, np.int64), {}, np.zeros(n, np.int32)
    for i in range(n):  # every producer is earlier: stream order is a dependency order
        vals = []
        for k in range(nr[i]):
            kind_, s = src[eoff[i] + k]
            assert kind_ == "v" or (s // 2 < i and s in out)
            vals.append(s if kind_ == "v" else out[s])
        if ro[i]:
            result[i] = i32(sum(u32(x) for x in vals))
            continue
        hw, o0, o1 = transfer(int(op[i]), vals)
        a0, a1 = int(addr[off[i]]), int(addr[off[i] + 1])
        if a0 != a1:
            out[2 * i] = o0
        out[2 * i + 1] = o1
        wflag[i] = hw
        if hw:
            for a in {a0, a1}:
                cnt[a] = cnt.get(a, 0) + 1
    rank = np.concatenate([[0], np.cumsum(wflag[:n])])
    outcome, log = np.zeros(n, np.uint32), np.full(int(rank[n]), EMPTY, np.uint32)
    for i in range(n):
        if rank[i + 1] != rank[i]:
            ts = base0 + rank[i] + 1
            log[ts - 1 - base0], outcome[i] = i, ts
        else:
            outcome[i] = (base0 + rank[i]) | 0x80000000
    cw = {}
    for x, c in tails:
        total = cnt.pop(x, 0)
        if total == 0:
            continue
        got = []
        while True:
            j, s = c >> 1, c & 1
            if rank[j + 1] != rank[j]:
                got.append((base0 + rank[j] + 1, out[c]))
                if len(got) == min(total, depth):
                    break
            kind_, sp = src[eoff[j] + s]  # j's read of x
            if kind_ == "v":
                break
            c = sp
        assert len(got) == min(total, depth)
        row = [int(z) for z in slots[x * depth:(x + 1) * depth]]
        new = list(row)
        for e, (ts, v) in enumerate(got):
            new[victim_rank_slot(row, (total - 1 - e) % depth)] = (int(ts) << 32) | u32(v)
        slots[x * depth:(x + 1) * depth] = np.array(new, np.uint64)
        cw[x] = got[0][0]
    assert not cnt
    return slots, log, outcome, result, base0 + int(rank[n]), cw


def stream_order(op, off, addr, depth, slots, base0):
    """One transaction at a time; each write replaces the victim of its account's slots."""
    slots, ts, n = slots.copy(), base0, len(op)
    nr = (op >> 2) & 63
    outcome, result, log, cw = np.zeros(n, np.uint32), np.zeros(n, np.int32), [], {}
    for i in range(n):
        vals = [latest(slots[a * depth:(a + 1) * depth]) for a in addr[off[i]:off[i] + nr[i]]]
        if (op[i] & 3) == 0:
            result[i] = i32(sum(u32(x) for x in vals))
            outcome[i] = ts | 0x80000000
            continue
        hw, o0, o1 = transfer(int(op[i]), vals)
        if not hw:
            outcome[i] = ts | 0x80000000
            continue
        ts += 1
        log.append(i)
        outcome[i] = ts
        a0, a1 = int(addr[off[i]]), int(addr[off[i] + 1])
        for a, v in ([(a1, o1)] if a0 == a1 else [(a0, o0), (a1, o1)]):
            row = [int(z) for z in slots[a * depth:(a + 1) * depth]]
            slots[a * depth + victim_rank_slot(row, 0)] = (ts << 32) | u32(v)
            cw[a] = ts
    return slots, np.array(log, np.uint32), outcome, result, ts, cw


CASES = {
    "64-accounts-radix": dict(n_acc=64, n=32 * 8, depth=4, exact=True, chunks=1, self_every=0,
                              kw=dict(seed=3, pr_read_pct=20, ro_reads=8, up_reads=3)),
    "16-accounts-depth2": dict(n_acc=16, n=32 * 40, depth=2, exact=True, chunks=1, self_every=0,
                               kw=dict(seed=5, pr_read_pct=10, ro_reads=4, up_reads=2)),
    "zipf-depth8-two-runs": dict(n_acc=300, n=32 * 64, depth=8, exact=True, chunks=2, self_every=0,
                                 kw=dict(seed=7, pr_read_pct=0, up_reads=4,
                                         dist=cg.DIST_ZIPF, zipf_theta=0.99)),
    "self-transfers": dict(n_acc=512, n=32 * 60, depth=4, exact=False, chunks=1, self_every=5,
                           kw=dict(seed=21, pr_read_pct=10, ro_reads=8, up_reads=3,
                                   dist=cg.DIST_ZIPF, zipf_theta=0.99)),
    "always-two-accounts-three-runs": dict(n_acc=2, n=32 * 30, depth=4, exact=False, chunks=3,
                                           self_every=0,
                                           kw=dict(seed=2, pr_read_pct=0, up_reads=2,
                                                   kind=cg.KIND_TRANSFER_ALWAYS)),
}


@pytest.mark.parametrize("case", list(CASES))
def test_flow_model_equals_stream_order(case):
    c = CASES[case]
    w = cg.bank_workload(c["n_acc"], c["n"], **c["kw"])
    s = cg.generate(w)
    if c["self_every"]:  # transfers that name one account twice write it once
        t = np.flatnonzero((s.op & 3) != 0)[::c["self_every"]]
        s.addr[s.off[t] + 1] = s.addr[s.off[t]]
    depth, n = c["depth"], c["n"] // c["chunks"]
    slots0 = np.full(c["n_acc"] * depth, np.uint64(EMPTY) << np.uint64(32), np.uint64)
    slots0[0::depth] = np.uint64(1000)
    a = b = slots0
    base, logs, outs, ress = 0, [], [], []
    for k in range(c["chunks"]):
        op, off = s.op[k * n:(k + 1) * n], s.off[k * n:(k + 1) * n]
        fa = flow_model(op, off, s.addr, c["n_acc"], a, depth, base, c["exact"])
        fb = stream_order(op, off, s.addr, depth, b, base)
        np.testing.assert_array_equal(fa[0], fb[0])  # versions in the same slots
        for x, y in zip(fa[1:4], fb[1:4]):           # log, outcomes, results
            np.testing.assert_array_equal(x, y)
        assert fa[4] == fb[4] and fa[5] == fb[5]     # final timestamp, commit words
        a, b, base = fa[0], fb[0], fa[4]
        logs.append((fa[1] + k * n).astype(np.uint32))
        outs.append(fa[2])
        ress.append(fa[3])
    if not c["self_every"]:  # a self-transfer keeps only its credit: no balance invariant
        err = orc.check(s.op, s.off, s.addr, c["n_acc"], np.full(c["n_acc"], 1000, np.int32),
                        depth, base, np.concatenate(logs), np.concatenate(outs),
                        np.concatenate(ress), a)
        assert err is None, err
