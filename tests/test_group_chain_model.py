"""CPU model of group commit's chain walk (csrc/bank_kernel.cuh, group_attempt step 6), with the
kernel's staging and arithmetic: from the first lane that depends on a lower one, lane 0 runs
the round's transfers in lane order over the table of locked accounts; each step's table values
are loaded one step ahead (before the previous step's two writes land) and patched with those
writes (a1 first: it is stored last), the amount is acc mod d by the multiply-shift magic, and
the funds check selects the writes. It must leave exactly what running the transfers one at a
time in lane order leaves (table values, each lane's writes, which lanes moved funds), with
transfers that name one account twice, table reads of accounts other lanes write, and
unconditional transfers."""
import random

M32 = 0xFFFFFFFF


def i32(x):
    x &= M32
    return x - (1 << 32) if x >> 31 else x


def serial(base, lanes):
    """One transfer at a time in lane order (the reference's semantics)."""
    base = list(base)
    out, moved = {}, set()
    for j, (x0, x1, ys, facc, d, always) in lanes:
        v0, v1 = base[x0], base[x1]
        amt = 1 + ((facc + sum(base[y] for y in ys)) & M32) % d
        if always or v0 >= amt:
            w0, w1 = i32(v0 - amt), i32(v1 + amt)
            base[x0], base[x1] = w0, w1
            out[j] = (w0, w1)
            moved.add(j)
    return base, out, moved


def walk(base, lanes, nt):
    """The kernel's walk: staged (x0, x1, table reads padded with slot 0, facc, d, magic)."""
    base = list(base)
    out, moved = {}, set()
    staged = []
    for j, (x0, x1, ys, facc, d, always) in lanes:
        staged.append((j, x0, x1, len(ys), list(ys) + [0] * (nt - len(ys)), facc, d,
                       M32 // d, always))
    _, x0, x1, _, tr, *_ = staged[0]
    l0, l1, lt = base[x0], base[x1], [base[y] for y in tr]
    px0 = px1 = None
    pw0 = pw1 = 0
    for i, (j, x0, x1, n, tr, facc, d, mg, always) in enumerate(staged):
        def fwd(s, loaded):
            return pw1 if s == px1 else pw0 if s == px0 else loaded
        v0, v1 = fwd(x0, l0), fwd(x1, l1)
        acc = facc
        for q in range(nt):
            acc = (acc + (fwd(tr[q], lt[q]) if q < n else 0)) & M32
        nxt = staged[i + 1] if i + 1 < len(staged) else staged[i]
        l0, l1, lt = base[nxt[1]], base[nxt[2]], [base[y] for y in nxt[4]]  # before this step's writes
        r = (acc - ((acc * mg) >> 32) * d) & M32
        r = r - d if r >= d else r
        amt = 1 + r
        ok = always or v0 >= amt
        w0 = i32(v0 - amt) if ok else v0
        w1 = i32(v1 + amt) if ok else v1
        base[x0], base[x1] = w0, w1
        out[j] = (w0, w1)
        if ok:
            moved.add(j)
        px0, px1, pw0, pw1 = x0, x1, w0, w1
    return base, out, moved


def test_chain_walk_equals_lane_order():
    rng = random.Random(2026)
    for _ in range(4000):
        slots = rng.choice([2, 3, 5, 8, 128])  # few slots: lanes share accounts often
        nt = rng.choice([2, 6])                 # table reads of a 4-read / 8-read kernel
        base = [rng.randint(-5, 60) for _ in range(128)]
        lanes = []
        for j in sorted(rng.sample(range(32), rng.randint(1, 32))):
            x0, x1 = rng.randrange(slots), rng.randrange(slots)
            ys = [rng.randrange(slots) for _ in range(rng.randint(0, nt))]
            lanes.append((j, (x0, x1, ys, rng.randint(0, M32), rng.randint(1, 50),
                              rng.random() < 0.2)))
        b1, o1, m1 = serial(base, lanes)
        b2, o2, m2 = walk(base, lanes, nt)
        assert b1 == b2 and m1 == m2
        assert all(o1[j] == o2[j] for j in m1)
