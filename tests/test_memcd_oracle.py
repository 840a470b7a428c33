"""CPU tests of the cache oracle (serial semantics + replay checker) and the request generator.

The checker is what the GPU cache tests trust, so it is pinned here on known answers (the
reference's slot rule, memcachedGPU/memcdSH.cu:365-387, and GET semantics, :400-440) and shown
to reject planted mistakes.
"""
import numpy as np
import pytest

import oracle as orc
import csmv_gb300 as cg


def _reqs(rng, n, n_keys, set_frac=0.5):
    rounds = n // 32
    kind = np.repeat((rng.random(rounds) < set_frac).astype(np.uint32), 32)
    ids = rng.integers(0, n_keys, n).astype(np.uint32)
    key = np.stack([ids, ids * 7 + 1, ids ^ 0x5555, ids + 3], axis=1).astype(np.uint32)
    val = rng.integers(0, 2**32, (n, 8), dtype=np.uint64).astype(np.uint32)
    return kind, key, val


def _key(i):
    return np.array([i, i * 7 + 1, i ^ 0x5555, i + 3], np.uint32)


def test_set_then_get_hits_and_misses():
    n_sets = 4
    kind = np.array([1] * 32 + [0] * 32, np.uint32)
    key = np.stack([_key(i) for i in range(32)] + [_key(i) for i in range(16)] +
                   [_key(1000 + i) for i in range(16)])
    val = np.arange(64 * 8, dtype=np.uint32).reshape(64, 8)
    found, vo, log, outc, tags, recs = orc.memcd_serial(kind, key, val, 1, n_sets)
    # 32 keys into 4 sets x 8 ways: a key survives unless its set overflowed
    sets = np.array([orc.lib().orc_memcd_mix(orc.p(_key(i))) % n_sets for i in range(32)])
    for i in range(16):
        later_same_set = np.sum(sets[i + 1:] == sets[i])
        before_same_set = np.sum(sets[:i] == sets[i])
        # LRU ties (all tick 1) go to the first way, so an overflowing set keeps churning way 0
        if before_same_set + later_same_set < 8:
            assert found[32 + i] == 1 and (vo[32 + i] == val[i]).all()
    assert (found[48:] == 0).all() and (vo[48:] == 0).all()
    assert list(log) == list(range(32)) and (outc[:32] == np.arange(1, 33)).all()
    assert (outc[32:] == (32 | orc.SNAP_FLAG)).all()


def test_set_overwrites_its_own_way_and_evicts_min_lru():
    n_sets = 1
    k = [_key(i) for i in range(9)]
    # ticks 1..8 fill the 8 ways in order; SET of key 3 again updates way 3 in place
    table = None
    base = 0
    for t in range(8):
        kind = np.ones(32, np.uint32)
        key = np.stack([k[t]] * 32)
        val = np.full((32, 8), t, np.uint32)
        _, _, log, _, tags, recs = orc.memcd_serial(kind, key, val, t + 1, n_sets, table, base)
        table, base = (tags, recs), base + len(log)
    tags, recs = table
    newest = lambda w: 2 * w + int((tags[2 * w + 1] >> np.uint64(32)) != 0xFFFFFFFF and
                                   (tags[2 * w + 1] >> np.uint64(32)) > (tags[2 * w] >> np.uint64(32)))
    for w in range(8):
        assert (recs[newest(w), 4:8] == k[w]).all() and recs[newest(w), 0] == w + 1
    # key 8 evicts the smallest LRU (way 0, tick 1)
    kind = np.ones(32, np.uint32)
    _, _, _, _, tags2, recs2 = orc.memcd_serial(kind, np.stack([k[8]] * 32),
                                                np.full((32, 8), 99, np.uint32), 9, n_sets,
                                                table, base)
    hits = [w for w in range(8) if (recs2[2 * w:2 * w + 2, 4:8] == k[8]).all(axis=1).any()]
    assert hits == [0]


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_check_accepts_serial_runs_across_batches(seed):
    rng = np.random.default_rng(seed)
    n_sets, table, base = 16, None, 0
    for tick in range(1, 4):
        kind, key, val = _reqs(rng, 512, 300)
        found, vo, log, outc, tags, recs = orc.memcd_serial(kind, key, val, tick, n_sets, table,
                                                            base)
        orc.memcd_check(kind, key, val, tick, n_sets, table, base, log, outc, found, vo, tags,
                        recs)
        table, base = (tags, recs), base + len(log)


def test_check_allows_holes_and_rejects_planted_mistakes():
    rng = np.random.default_rng(9)
    n_sets = 8
    kind, key, val = _reqs(rng, 1024, 120)
    found, vo, log, outc, tags, recs = orc.memcd_serial(kind, key, val, 1, n_sets)
    # a hole: shift every ts from position 5 by one
    log_h = np.concatenate([log[:5], [0xFFFFFFFF], log[5:]]).astype(np.uint32)
    outc_h = outc.copy()
    for k, r in enumerate(log_h):
        if r != 0xFFFFFFFF:
            outc_h[r] = k + 1
    sets_gets = outc_h.copy()
    snaps = outc & ~np.uint32(orc.SNAP_FLAG)
    g = kind == 0
    sets_gets[g] = (snaps[g] + (snaps[g] >= 5)) | orc.SNAP_FLAG
    tags_h = tags.copy()
    for v in range(tags.shape[0]):
        t = int(tags[v]) >> 32
        if t != 0xFFFFFFFF and t >= 6:
            tags_h[v] = np.uint64(((t + 1) << 32) | (int(tags[v]) & 0xFFFFFFFF))
    orc.memcd_check(kind, key, val, 1, n_sets, None, 0, log_h, sets_gets, found, vo, tags_h,
                    recs)
    # wrong GET value
    hit = np.flatnonzero((kind == 0) & (found == 1))[0]
    bad = vo.copy()
    bad[hit, 3] ^= 1
    with pytest.raises(AssertionError):
        orc.memcd_check(kind, key, val, 1, n_sets, None, 0, log, outc, found, bad, tags, recs)
    # a GET that claims a miss
    badf = found.copy()
    badf[hit] = 0
    with pytest.raises(AssertionError):
        orc.memcd_check(kind, key, val, 1, n_sets, None, 0, log, outc, badf, vo, tags, recs)
    # a changed version record
    badr = recs.copy()
    ts = (tags >> np.uint64(32)).astype(np.int64)
    ts[ts == 0xFFFFFFFF] = -1
    badr[int(np.argmax(ts)), 9] ^= 1
    with pytest.raises(AssertionError):
        orc.memcd_check(kind, key, val, 1, n_sets, None, 0, log, outc, found, vo, tags, badr)
    # a SET missing from the log
    with pytest.raises(AssertionError):
        orc.memcd_check(kind, key, val, 1, n_sets, None, 0, log[:-1], outc, found, vo, tags,
                        recs)


def test_check_rejects_swapped_dependent_sets():
    """Two SETs of the same key in swapped commit order leave a different newest value."""
    n_sets = 2
    kind = np.ones(64, np.uint32)
    key = np.stack([_key(5)] * 64)
    val = np.arange(64 * 8, dtype=np.uint32).reshape(64, 8)
    found, vo, log, outc, tags, recs = orc.memcd_serial(kind, key, val, 1, n_sets)
    log2 = log.copy()
    log2[[62, 63]] = log2[[63, 62]]
    outc2 = outc.copy()
    outc2[[62, 63]] = outc2[[63, 62]]
    with pytest.raises(AssertionError):
        orc.memcd_check(kind, key, val, 1, n_sets, None, 0, log2, outc2, found, vo, tags, recs)


def test_product_generator_shape_and_skew():
    w = cg.memcd_workload(1 << 22, 1 << 16, seed=5, get_pct=99)
    r = cg.memcd_generate(w)
    k = r.kind.reshape(-1, 32)
    assert (k == k[:, :1]).all()                       # rounds are uniform
    assert 0.97 < (r.kind == 0).mean() < 1.0           # 99 % GET rounds
    ids = r.key[:, 0]
    assert ids.max() < (1 << 22)
    # key words are a function of the id
    _, first = np.unique(ids, return_index=True)
    lut = {int(i): tuple(r.key[j]) for i, j in zip(ids[first], first)}
    assert all(tuple(r.key[j]) == lut[int(ids[j])] for j in range(0, len(ids), 97))
    # Zipf(0.99): the most popular id is drawn far more often than 1/n
    assert np.bincount(ids).max() > 0.02 * len(ids)
    assert (r.val[r.kind == 0] == 0).all()
    r2 = cg.memcd_generate(w)
    assert (r2.key == r.key).all() and (r2.val == r.val).all()
