"""GPU tests of the cache's serving loop (csmv_serve_*): results equal the batch engine's, a
batch's results are the same served alone and in a mix of overlapping batches (exact: GET
results are integers), overlapping batches that share hot keys replay exactly in the oracle
from the session's commit log, and admission holds batches back until room frees up."""
import time

import numpy as np
import pytest

import csmv_gb300 as cg
import oracle as orc

pytestmark = pytest.mark.gpu


def _ids_requests(ids, kind, seed=0):
    """Requests of one kind (0 GET / 1 SET) for explicit key ids: key words {id, id * 2654435761,
    id ^ 0x5bd1e995, id + 7} (uint32), SET values from the generator."""
    ids = np.asarray(ids, np.uint32)
    n = len(ids)
    assert n % 32 == 0
    req = cg.memcd_generate(cg.memcd_workload(1 << 20, n, seed=seed, get_pct=0 if kind else 100,
                                              dist=cg.DIST_UNIFORM))
    req.key[:] = np.stack([ids, ids * np.uint32(2654435761), ids ^ np.uint32(0x5bd1e995),
                           ids + np.uint32(7)], axis=1)
    req.kind[:] = kind
    return req


def _wait(srv, bid, timeout=30.0):
    t0 = time.time()
    while True:
        r = srv.poll(bid)
        if r is not None:
            return r
        assert time.time() - t0 < timeout, "batch did not complete"
        time.sleep(0.0002)


@pytest.mark.parametrize("serial", [0, 1])
def test_serving_results_equal_the_batch_engine(serial):
    """(serial: one batch on the device at a time.)"""
    n_sets = 1 << 14
    rng = np.random.default_rng(1)
    keys = rng.choice(1 << 24, 1 << 14, replace=False).astype(np.uint32)
    fill = _ids_requests(keys, 1, seed=3)
    gets = _ids_requests(np.concatenate([keys[:3000], rng.integers(0, 1 << 24, 2120)]).astype(np.uint32), 0)
    with cg.Memcd(n_sets=n_sets, client_warps=4, max_req=1 << 14) as ref:
        ref.run(fill)
        f_ref, v_ref, _ = ref.run(gets)
    with cg.Server(n_sets=n_sets, client_warps=4, arena_requests=1 << 15,
                   serial_batches=serial) as srv:
        srv.start()
        _wait(srv, srv.submit(fill))
        f, v, ns = _wait(srv, srv.submit(gets))
        st = srv.stop()
    assert st.error == 0 and st.commits_update == fill.n_req
    np.testing.assert_array_equal(f, f_ref)
    np.testing.assert_array_equal(v, v_ref)
    assert f[:3000].all() and ns > 0


def test_results_same_alone_and_in_a_mix_of_overlapping_batches():
    """X (GETs) served alone, then again while batches Y that GET and SET other, already stored
    keys are in flight: X's results are identical, and the batches did overlap."""
    n_sets = 1 << 14
    rng = np.random.default_rng(2)
    keys = rng.choice(1 << 24, 1 << 14, replace=False).astype(np.uint32)
    kx, ky = keys[:4096], keys[4096:]
    with cg.Server(n_sets=n_sets, client_warps=4, arena_requests=1 << 17,
                   serial_batches=0) as srv:
        srv.start()
        _wait(srv, srv.submit(_ids_requests(keys, 1, seed=5)))
        x = _ids_requests(rng.permutation(kx), 0)
        alone = _wait(srv, srv.submit(x))
        ys = []
        for i in range(6):  # SETs update stored keys only (no insertion, so no eviction)
            ids = rng.choice(ky, 8192).astype(np.uint32)
            ys.append(srv.submit(_ids_requests(ids, 1 if i % 2 else 0, seed=10 + i)))
        in_flight = sum(srv.poll(b, results=False) is None for b in ys)
        xb = srv.submit(x)
        mix = _wait(srv, xb)
        for b in ys:
            _wait(srv, b)
        st = srv.stop()
    assert st.error == 0
    assert in_flight > 0, "the mix did not overlap"
    np.testing.assert_array_equal(mix[0], alone[0])
    np.testing.assert_array_equal(mix[1], alone[1])
    assert alone[0].all()


def test_admission_holds_batches_until_room_frees():
    with cg.Server(n_sets=1 << 12, client_warps=2, arena_requests=1 << 12) as srv:
        srv.start()
        req = cg.memcd_generate(cg.memcd_workload(1 << 16, 2048, seed=4, get_pct=95))
        ids, refused = [], 0
        for _ in range(40):
            b = srv.submit(req)
            if b is None:
                refused += 1
                time.sleep(0.001)
            else:
                ids.append(b)
        for b in ids:
            _wait(srv, b)
        st = srv.stop()
    assert refused > 0 and len(ids) >= 2 and st.error == 0
    assert st.commits_readonly + st.commits_update == 2048 * len(ids)


def test_overlapping_batches_sharing_hot_keys_replay_exactly():
    """Batches that GET and SET the SAME hot keys (Zipf over a small key set, inserts and
    evictions included) are served overlapped; the session's commit log and every request's
    outcome replay exactly in the oracle from the table the session started with: each SET's
    installed entry and each GET's result equal the serial replay in commit order."""
    n_sets = 1 << 10
    n_b, per = 24, 2048
    with cg.Server(n_sets=n_sets, client_warps=4, arena_requests=1 << 16,
                   max_inflight_sets=1 << 15, log_cap=1 << 17, serial_batches=0) as srv:
        srv.start()  # a session of fills, then the table it leaves is the replay's start
        fill = cg.memcd_generate(cg.memcd_workload(1 << 13, 8192, seed=21, get_pct=0))
        _wait(srv, srv.submit(fill, tick=1))
        srv.stop()
        table0 = srv.table()
        reqs = [cg.memcd_generate(cg.memcd_workload(1 << 13, per, seed=100 + i,
                                                    get_pct=60 + (i % 4) * 10,
                                                    dist=cg.DIST_ZIPF, zipf_theta=0.99))
                for i in range(n_b)]
        srv.start()
        ids = [srv.submit(r, tick=2) for r in reqs]
        assert all(b is not None for b in ids)
        overlapped = sum(srv.poll(b, results=False) is None for b in ids[1:])
        res = [_poll_logged(srv, b) for b in ids]
        st = srv.stop()
        log_txn, base = srv.log()
        tags, recs = srv.table()
    assert st.error == 0
    assert overlapped > 0, "the batches did not overlap"
    kind = np.concatenate([r.kind for r in reqs])
    key = np.concatenate([r.key for r in reqs])
    val = np.concatenate([r.val for r in reqs])
    found = np.concatenate([x[0] for x in res])
    val_out = np.concatenate([x[1] for x in res])
    outcome = np.concatenate([x[2] for x in res])
    n_set = int(np.count_nonzero(kind == cg.MEMCD_SET))
    assert st.commits_update == n_set and st.commits_readonly == kind.shape[0] - n_set
    orc.memcd_check(kind, key, val, 2, n_sets, table0, base, log_txn, outcome, found, val_out,
                    tags, recs)


def _poll_logged(srv, bid, timeout=30.0):
    t0 = time.time()
    while True:
        r = srv.poll(bid, outcome=True)
        if r is not None:
            return r
        assert time.time() - t0 < timeout, "batch did not complete"
        time.sleep(0.0002)
