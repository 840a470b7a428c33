"""GPU parity tests of the transactional cache (memcachedGPU/memcdSH.cu) through the C ABI.

Bar (integer path, bit-exact): the batch's SETs replayed serially in commit-ts order from the
table before the batch reproduce the device's version store bit for bit (tags and records), and
every GET returns what the serial state at its snapshot holds (hit flag and all 8 value words).
"""
import numpy as np
import pytest

import csmv_gb300 as cg
import oracle as orc
from gpu_util import memcd_run_checked

pytestmark = pytest.mark.gpu


def _mixed_requests(seed, n, n_keys, set_pct):
    return cg.memcd_generate(cg.memcd_workload(n_keys, n, seed=seed, get_pct=100 - set_pct,
                                               dist=cg.DIST_UNIFORM))


@pytest.mark.parametrize("batch", [cg.BATCH_CTA, cg.BATCH_WARP])
def test_small_table_heavy_sets_exact_over_batches(batch):
    """64 sets x 8 ways, half the rounds SETs over 2000 keys: constant eviction and conflicts."""
    with cg.Memcd(n_sets=64, client_warps=4, ctas=8, batch=batch, max_req=8192) as cache:
        for b in range(4):
            memcd_run_checked(cache, _mixed_requests(10 + b, 8192, 2000, 50))


def test_one_hot_key_contention_exact():
    """Every request on one key: SETs serialise on one entry, GETs race them."""
    w = cg.memcd_workload(1, 4096, seed=3, get_pct=60, dist=cg.DIST_UNIFORM)
    with cg.Memcd(n_sets=16, client_warps=8, ctas=16, max_req=4096) as cache:
        for _ in range(2):
            memcd_run_checked(cache, cg.memcd_generate(w))


def test_cache_config_zipf_99_1_exact():
    """8-way sets, Zipf(0.99) over 4M keys, 99 % GET / 1 % SET rounds, 64 K-request batches
    (the table has 2^18 sets here so the host replay stays quick)."""
    w = cg.memcd_workload(1 << 22, 1 << 16, seed=1, get_pct=99)
    with cg.Memcd(n_sets=1 << 18, client_warps=4, max_req=1 << 16) as cache:
        # warm the table with SET-only batches, then the 99/1 mix
        warm = cg.memcd_workload(1 << 22, 1 << 16, seed=2, get_pct=0)
        memcd_run_checked(cache, cg.memcd_generate(warm))
        for s in range(3):
            w.seed = 100 + s
            found, _, st = memcd_run_checked(cache, cg.memcd_generate(w))
            assert found.sum() > 0


def test_full_size_table_device_pointers_exact():
    """2^20 sets (8 M entries, 16 M versions) driven through the device-pointer entry point,
    checked against the serial replay like the host-buffer path."""
    torch = pytest.importorskip("torch")
    w = cg.memcd_workload(1 << 22, 1 << 16, seed=7, get_pct=90)
    req = cg.memcd_generate(w)
    with cg.Memcd(n_sets=1 << 20, client_warps=4, max_req=1 << 16) as cache:
        cache.run(cg.memcd_generate(cg.memcd_workload(1 << 22, 1 << 16, seed=8, get_pct=0)))
        table0 = cache.table()
        d = {k: torch.from_numpy(np.ascontiguousarray(v).view(np.int32)).cuda()
             for k, v in (("kind", req.kind), ("key", req.key), ("val", req.val))}
        f = torch.full((req.n_req,), 7, dtype=torch.int32, device="cuda")
        o = torch.full((req.n_req, 8), 7, dtype=torch.int32, device="cuda")
        b = cg.MemcdBatch(req.n_req, cache.tick, d["kind"].data_ptr(), d["key"].data_ptr(),
                          d["val"].data_ptr(), f.data_ptr(), o.data_ptr())
        st = cache.run_device(b)
        torch.cuda.synchronize()
        assert st.commits_update + st.commits_readonly == req.n_req
        found = f.cpu().numpy().view(np.uint32)
        vo = o.cpu().numpy().view(np.uint32)
        log_txn, outcome, base = cache.log(req.n_req)
        tags, recs = cache.table()
        orc.memcd_check(req.kind, req.key, req.val, cache.tick, cache.cfg.n_sets, table0, base,
                        log_txn, outcome, found, vo, tags, recs)
        assert found.sum() > 0


def test_mixed_round_is_rejected():
    w = cg.memcd_workload(100, 64, seed=1, get_pct=50, dist=cg.DIST_UNIFORM)
    req = cg.memcd_generate(w)
    req.kind[5] = 1 - req.kind[5]
    with cg.Memcd(n_sets=16, client_warps=1, ctas=1, max_req=64) as cache:
        with pytest.raises(cg.CsmvError) as e:
            cache.run(req)
        assert e.value.status == 1
