"""GPU tests of the autotuners: csmv_bank_autotune tries every candidate shape and commit method,
the chosen one is the fastest of the re-measured candidates, and a bank built with it runs the
workload exactly; csmv_memcd_autotune does the same for the cache's launch shape, and a cache
built with its choice replays exactly."""
import numpy as np
import pytest

import csmv_gb300 as cg
from gpu_util import c1_workload, memcd_run_checked, run_checked

pytestmark = pytest.mark.gpu


def test_autotune_picks_the_fastest_measured_shape_and_it_runs_exactly():
    w = c1_workload(n_txn=1 << 15)
    s = cg.generate(w)
    best, trials = cg.autotune(s, repeats=2, n_accounts=w.n_accounts, init_value=1000)
    # 2 commit methods x 2 read specialisations (the sample's transfers read 2 accounts) x
    # 2 depths x 4 client-warp counts x 2 CTAs per SM
    assert len(trials) == 64
    assert {t["prevalidate"] for t in trials} == {1, 3}
    assert {t["max_reads"] for t in trials} == {0, 4}
    ok = [t for t in trials if t["status"] == 0]
    assert ok, trials
    key = lambda t: (t["client_warps"], t["ctas"], t["version_depth"], t["prevalidate"],
                     t["max_reads"])
    rerun = [t for t in ok if t["runs"] > 1]
    assert rerun
    win = max(rerun, key=lambda t: t["tx_per_s"])
    assert key(win) == (best.client_warps, best.ctas, best.version_depth, best.prevalidate,
                        best.max_reads)
    run_checked(w, client_warps=best.client_warps, ctas=best.ctas,
                version_depth=best.version_depth, prevalidate=best.prevalidate,
                max_reads=best.max_reads)


def test_memcd_autotune_picks_a_measured_shape_and_it_replays_exactly():
    fill = cg.memcd_generate(cg.memcd_workload(1 << 16, 1 << 14, seed=3, get_pct=0))
    sample = cg.memcd_generate(cg.memcd_workload(1 << 16, 1 << 15, seed=4, get_pct=95))
    best, trials = cg.memcd_autotune(sample, fill, repeats=2, n_sets=1 << 12)
    assert len(trials) == 8
    ok = [t for t in trials if t["status"] == 0 and t["runs"] > 1]
    assert ok, trials
    win = max(ok, key=lambda t: t["tx_per_s"])
    assert (win["client_warps"], win["ctas"]) == (best.client_warps, best.ctas)
    with cg.Memcd(best) as cache:
        memcd_run_checked(cache, fill)
        memcd_run_checked(cache, sample)
