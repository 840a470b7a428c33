"""GPU test of the autotuner (csmv_bank_autotune): every candidate shape is tried, the chosen one
is the fastest of the re-measured candidates, and a bank built with it runs the workload
exactly."""
import numpy as np
import pytest

import csmv_gb300 as cg
from gpu_util import c1_workload, run_checked

pytestmark = pytest.mark.gpu


def test_autotune_picks_the_fastest_measured_shape_and_it_runs_exactly():
    w = c1_workload(n_txn=1 << 15)
    s = cg.generate(w)
    best, trials = cg.autotune(s, repeats=2, n_accounts=w.n_accounts, init_value=1000)
    assert len(trials) == 16
    ok = [t for t in trials if t["status"] == 0]
    assert ok, trials
    shapes = {(t["client_warps"], t["ctas"], t["version_depth"]) for t in trials}
    assert (best.client_warps, best.ctas, best.version_depth) in shapes
    rerun = [t for t in ok if t["runs"] > 1]
    assert rerun
    win = max(rerun, key=lambda t: t["tx_per_s"])
    assert (win["client_warps"], win["ctas"], win["version_depth"]) == (
        best.client_warps, best.ctas, best.version_depth)
    run_checked(w, client_warps=best.client_warps, ctas=best.ctas,
                version_depth=best.version_depth)
