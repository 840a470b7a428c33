"""GPU tests of the reference's naive baseline STM restated as a comparison arm
(csmv_bank_run_baseline_device): every run replays exactly in the oracle (commit log in
timestamp order, read-only results at their snapshots, version slots), on uniform and Zipf
banks, with max_reads 4 and 8, and interleaved with the commit engine on one bank."""
import numpy as np
import pytest

import csmv_gb300 as cg
import oracle as orc
from gpu_util import c1_workload, sub_stream, to_device, zipf_bank_workload

pytestmark = pytest.mark.gpu


def _run_baseline(w, *, depth=4, **cfg):
    torch = pytest.importorskip("torch")
    s = cg.generate(w)
    ds, keep = to_device(torch, s)
    with cg.Bank(n_accounts=w.n_accounts, max_txn=w.n_txn, version_depth=depth, **cfg) as bank:
        bank.load()
        st = bank.run_baseline_device(ds)
        log_txn, outcome, result = bank.log(w.n_txn, st.final_ts)
        slots = bank.versions()
    assert st.error == 0 and st.commits == w.n_txn
    # dense timestamps: only committed transfers take one
    assert st.commits_update + st.commits_nowrite == st.final_ts
    init = np.full(w.n_accounts, 1000, np.int32)
    err = orc.check(s.op, s.off, s.addr, w.n_accounts, init, depth, st.final_ts, log_txn, outcome,
                    result, slots)
    assert err is None, err
    return st


@pytest.mark.parametrize("max_reads", [4, 8])
def test_baseline_uniform_exact(max_reads):
    """4096 accounts, 2^14 transactions, 90/10, 8 client warps x 8 CTAs."""
    _run_baseline(c1_workload(n_txn=1 << 14, up_reads=4), ctas=8, client_warps=8,
                  max_reads=max_reads, log_commits=1)


def test_baseline_contended_exact():
    """A small bank (256 accounts) so sections meet conflicting records and lower lanes."""
    st = _run_baseline(c1_workload(n_txn=1 << 13, n_accounts=256, up_reads=4, ro_reads=16,
                                   pr_read_pct=20),
                       ctas=16, client_warps=4, log_commits=1)
    assert st.aborts_read_write > 0


def test_baseline_zipf_exact():
    """The contended Zipf(0.99) bank on 2^20 accounts, read 4 / write 2, 20 % scans of 32."""
    _run_baseline(zipf_bank_workload(1 << 15), depth=8, ctas=152, client_warps=2, max_reads=4,
                  log_commits=1)


def test_baseline_interleaves_with_engine():
    """Engine run, baseline run, engine run, baseline run on one bank: the commit order carries
    across them and the concatenated log replays exactly."""
    torch = pytest.importorskip("torch")
    n_acc, n = 4096, 32 * 256
    w = c1_workload(n_txn=4 * n, n_accounts=n_acc, seed=23, dist=cg.DIST_ZIPF, zipf_theta=0.9,
                    up_reads=4)
    s = cg.generate(w)
    logs, outs, ress = [], [], []
    with cg.Bank(n_accounts=n_acc, max_txn=n, ctas=8, client_warps=4, log_commits=1) as bank:
        bank.load()
        prev = 0
        for i in range(4):
            ds, keep = to_device(torch, sub_stream(s, i * n, (i + 1) * n))
            st = (bank.run_device if i % 2 == 0 else bank.run_baseline_device)(ds)
            assert st.error == 0 and st.commits == n
            lt, oc, rs = bank.log(n, st.final_ts - prev)
            logs.append(np.where(lt != 0xFFFFFFFF, lt + i * n, lt).astype(np.uint32))
            outs.append(oc)
            ress.append(rs)
            prev = st.final_ts
        slots = bank.versions()
    err = orc.check(s.op, s.off, s.addr, n_acc, np.full(n_acc, 1000, np.int32), 4, prev,
                    np.concatenate(logs), np.concatenate(outs), np.concatenate(ress), slots)
    assert err is None, err


def test_baseline_refuses_engine_only_stream_fields():
    torch = pytest.importorskip("torch")
    w = c1_workload(n_txn=1024)
    s = cg.generate(w)
    ds, keep = to_device(torch, s)
    bo = torch.zeros(w.n_txn, dtype=torch.int32, device="cuda")
    ds.backoff = bo.data_ptr()
    with cg.Bank(n_accounts=w.n_accounts, max_txn=w.n_txn) as bank:
        bank.load()
        with pytest.raises(cg.CsmvError):
            bank.run_baseline_device(ds)
