"""A bank client written in the reference's style, compiled against include/csmv_ref_api.cuh (the
reference's device API signatures - TXBegin, TXRead, TXReadOnly, TXWrite, TXPreValidation,
TXAddToRecord, TXWriteBack - on this project's version store), runs on the GPU and replays
exactly in the CPU oracle: every commit in commit-timestamp order reproduces the final version
slots bit for bit, read-only sums and no-write transfers match the state at their snapshots, and
the balance is conserved."""
import ctypes as C

import numpy as np
import pytest

import csmv_gb300 as cg
import oracle as orc
from csmv_gb300 import build as b
from gpu_util import c1_workload

pytestmark = pytest.mark.gpu


def _lib():
    L = C.CDLL(str(b.DEVTEST_LIB))
    fn = L.csmv_devtest_refapi_bank
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p] * 3 + [C.c_uint32, C.c_uint64, C.c_uint32, C.c_void_p, C.c_uint32,
                                      C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p,
                                      C.c_void_p, C.c_void_p]
    L.csmv_devtest_refapi_depth.restype = C.c_int
    return L


@pytest.mark.parametrize("dist,n_acc", [(cg.DIST_UNIFORM, 4096), (cg.DIST_ZIPF, 2048)])
def test_reference_style_client_replays_exactly(dist, n_acc):
    L = _lib()
    depth = L.csmv_devtest_refapi_depth()
    w = c1_workload(n_txn=8 * 128 * 32, n_accounts=n_acc, dist=dist, zipf_theta=0.99, up_reads=4,
                    pr_read_pct=10, seed=17)
    s = cg.generate(w)
    init = np.full(n_acc, 1000, np.int32)
    slots = np.zeros(n_acc * depth, np.uint64)
    log = np.zeros(w.n_txn, np.uint32)
    outcome = np.zeros(w.n_txn, np.uint32)
    result = np.zeros(w.n_txn, np.int32)
    final_ts = C.c_uint32()
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    rc = L.csmv_devtest_refapi_bank(p(s.op), p(s.off), p(s.addr), w.n_txn, s.addr.shape[0], n_acc,
                                    p(init), 8, 128, p(slots), p(log), w.n_txn, p(outcome),
                                    p(result), C.byref(final_ts))
    assert rc == 0, rc
    n = final_ts.value
    assert 0 < n <= w.n_txn and (log[:n] != 0xFFFFFFFF).all()
    err = orc.check(s.op, s.off, s.addr, n_acc, init, depth, n, log[:n], outcome, result, slots)
    assert err is None, err
