"""ctypes binding of the CPU oracle (oracle/liboracle.so). TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference legs import this
module, as the checker and the CPU baseline; the product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
REF_LIB = HERE / "_ref" / "libcsmv_ref.so"
SNAP_FLAG = 0x80000000


def build(force: bool = False) -> Path:
    """Compile the oracle (gcc) and, when the reference tree is present, the reference pin."""
    src = HERE / "csmv_oracle.c"
    if force or not LIB.exists() or LIB.stat().st_mtime < max(
            src.stat().st_mtime, (HERE / "csmv_oracle.h").stat().st_mtime):
        subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-std=c11", "-pthread", str(src),
                        "-o", str(LIB), "-lm"], check=True)
    subprocess.run(["bash", str(HERE / "ref_build.sh")], check=True, capture_output=True)
    return LIB


class Workload(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("n_accounts", C.c_uint32), ("n_txn", C.c_uint32),
                ("pr_read_pct", C.c_uint32), ("ro_reads", C.c_uint32), ("up_reads", C.c_uint32),
                ("kind", C.c_uint32), ("amt_lo", C.c_uint32), ("amt_hi", C.c_uint32),
                ("dist", C.c_uint32), ("zipf_theta", C.c_double), ("hot_frac", C.c_double),
                ("hot_prob", C.c_double), ("shift_every", C.c_uint32)]


class Record(C.Structure):
    _fields_ = [("txn", C.c_uint32), ("n_writes", C.c_uint32), ("ws", C.c_uint32 * 4)]


class SimStats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("commits_update", "commits_readonly",
                                          "commits_nowrite", "aborts_prevalid",
                                          "aborts_read_write", "rounds",
                                          "aborts_write_write")] + [
        ("final_ts", C.c_uint32)]


_lib = None
_ref = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        _lib = C.CDLL(str(LIB))
        _sigs(_lib, {
            "orc_rand_r": (C.c_uint64, [P]),
            "orc_h64": (C.c_uint64, [C.c_uint64]),
            "orc_rnd32": (C.c_uint32, [C.c_uint64, C.c_uint64, C.c_uint64]),
            "orc_bank_stream_size": (I, [P, P]),
            "orc_bank_generate": (I, [P, P, P, P]),
            "orc_ref_read": (I, [C.c_uint16, C.c_uint16, P, P, I, U, P]),
            "orc_ref_writeback": (None, [P, P, P, P, I, U, C.c_int32]),
            "orc_packed_read": (I, [P, I, U, P]),
            "orc_packed_victim": (I, [P, I]),
            "orc_packed_writeback": (None, [P, I, U, C.c_int32]),
            "orc_prevalidate": (U, [P, P, I, P, P, I, U, P]),
            "orc_ref_validate": (I, [P, I, I, I, I, I, P, I]),
            "orc_batched_validate": (I, [P, I, I, I, I, I, P, I]),
            "orc_collab_validate": (None, [P, I, I, I, P, P, P, I, P]),
            "orc_batched_ts": (None, [U, U, P]),
            "orc_window_validate": (I, [P, U, U, U, P, I, I]),
            "orc_memcd_set_slot": (I, [P, P, P, I, C.c_int32]),
            "orc_bank_exec": (I, [U, P, P, P, P, P]),
            "orc_bank_check": (I, [U, P, P, P, U, P, I, U, P, P, P, P, C.c_char_p, I]),
            "orc_bank_check_groups": (I, [U, P, P, P, U, P, I, U, P, P, P, P, P, C.c_char_p, I]),
            "orc_bank_sim_1warp": (I, [U, P, P, P, U, P, I, I, I, P, P, P, P, P]),
            "orc_bank_serial": (I, [U, P, P, P, U, P, P]),
            "orc_bank_locked": (I, [U, P, P, P, U, P, I, P]),
            "orc_memcd_mix": (U, [P]),
            "orc_memcd_init_table": (None, [U, P, P]),
            "orc_memcd_serial": (None, [U, P, P, P, U, U, U, P, P, P, P, P, P, P]),
            "orc_memcd_check": (I, [U, P, P, P, U, U, P, P, U, U, P, P, P, P, P, P,
                                    C.c_char_p, I]),
            "orc_memcd_serial_time": (I, [U, P, P, P, U, U, P, P, P, P, P]),
        })
    return _lib


P, I, U = C.c_void_p, C.c_int, C.c_uint32


def _sigs(lib_, table):
    for name, (res, args) in table.items():
        fn = getattr(lib_, name)
        fn.restype = res
        fn.argtypes = args


def ref() -> C.CDLL | None:
    """The reference's own functions compiled for the host, or None without the reference tree."""
    global _ref
    if _ref is None and REF_LIB.exists():
        _ref = C.CDLL(str(REF_LIB))
        _sigs(_ref, {
            "ref_rand_r": (C.c_uint64, [P]),
            "ref_sh_read": (I, [C.c_uint16, C.c_uint16, P, P, U, I, P]),
            "ref_sh_writeback": (None, [P, P, P, P, U, C.c_int32]),
            "ref_sh_validate": (I, [P, I, I, I, I, P, I]),
            "ref_sh_add_to_record": (U, [P, P, P, P, I, P, I, P, I]),
            "ref_bt_validate": (I, [P, I, I, I, I, P, I]),
            "ref_bt_prevalidate": (U, [P, P, I, P, P, I]),
        })
    return _ref


def p(a: np.ndarray) -> int:
    return a.ctypes.data


def generate(w: Workload):
    n = C.c_uint64()
    assert lib().orc_bank_stream_size(C.byref(w), C.byref(n)) == 0
    op = np.empty(w.n_txn, np.uint32)
    off = np.empty(w.n_txn, np.uint32)
    addr = np.empty(n.value, np.uint32)
    assert lib().orc_bank_generate(C.byref(w), p(op), p(off), p(addr)) == 0
    return op, off, addr


def check(op, off, addr, n_accounts, init, depth, final_ts, log_txn, outcome, result,
          final_slots=None, groups=None) -> str | None:
    """Serial replay in commit-ts order; None when the run is exact, else the first violation.
    groups: bitmap (uint32 words) of the timestamps that end a commit group (None: every one)."""
    msg = C.create_string_buffer(512)
    init = np.ascontiguousarray(init, np.int32)
    log_txn = np.ascontiguousarray(log_txn, np.uint32)
    if log_txn.size == 0:
        log_txn = np.zeros(1, np.uint32)
    g = np.ascontiguousarray(groups, np.uint32) if groups is not None else None
    rc = lib().orc_bank_check_groups(
        C.c_uint32(len(op)), p(op), p(off), p(addr), C.c_uint32(n_accounts), p(init),
        C.c_int(depth), C.c_uint32(final_ts), p(log_txn), p(np.ascontiguousarray(outcome, np.uint32)),
        p(np.ascontiguousarray(result, np.int32)), p(g) if g is not None else None,
        p(np.ascontiguousarray(final_slots, np.uint64)) if final_slots is not None else None,
        msg, 512)
    return None if rc == 0 else msg.value.decode()


def sim_1warp(op, off, addr, n_accounts, init, depth, prevalidate=True, locks=True):
    n = len(op)
    slots = np.empty(n_accounts * depth, np.uint64)
    log_txn = np.zeros(n, np.uint32)
    outcome = np.zeros(n, np.uint32)
    result = np.zeros(n, np.int32)
    st = SimStats()
    init = np.ascontiguousarray(init, np.int32)
    rc = lib().orc_bank_sim_1warp(C.c_uint32(n), p(op), p(off), p(addr), C.c_uint32(n_accounts),
                                  p(init), C.c_int(depth), C.c_int(int(prevalidate)),
                                  C.c_int(int(locks)), p(slots),
                                  p(log_txn), p(outcome), p(result), C.byref(st))
    assert rc == 0
    return slots, log_txn[:st.final_ts], outcome, result, st


def serial(op, off, addr, n_accounts, init):
    vals = np.ascontiguousarray(init, np.int32).copy()
    ns = C.c_uint64()
    lib().orc_bank_serial(C.c_uint32(len(op)), p(op), p(off), p(addr), C.c_uint32(n_accounts),
                          p(vals), C.byref(ns))
    return vals, ns.value


def locked(op, off, addr, n_accounts, init, nthreads):
    vals = np.ascontiguousarray(init, np.int32).copy()
    ns = C.c_uint64()
    lib().orc_bank_locked(C.c_uint32(len(op)), p(op), p(off), p(addr), C.c_uint32(n_accounts),
                          p(vals), C.c_int(nthreads), C.byref(ns))
    return vals, ns.value


def cpu_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


# ---------------------------------------------------------------------------------------------
# transactional cache
# ---------------------------------------------------------------------------------------------

MC_VERSIONS = 16  # 8 ways x 2 versions per set


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def memcd_empty_table(n_sets: int):
    tags = np.empty(n_sets * MC_VERSIONS, np.uint64)
    recs = np.empty((n_sets * MC_VERSIONS, 16), np.uint32)
    lib().orc_memcd_init_table(n_sets, p(tags), p(recs))
    return tags, recs


def memcd_serial(kind, key, val, tick, n_sets, table=None, base_ts=0):
    """Serial execution in request order: (found, val_out, log_txn, outcome, tags, recs)."""
    kind, key, val = _c(kind, np.uint32), _c(key, np.uint32), _c(val, np.uint32)
    n = kind.shape[0]
    tags, recs = memcd_empty_table(n_sets) if table is None else (table[0].copy(), table[1].copy())
    found = np.empty(n, np.uint32)
    val_out = np.empty((n, 8), np.uint32)
    log_txn = np.empty(max(1, n), np.uint32)
    outcome = np.empty(n, np.uint32)
    n_log = C.c_uint32()
    lib().orc_memcd_serial(n, p(kind), p(key), p(val), tick, n_sets, base_ts, p(tags), p(recs),
                           p(found), p(val_out), p(log_txn), p(outcome), C.byref(n_log))
    return found, val_out, log_txn[:n_log.value], outcome, tags, recs


def memcd_check(kind, key, val, tick, n_sets, table0, base_ts, log_txn, outcome, found, val_out,
                tags, recs):
    """Replay checker; raises AssertionError with the oracle's message on a mismatch."""
    kind, key, val = _c(kind, np.uint32), _c(key, np.uint32), _c(val, np.uint32)
    log_txn, outcome = _c(log_txn, np.uint32), _c(outcome, np.uint32)
    found, val_out = _c(found, np.uint32), _c(val_out, np.uint32)
    tags, recs = _c(tags, np.uint64), _c(recs, np.uint32)
    t0 = r0 = None
    if table0 is not None:
        t0, r0 = _c(table0[0], np.uint64), _c(table0[1], np.uint32)
    msg = C.create_string_buffer(512)
    rc = lib().orc_memcd_check(kind.shape[0], p(kind), p(key), p(val), tick, n_sets,
                               p(t0) if t0 is not None else None,
                               p(r0) if r0 is not None else None, base_ts, log_txn.shape[0],
                               p(log_txn), p(outcome), p(found), p(val_out), p(tags), p(recs),
                               msg, 512)
    if rc != 0:
        raise AssertionError(f"cache replay: {msg.value.decode()}")


def memcd_serial_time(kind, key, val, tick, n_sets) -> float:
    """Seconds of one serial pass over the requests from an empty table."""
    kind, key, val = _c(kind, np.uint32), _c(key, np.uint32), _c(val, np.uint32)
    n = kind.shape[0]
    tags, recs = memcd_empty_table(n_sets)
    found = np.empty(n, np.uint32)
    val_out = np.empty((n, 8), np.uint32)
    ns = C.c_uint64()
    lib().orc_memcd_serial_time(n, p(kind), p(key), p(val), tick, n_sets, p(tags), p(recs),
                                p(found), p(val_out), C.byref(ns))
    return ns.value * 1e-9
