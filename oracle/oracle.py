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
            "orc_bank_sim_1warp": (I, [U, P, P, P, U, P, I, I, I, P, P, P, P, P]),
            "orc_bank_serial": (I, [U, P, P, P, U, P, P]),
            "orc_bank_locked": (I, [U, P, P, P, U, P, I, P]),
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
          final_slots=None) -> str | None:
    """Serial replay in commit-ts order; None when the run is exact, else the first violation."""
    msg = C.create_string_buffer(512)
    init = np.ascontiguousarray(init, np.int32)
    log_txn = np.ascontiguousarray(log_txn, np.uint32)
    if log_txn.size == 0:
        log_txn = np.zeros(1, np.uint32)
    rc = lib().orc_bank_check(
        C.c_uint32(len(op)), p(op), p(off), p(addr), C.c_uint32(n_accounts), p(init),
        C.c_int(depth), C.c_uint32(final_ts), p(log_txn), p(np.ascontiguousarray(outcome, np.uint32)),
        p(np.ascontiguousarray(result, np.int32)),
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
