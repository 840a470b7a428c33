"""Python binding (ctypes) of the CSMV GB300 C ABI (include/csmv.h).

Mirrors the reference's host interface for the commit path: ``Bank`` stands in for the
TXInit / parent_kernel / TXEnd sequence of bank/csmv_sh/exe.cu:340-529 (create + load, run,
read back), ``Memcd`` for the cache set-up and batch loop of memcachedGPU/memcdSH.cu:557-651,
with statistics named after the reference's Statistics struct (bank/csmv_sh/API.cuh:112-119). There is no CPU fallback: every call goes through
``lib/libcsmv.so`` and raises when the library is missing or a call fails.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass
from pathlib import Path

import numpy as np

PKG_ROOT = Path(__file__).resolve().parent.parent
LIB_PATH = PKG_ROOT / "lib" / "libcsmv.so"

STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "out of memory",
          4: "bounded device wait timed out", 5: "capacity exceeded", 6: "no sm_103 device",
          7: "call out of order", 8: "file error"}

KIND_READONLY, KIND_TRANSFER, KIND_TRANSFER_ALWAYS = 0, 1, 2
DIST_UNIFORM, DIST_ZIPF, DIST_HOTSPOT = 0, 1, 2
VALIDATE_STAMP, VALIDATE_RING, VALIDATE_RING_LANE = 0, 1, 2
WRITEBACK_CLIENT, WRITEBACK_SERVER = 0, 1
BATCH_LANE, BATCH_WARP, BATCH_CTA, BATCH_CLUSTER = 0, 1, 2, 3
SNAP_FLAG = 0x80000000
MEMCD_GET, MEMCD_SET = 0, 1
MEMCD_WAYS, MEMCD_DEPTH, KEY_WORDS, VAL_WORDS = 8, 2, 4, 8
HOLE = 0xFFFFFFFF


class CsmvError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str):
        super().__init__(f"{where}: {STATUS.get(status, status)} ({detail})")
        self.status = status


class BankWorkload(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("n_accounts", C.c_uint32), ("n_txn", C.c_uint32),
                ("pr_read_pct", C.c_uint32), ("ro_reads", C.c_uint32), ("up_reads", C.c_uint32),
                ("kind", C.c_uint32), ("amt_lo", C.c_uint32), ("amt_hi", C.c_uint32),
                ("dist", C.c_uint32), ("zipf_theta", C.c_double), ("hot_frac", C.c_double),
                ("hot_prob", C.c_double), ("shift_every", C.c_uint32)]


class BankStream(C.Structure):
    _fields_ = [("n_txn", C.c_uint32), ("op", C.c_void_p), ("off", C.c_void_p),
                ("addr", C.c_void_p), ("n_addr", C.c_uint64), ("txn_aborts", C.c_void_p),
                ("split_round", C.c_uint32), ("deferred_warps", C.c_uint32),
                ("backoff", C.c_void_p), ("txn_waits", C.c_void_p), ("lock_last", C.c_void_p),
                ("lane_start", C.c_void_p)]


class BankConfig(C.Structure):
    _fields_ = [(n, C.c_uint32) for n in ("n_accounts",)] + [("init_value", C.c_int32)] + [
        (n, C.c_uint32) for n in ("version_depth", "ring_size", "client_warps", "ctas",
                                  "cluster_size", "validate", "writeback", "batch",
                                  "prevalidate", "log_commits", "max_txn", "spin_limit_log2")
    ] + [("device", C.c_int32), ("flow_warps", C.c_uint32), ("max_reads", C.c_uint32),
         ("group_grace", C.c_uint32), ("group_read_wait", C.c_uint32)]


class Stats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in (
        "commits_update", "commits_readonly", "commits_nowrite", "aborts_data_age",
        "aborts_record_age", "aborts_read_write", "aborts_prevalid", "aborts_write_write",
        "sections", "rounds")] + [
        ("final_ts", C.c_uint32), ("error", C.c_uint32), ("kernel_ms", C.c_double),
        ("total_ms", C.c_double)]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_}

    @property
    def commits(self) -> int:
        return self.commits_update + self.commits_readonly + self.commits_nowrite

    @property
    def aborts(self) -> int:
        return (self.aborts_data_age + self.aborts_record_age + self.aborts_read_write +
                self.aborts_prevalid + self.aborts_write_write)

    @property
    def abort_rate(self) -> float:
        """aborts / (aborts + commits), as the reference prints it (bank/csmv_sh/exe.cu:467-471)."""
        tot = self.aborts + self.commits
        return self.aborts / tot if tot else 0.0


class MemcdWorkload(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("n_keys", C.c_uint32), ("n_req", C.c_uint32),
                ("get_pct", C.c_uint32), ("dist", C.c_uint32), ("zipf_theta", C.c_double)]


class MemcdBatch(C.Structure):
    _fields_ = [("n_req", C.c_uint32), ("tick", C.c_uint32), ("kind", C.c_void_p),
                ("key", C.c_void_p), ("val", C.c_void_p), ("found", C.c_void_p),
                ("val_out", C.c_void_p)]


class MemcdConfig(C.Structure):
    _fields_ = [(n, C.c_uint32) for n in (
        "n_sets", "n_ways", "version_depth", "client_warps", "ctas", "batch", "log_commits",
        "max_req", "spin_limit_log2")] + [("device", C.c_int32)]


class TuneTrial(C.Structure):
    _fields_ = [(n, C.c_uint32) for n in ("client_warps", "ctas", "version_depth", "runs")] + [
        ("status", C.c_int32), ("tx_per_s", C.c_double), ("abort_rate", C.c_double),
        ("prevalidate", C.c_uint32), ("max_reads", C.c_uint32)]


class TuneResult(C.Structure):
    _fields_ = [("best", BankConfig), ("n_trials", C.c_uint32), ("trials", TuneTrial * 64)]


class MemcdTuneResult(C.Structure):
    _fields_ = [("best", MemcdConfig), ("n_trials", C.c_uint32), ("trials", TuneTrial * 64)]


class ServeConfig(C.Structure):
    _fields_ = [(n, C.c_uint32) for n in ("n_sets", "client_warps", "ctas", "arena_requests",
                                          "max_inflight_sets", "idle_timeout_ms")] + [
        ("device", C.c_int32), ("log_cap", C.c_uint32), ("serial_batches", C.c_uint32)]


class SchedConfig(C.Structure):
    _fields_ = [("n_accounts", C.c_uint32), ("max_txn", C.c_uint32),
                ("probe_rounds_pct", C.c_uint32), ("probe_every", C.c_uint32),
                ("train_steps", C.c_uint32),
                ("lr", C.c_float), ("threshold", C.c_float), ("defer_threshold", C.c_float),
                ("deferred_warps", C.c_uint32), ("serial_lane", C.c_uint32),
                ("seed", C.c_uint64), ("device", C.c_int32), ("plan", C.c_uint32),
                ("hot_count", C.c_uint32), ("score", C.c_uint32), ("backoff_ns", C.c_uint32),
                ("hot_last", C.c_uint32), ("key_written", C.c_uint32), ("hot_lanes", C.c_uint32)]


class SchedReport(C.Structure):
    _fields_ = [("probe", Stats), ("planned", Stats), ("serial", Stats), ("loss", C.c_float),
                ("n_probe", C.c_uint32), ("n_planned", C.c_uint32), ("n_flagged", C.c_uint32),
                ("n_deferred_rounds", C.c_uint32), ("n_serial", C.c_uint32),
                ("train_ms", C.c_double), ("plan_ms", C.c_double)]

    @property
    def commits(self) -> int:
        return self.probe.commits + self.planned.commits + self.serial.commits

    @property
    def aborts(self) -> int:
        return self.probe.aborts + self.planned.aborts + self.serial.aborts

    @property
    def kernel_ms(self) -> float:
        return self.probe.kernel_ms + self.planned.kernel_ms + self.serial.kernel_ms


_lib = None


def lib() -> C.CDLL:
    """Load libcsmv.so (raises when it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is missing: build it with csmv_gb300.build.build() "
                           "(the CSMV path has no CPU fallback)")
    L = C.CDLL(str(LIB_PATH))
    P, U32, I32 = C.c_void_p, C.c_uint32, C.c_int
    sigs = {
        "csmv_bank_config_default": (None, [C.POINTER(BankConfig)]),
        "csmv_bank_stream_size": (I32, [C.POINTER(BankWorkload), C.POINTER(C.c_uint64)]),
        "csmv_bank_generate": (I32, [C.POINTER(BankWorkload), P, P, P]),
        "csmv_stream_save": (I32, [C.c_char_p, C.POINTER(BankStream)]),
        "csmv_stream_info": (I32, [C.c_char_p, C.POINTER(U32), C.POINTER(C.c_uint64)]),
        "csmv_stream_load": (I32, [C.c_char_p, P, P, P, U32, C.c_uint64]),
        "csmv_log_save": (I32, [C.c_char_p, U32, P, U32, P, P, U32]),
        "csmv_log_info": (I32, [C.c_char_p, C.POINTER(U32), C.POINTER(U32), C.POINTER(U32)]),
        "csmv_log_load": (I32, [C.c_char_p, P, U32, P, P, U32]),
        "csmv_bank_create": (I32, [C.POINTER(BankConfig), C.POINTER(P)]),
        "csmv_bank_load": (I32, [P, P]),
        "csmv_bank_run": (I32, [P, C.POINTER(BankStream), C.POINTER(Stats)]),
        "csmv_bank_run_device": (I32, [P, C.POINTER(BankStream), C.POINTER(Stats)]),
        "csmv_bank_read_values": (I32, [P, P]),
        "csmv_bank_read_versions": (I32, [P, P]),
        "csmv_bank_read_log": (I32, [P, P, U32, P, P, U32]),
        "csmv_bank_read_groups": (I32, [P, P, U32]),
        "csmv_measure_atomics": (I32, [C.c_int32, P]),
        "csmv_bank_device_info": (I32, [P, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                        C.POINTER(C.c_int), C.POINTER(C.c_size_t)]),
        "csmv_bank_destroy": (None, [P]),
        "csmv_memcd_generate": (I32, [C.POINTER(MemcdWorkload), P, P, P]),
        "csmv_memcd_config_default": (None, [C.POINTER(MemcdConfig)]),
        "csmv_memcd_create": (I32, [C.POINTER(MemcdConfig), C.POINTER(P)]),
        "csmv_memcd_clear": (I32, [P]),
        "csmv_memcd_run": (I32, [P, C.POINTER(MemcdBatch), C.POINTER(Stats)]),
        "csmv_memcd_run_device": (I32, [P, C.POINTER(MemcdBatch), C.POINTER(Stats)]),
        "csmv_memcd_read_table": (I32, [P, P, P]),
        "csmv_memcd_read_log": (I32, [P, P, U32, P, U32, C.POINTER(C.c_uint32)]),
        "csmv_memcd_device_info": (I32, [P, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                         C.POINTER(C.c_int), C.POINTER(C.c_size_t)]),
        "csmv_memcd_destroy": (None, [P]),
        "csmv_mlp_create": (I32, [C.c_int32, C.c_uint64, C.POINTER(P)]),
        "csmv_mlp_set_params": (I32, [P, P]),
        "csmv_mlp_get_params": (I32, [P, P]),
        "csmv_mlp_forward": (I32, [P, U32, P, P]),
        "csmv_mlp_grad": (I32, [P, U32, P, P, C.POINTER(C.c_float)]),
        "csmv_mlp_get_grads": (I32, [P, P]),
        "csmv_mlp_adam_step": (I32, [P, C.c_float]),
        "csmv_mlp_destroy": (None, [P]),
        "csmv_bank_autotune": (I32, [C.POINTER(BankConfig), C.POINTER(BankStream), P, U32,
                                     C.POINTER(TuneResult)]),
        "csmv_memcd_autotune": (I32, [C.POINTER(MemcdConfig), C.POINTER(MemcdBatch),
                                      C.POINTER(MemcdBatch), U32, C.POINTER(MemcdTuneResult)]),
        "csmv_serve_config_default": (None, [C.POINTER(ServeConfig)]),
        "csmv_serve_create": (I32, [C.POINTER(ServeConfig), C.POINTER(P)]),
        "csmv_serve_start": (I32, [P]),
        "csmv_serve_submit": (I32, [P, C.POINTER(MemcdBatch), C.POINTER(C.c_uint64)]),
        "csmv_serve_poll": (I32, [P, C.c_uint64, C.POINTER(C.c_uint32), P, P,
                                  C.POINTER(C.c_uint64)]),
        "csmv_serve_poll_logged": (I32, [P, C.c_uint64, C.POINTER(C.c_uint32), P, P, P,
                                         C.POINTER(C.c_uint64)]),
        "csmv_serve_read_log": (I32, [P, P, C.c_uint32, C.POINTER(C.c_uint32),
                                      C.POINTER(C.c_uint32)]),
        "csmv_serve_stop": (I32, [P, C.POINTER(Stats)]),
        "csmv_serve_read_table": (I32, [P, P, P]),
        "csmv_serve_destroy": (None, [P]),
        "csmv_sched_config_default": (None, [C.POINTER(SchedConfig)]),
        "csmv_sched_create": (I32, [C.POINTER(SchedConfig), C.POINTER(P)]),
        "csmv_sched_run": (I32, [P, P, C.POINTER(BankStream), C.POINTER(SchedReport)]),
        "csmv_sched_probe": (I32, [P, P, C.POINTER(BankStream), C.POINTER(SchedReport)]),
        "csmv_sched_plan_run": (I32, [P, P, C.POINTER(BankStream), C.POINTER(SchedReport)]),
        "csmv_sched_serial_run": (I32, [P, P, C.POINTER(BankStream), C.POINTER(SchedReport)]),
        "csmv_bank_run_serial_device": (I32, [P, C.POINTER(BankStream), C.POINTER(Stats)]),
        "csmv_bank_run_flow_device": (I32, [P, C.POINTER(BankStream), C.POINTER(Stats)]),
        "csmv_bank_run_baseline_device": (I32, [P, C.POINTER(BankStream), C.POINTER(Stats)]),
        "csmv_sched_read_plan": (I32, [P, P, U32, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
        "csmv_sched_mlp": (P, [P]),
        "csmv_sched_destroy": (None, [P]),
        "csmv_pinned_alloc": (I32, [C.c_size_t, C.POINTER(P)]),
        "csmv_pinned_free": (None, [P]),
        "csmv_last_error": (C.c_char_p, []),
        "csmv_status_str": (C.c_char_p, [I32]),
        "csmv_abi_version": (I32, []),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _check(st: int, where: str) -> None:
    if st != 0:
        raise CsmvError(st, where, lib().csmv_last_error().decode(errors="replace"))


def _ptr(a: np.ndarray) -> int:
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


# ---------------------------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------------------------

def bank_workload(n_accounts: int, n_txn: int, *, seed: int = 1, pr_read_pct: int = 10,
                  ro_reads: int = 8, up_reads: int = 2, kind: int = KIND_TRANSFER,
                  amt_lo: int = 1, amt_hi: int = 10, dist: int = DIST_UNIFORM,
                  zipf_theta: float = 0.99, hot_frac: float = 0.01, hot_prob: float = 0.9,
                  shift_every: int = 1 << 20) -> BankWorkload:
    return BankWorkload(seed, n_accounts, n_txn, pr_read_pct, ro_reads, up_reads, kind, amt_lo,
                        amt_hi, dist, zipf_theta, hot_frac, hot_prob, shift_every)


@dataclass
class Stream:
    op: np.ndarray
    off: np.ndarray
    addr: np.ndarray

    @property
    def n_txn(self) -> int:
        return int(self.op.shape[0])

    def c_struct(self) -> BankStream:
        return BankStream(self.n_txn, _ptr(self.op), _ptr(self.off), _ptr(self.addr),
                          int(self.addr.shape[0]))


class PinnedArray:
    """numpy view over page-locked host memory (freed with the object)."""

    def __init__(self, n: int, dtype=np.uint32):
        self.dtype = np.dtype(dtype)
        p = C.c_void_p()
        _check(lib().csmv_pinned_alloc(max(1, n) * self.dtype.itemsize, C.byref(p)),
               "csmv_pinned_alloc")
        self._p = p
        buf = (C.c_char * (max(1, n) * self.dtype.itemsize)).from_address(p.value)
        self.array = np.frombuffer(buf, dtype=self.dtype)[:n]

    def __del__(self):
        if getattr(self, "_p", None) is not None and _lib is not None:
            _lib.csmv_pinned_free(self._p)
            self._p = None


def generate(w: BankWorkload, pinned: bool = False) -> Stream:
    """Host generator of the library (csmv_bank_generate)."""
    n_addr = C.c_uint64()
    _check(lib().csmv_bank_stream_size(C.byref(w), C.byref(n_addr)), "csmv_bank_stream_size")
    if pinned:
        holders = [PinnedArray(w.n_txn), PinnedArray(w.n_txn), PinnedArray(n_addr.value)]
        op, off, addr = (h.array for h in holders)
    else:
        holders = []
        op = np.empty(w.n_txn, np.uint32)
        off = np.empty(w.n_txn, np.uint32)
        addr = np.empty(n_addr.value, np.uint32)
    _check(lib().csmv_bank_generate(C.byref(w), _ptr(op), _ptr(off), _ptr(addr)),
           "csmv_bank_generate")
    s = Stream(op, off, addr)
    s._holders = holders  # keep pinned memory alive
    return s


def save_stream(path, s: Stream) -> None:
    """Write a host stream to a stream file (csmv_stream_save)."""
    op, off, addr = (np.ascontiguousarray(a, np.uint32) for a in (s.op, s.off, s.addr))
    bs = BankStream(int(op.shape[0]), _ptr(op), _ptr(off), _ptr(addr), int(addr.shape[0]))
    _check(lib().csmv_stream_save(os.fsencode(path), C.byref(bs)), "csmv_stream_save")


def load_stream(path) -> Stream:
    """Read a stream file (csmv_stream_info + csmv_stream_load)."""
    n_txn, n_addr = C.c_uint32(), C.c_uint64()
    _check(lib().csmv_stream_info(os.fsencode(path), C.byref(n_txn), C.byref(n_addr)),
           "csmv_stream_info")
    op = np.empty(n_txn.value, np.uint32)
    off = np.empty(n_txn.value, np.uint32)
    addr = np.empty(n_addr.value, np.uint32)
    _check(lib().csmv_stream_load(os.fsencode(path), _ptr(op), _ptr(off), _ptr(addr),
                                  n_txn.value, n_addr.value), "csmv_stream_load")
    return Stream(op, off, addr)


def save_log(path, base_ts: int, log_txn, outcome, result) -> None:
    """Write a run's commit log (csmv_log_save)."""
    lt = np.ascontiguousarray(log_txn, np.uint32)
    oc = np.ascontiguousarray(outcome, np.uint32)
    rs = np.ascontiguousarray(result, np.int32)
    assert oc.shape == rs.shape
    _check(lib().csmv_log_save(os.fsencode(path), base_ts, _ptr(lt), int(lt.shape[0]), _ptr(oc),
                               _ptr(rs), int(oc.shape[0])), "csmv_log_save")


def load_log(path):
    """Read a commit-log file: (base_ts, log_txn, outcome, result)."""
    n_txn, n_log, base = C.c_uint32(), C.c_uint32(), C.c_uint32()
    _check(lib().csmv_log_info(os.fsencode(path), C.byref(n_txn), C.byref(n_log), C.byref(base)),
           "csmv_log_info")
    lt = np.empty(n_log.value, np.uint32)
    oc = np.empty(n_txn.value, np.uint32)
    rs = np.empty(n_txn.value, np.int32)
    _check(lib().csmv_log_load(os.fsencode(path), _ptr(lt), n_log.value, _ptr(oc), _ptr(rs),
                               n_txn.value), "csmv_log_load")
    return base.value, lt, oc, rs


# ---------------------------------------------------------------------------------------------
# bank engine
# ---------------------------------------------------------------------------------------------

def bank_config(**kw) -> BankConfig:
    cfg = BankConfig()
    lib().csmv_bank_config_default(C.byref(cfg))
    for k, v in kw.items():
        if not hasattr(cfg, k):
            raise KeyError(f"unknown bank config field {k}")
        setattr(cfg, k, v)
    return cfg


class Bank:
    """One CSMV bank instance on one GPU (TXInit ... TXEnd of the reference)."""

    def __init__(self, cfg: BankConfig | None = None, **kw):
        self.cfg = cfg if cfg is not None else bank_config(**kw)
        h = C.c_void_p()
        _check(lib().csmv_bank_create(C.byref(self.cfg), C.byref(h)), "csmv_bank_create")
        self._h = h
        self.last_stats: Stats | None = None

    def close(self) -> None:
        if getattr(self, "_h", None) is not None:
            lib().csmv_bank_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def load(self, values: np.ndarray | None = None) -> None:
        if values is not None:
            values = np.ascontiguousarray(values, dtype=np.int32)
            assert values.shape[0] == self.cfg.n_accounts
        _check(lib().csmv_bank_load(self._h, _ptr(values) if values is not None else None),
               "csmv_bank_load")

    def run(self, stream: Stream, txn_aborts: np.ndarray | None = None, split_round: int = 0,
            deferred_warps: int = 0, backoff: np.ndarray | None = None,
            txn_waits: np.ndarray | None = None, lock_last: np.ndarray | None = None,
            lane_start: np.ndarray | None = None) -> Stats:
        """Host buffers in: copies the stream to the device inside the call. txn_aborts (uint32
        [n_txn]) receives each transaction's failed attempts; split_round/deferred_warps set
        up the deferred queue; backoff (uint32 [n_txn], ns) bounds each transaction's pause
        before a retry; lock_last (uint8 [n_accounts]) gives group commit's heat classes;
        lane_start (uint32 [deferred_warps + 1]) cuts the deferred queue into one lane of rounds
        per deferred warp (csmv_bank_stream)."""
        st = Stats()
        s = stream.c_struct()
        if txn_aborts is not None:
            assert txn_aborts.dtype == np.uint32 and txn_aborts.shape[0] >= stream.n_txn
            s.txn_aborts = _ptr(txn_aborts)
        if backoff is not None:
            assert backoff.dtype == np.uint32 and backoff.shape[0] >= stream.n_txn
            s.backoff = _ptr(backoff)
        if txn_waits is not None:
            assert txn_waits.dtype == np.uint32 and txn_waits.shape[0] >= stream.n_txn
            s.txn_waits = _ptr(txn_waits)
        if lock_last is not None:
            assert lock_last.dtype == np.uint8 and lock_last.shape[0] == self.cfg.n_accounts
            s.lock_last = _ptr(lock_last)
        if lane_start is not None:
            lane_start = np.ascontiguousarray(lane_start, np.uint32)
            assert lane_start.shape[0] == deferred_warps + 1
            s.lane_start = _ptr(lane_start)
        s.split_round, s.deferred_warps = split_round, deferred_warps
        rc = lib().csmv_bank_run(self._h, C.byref(s), C.byref(st))
        self.last_stats = st
        _check(rc, "csmv_bank_run")
        return st

    def run_device(self, dev_stream: BankStream) -> Stats:
        st = Stats()
        rc = lib().csmv_bank_run_device(self._h, C.byref(dev_stream), C.byref(st))
        self.last_stats = st
        _check(rc, "csmv_bank_run_device")
        return st

    def run_serial_device(self, dev_stream: BankStream) -> Stats:
        """The serial lane: stream order, one warp, exclusive (csmv_bank_run_serial_device)."""
        st = Stats()
        rc = lib().csmv_bank_run_serial_device(self._h, C.byref(dev_stream), C.byref(st))
        self.last_stats = st
        _check(rc, "csmv_bank_run_serial_device")
        return st

    def run_flow_device(self, dev_stream: BankStream) -> Stats:
        """The dataflow lane: the serial lane's results and end state, transactions run as their
        inputs arrive (csmv_bank_run_flow_device)."""
        st = Stats()
        rc = lib().csmv_bank_run_flow_device(self._h, C.byref(dev_stream), C.byref(st))
        self.last_stats = st
        _check(rc, "csmv_bank_run_flow_device")
        return st

    def run_baseline_device(self, dev_stream: BankStream) -> Stats:
        """The reference's naive baseline STM on this bank: snapshot reads, validation against
        commit records, one global commit section (csmv_bank_run_baseline_device)."""
        st = Stats()
        rc = lib().csmv_bank_run_baseline_device(self._h, C.byref(dev_stream), C.byref(st))
        self.last_stats = st
        _check(rc, "csmv_bank_run_baseline_device")
        return st

    def values(self) -> np.ndarray:
        out = np.empty(self.cfg.n_accounts, np.int32)
        _check(lib().csmv_bank_read_values(self._h, _ptr(out)), "csmv_bank_read_values")
        return out

    def versions(self) -> np.ndarray:
        out = np.empty(self.cfg.n_accounts * self.cfg.version_depth, np.uint64)
        _check(lib().csmv_bank_read_versions(self._h, _ptr(out)), "csmv_bank_read_versions")
        return out

    def log(self, n_txn: int, n_commits: int):
        log_txn = np.empty(max(1, n_commits), np.uint32)
        outcome = np.empty(n_txn, np.uint32)
        result = np.empty(n_txn, np.int32)
        _check(lib().csmv_bank_read_log(self._h, _ptr(log_txn), max(1, n_commits), _ptr(outcome),
                                        _ptr(result), n_txn), "csmv_bank_read_log")
        return log_txn[:n_commits], outcome, result

    def groups(self, n_commits: int) -> np.ndarray:
        """Bitmap (uint32 words) of the last run's timestamps that end a commit group."""
        out = np.empty(max(1, (n_commits + 31) // 32), np.uint32)
        _check(lib().csmv_bank_read_groups(self._h, _ptr(out), max(1, n_commits)),
               "csmv_bank_read_groups")
        return out

    def results(self, n_txn: int):
        """Per-transaction outcomes and read-only results of the last run (no commit log)."""
        outcome = np.empty(n_txn, np.uint32)
        result = np.empty(n_txn, np.int32)
        _check(lib().csmv_bank_read_log(self._h, None, 0, _ptr(outcome), _ptr(result), n_txn),
               "csmv_bank_read_log")
        return outcome, result

    def device_info(self) -> dict:
        a, b, c_, d = C.c_int(), C.c_int(), C.c_int(), C.c_size_t()
        _check(lib().csmv_bank_device_info(self._h, C.byref(a), C.byref(b), C.byref(c_),
                                           C.byref(d)), "csmv_bank_device_info")
        return {"n_sms": a.value, "ctas": b.value, "threads_per_cta": c_.value,
                "device_bytes": d.value}


# ---------------------------------------------------------------------------------------------
# transactional cache
# ---------------------------------------------------------------------------------------------

def memcd_workload(n_keys: int, n_req: int, *, seed: int = 1, get_pct: int = 99,
                   dist: int = DIST_ZIPF, zipf_theta: float = 0.99) -> MemcdWorkload:
    return MemcdWorkload(seed, n_keys, n_req, get_pct, dist, zipf_theta)


@dataclass
class Requests:
    kind: np.ndarray   # [n] uint32
    key: np.ndarray    # [n, 4] uint32
    val: np.ndarray    # [n, 8] uint32

    @property
    def n_req(self) -> int:
        return int(self.kind.shape[0])


def memcd_generate(w: MemcdWorkload, pinned: bool = False) -> Requests:
    """Host generator of the library (csmv_memcd_generate)."""
    n = w.n_req
    if pinned:
        holders = [PinnedArray(n), PinnedArray(4 * n), PinnedArray(8 * n)]
        kind, key, val = (h.array for h in holders)
    else:
        holders = []
        kind, key, val = (np.empty(n, np.uint32), np.empty(4 * n, np.uint32),
                          np.empty(8 * n, np.uint32))
    _check(lib().csmv_memcd_generate(C.byref(w), _ptr(kind), _ptr(key), _ptr(val)),
           "csmv_memcd_generate")
    r = Requests(kind, key.reshape(n, 4), val.reshape(n, 8))
    r._holders = holders
    return r


def memcd_config(**kw) -> MemcdConfig:
    cfg = MemcdConfig()
    lib().csmv_memcd_config_default(C.byref(cfg))
    for k, v in kw.items():
        if not hasattr(cfg, k):
            raise KeyError(f"unknown memcd config field {k}")
        setattr(cfg, k, v)
    return cfg


class Memcd:
    """One transactional cache on one GPU. ``run`` is one iteration of the reference's batch
    loop; the LRU tick starts at 1 and advances after every batch (memcdSH.cu:573,648)."""

    def __init__(self, cfg: MemcdConfig | None = None, **kw):
        self.cfg = cfg if cfg is not None else memcd_config(**kw)
        h = C.c_void_p()
        _check(lib().csmv_memcd_create(C.byref(self.cfg), C.byref(h)), "csmv_memcd_create")
        self._h = h
        self.tick = 1
        self.last_stats: Stats | None = None
        self.clear()

    def close(self) -> None:
        if getattr(self, "_h", None) is not None:
            lib().csmv_memcd_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def clear(self) -> None:
        _check(lib().csmv_memcd_clear(self._h), "csmv_memcd_clear")
        self.tick = 1

    def run(self, req: Requests, found: np.ndarray | None = None,
            val_out: np.ndarray | None = None, tick: int | None = None):
        """Host buffers in and out; returns (found, val_out, stats)."""
        n = req.n_req
        found = np.empty(n, np.uint32) if found is None else found
        val_out = np.empty((n, 8), np.uint32) if val_out is None else val_out
        t = self.tick if tick is None else tick
        b = MemcdBatch(n, t, _ptr(req.kind), _ptr(req.key), _ptr(req.val), _ptr(found),
                       _ptr(val_out))
        st = Stats()
        rc = lib().csmv_memcd_run(self._h, C.byref(b), C.byref(st))
        self.last_stats = st
        _check(rc, "csmv_memcd_run")
        if tick is None:
            self.tick += 1
        return found, val_out, st

    def run_device(self, batch: MemcdBatch) -> Stats:
        st = Stats()
        rc = lib().csmv_memcd_run_device(self._h, C.byref(batch), C.byref(st))
        self.last_stats = st
        _check(rc, "csmv_memcd_run_device")
        return st

    def table(self):
        """(tags [n_sets*16] uint64, recs [n_sets*16, 16] uint32)."""
        nv = self.cfg.n_sets * MEMCD_WAYS * MEMCD_DEPTH
        tags = np.empty(nv, np.uint64)
        recs = np.empty((nv, 16), np.uint32)
        _check(lib().csmv_memcd_read_table(self._h, _ptr(tags), _ptr(recs)),
               "csmv_memcd_read_table")
        return tags, recs

    def log(self, n_req: int):
        """(log_txn, outcome[n_req], base_ts) of the last run: log_txn[k] is the request that
        committed with timestamp base_ts + k + 1 (HOLE for a failed validation)."""
        base = C.c_uint32()
        _check(lib().csmv_memcd_read_log(self._h, None, 0, None, 0, C.byref(base)),
               "csmv_memcd_read_log")
        n_log = self.last_stats.final_ts - base.value
        log_txn = np.empty(max(1, n_log), np.uint32)
        outcome = np.empty(max(1, n_req), np.uint32)
        _check(lib().csmv_memcd_read_log(self._h, _ptr(log_txn), max(1, n_log), _ptr(outcome),
                                         n_req, C.byref(base)), "csmv_memcd_read_log")
        return log_txn[:n_log], outcome[:n_req], base.value

    def device_info(self) -> dict:
        a, b, c_, d = C.c_int(), C.c_int(), C.c_int(), C.c_size_t()
        _check(lib().csmv_memcd_device_info(self._h, C.byref(a), C.byref(b), C.byref(c_),
                                            C.byref(d)), "csmv_memcd_device_info")
        return {"n_sms": a.value, "ctas": b.value, "threads_per_cta": c_.value,
                "device_bytes": d.value}


# ---------------------------------------------------------------------------------------------
# serving loop
# ---------------------------------------------------------------------------------------------

def serve_config(**kw) -> ServeConfig:
    cfg = ServeConfig()
    lib().csmv_serve_config_default(C.byref(cfg))
    for k, v in kw.items():
        if not hasattr(cfg, k):
            raise KeyError(f"unknown serve config field {k}")
        setattr(cfg, k, v)
    return cfg


class Server:
    """The cache's serving loop (csmv_serve_*): a persistent kernel per session, request
    batches admitted from a mapped host ring as they arrive."""

    def __init__(self, cfg: ServeConfig | None = None, **kw):
        self.cfg = cfg if cfg is not None else serve_config(**kw)
        h = C.c_void_p()
        _check(lib().csmv_serve_create(C.byref(self.cfg), C.byref(h)), "csmv_serve_create")
        self._h = h
        self.tick = 1
        self._sizes = {}

    def close(self) -> None:
        if getattr(self, "_h", None) is not None:
            lib().csmv_serve_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def start(self) -> None:
        _check(lib().csmv_serve_start(self._h), "csmv_serve_start")
        self._sizes = {}

    def submit(self, req: Requests, tick: int | None = None):
        """Batch id, or None when admission refuses it for now (no room)."""
        t = self.tick if tick is None else tick
        b = MemcdBatch(req.n_req, t, _ptr(req.kind), _ptr(req.key), _ptr(req.val), None, None)
        bid = C.c_uint64()
        rc = lib().csmv_serve_submit(self._h, C.byref(b), C.byref(bid))
        if rc == 5:
            return None
        _check(rc, "csmv_serve_submit")
        if tick is None:
            self.tick += 1
        self._sizes[bid.value] = req.n_req
        return bid.value

    def poll(self, batch_id: int, results: bool = True, outcome: bool = False):
        """None while running; else (found, val_out, device_ns) (arrays None if not asked), and
        with outcome=True (log_cap > 0) (found, val_out, outcome, device_ns)."""
        n = self._sizes[batch_id]
        done = C.c_uint32()
        ns = C.c_uint64()
        found = np.empty(n, np.uint32) if results else None
        out = np.empty((n, 8), np.uint32) if results else None
        oc = np.empty(n, np.uint32) if outcome else None
        _check(lib().csmv_serve_poll_logged(self._h, batch_id, C.byref(done),
                                            _ptr(found) if results else None,
                                            _ptr(out) if results else None,
                                            _ptr(oc) if outcome else None, C.byref(ns)),
               "csmv_serve_poll_logged")
        if not done.value:
            return None
        if outcome:
            return found, out, oc, ns.value
        return found, out, ns.value

    def log(self):
        """(log_txn, base_ts) of the last session (log_cap > 0): log_txn[k] is the arena index of
        the request that committed with timestamp base_ts + k + 1 (HOLE for a hole)."""
        used, base = C.c_uint32(), C.c_uint32()
        _check(lib().csmv_serve_read_log(self._h, None, 0, C.byref(used), C.byref(base)),
               "csmv_serve_read_log")
        log = np.empty(max(1, used.value), np.uint32)
        _check(lib().csmv_serve_read_log(self._h, _ptr(log), log.shape[0], C.byref(used),
                                         C.byref(base)), "csmv_serve_read_log")
        return log[:used.value], base.value

    def stop(self) -> Stats:
        st = Stats()
        _check(lib().csmv_serve_stop(self._h, C.byref(st)), "csmv_serve_stop")
        return st

    def table(self):
        nv = self.cfg.n_sets * MEMCD_WAYS * MEMCD_DEPTH
        tags = np.empty(nv, np.uint64)
        recs = np.empty((nv, 16), np.uint32)
        _check(lib().csmv_serve_read_table(self._h, _ptr(tags), _ptr(recs)), "csmv_serve_read_table")
        return tags, recs


def requests_slice(req: Requests, lo: int, hi: int) -> Requests:
    return Requests(np.ascontiguousarray(req.kind[lo:hi]), np.ascontiguousarray(req.key[lo:hi]),
                    np.ascontiguousarray(req.val[lo:hi]))


# ---------------------------------------------------------------------------------------------
# conflict predictor network
# ---------------------------------------------------------------------------------------------

MLP_IN, MLP_HIDDEN, MLP_PARAMS = 64, 128, 24964


class Mlp:
    """The conflict predictor network on one GPU (csmv_mlp_*). Sample arrays are device
    pointers (ints): features bf16 [n][64], labels and outputs fp32 [n]."""

    def __init__(self, seed: int = 1, device: int = 0):
        h = C.c_void_p()
        _check(lib().csmv_mlp_create(device, seed, C.byref(h)), "csmv_mlp_create")
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None) is not None:
            lib().csmv_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def params(self) -> np.ndarray:
        out = np.empty(MLP_PARAMS, np.float32)
        _check(lib().csmv_mlp_get_params(self._h, _ptr(out)), "csmv_mlp_get_params")
        return out

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.shape == (MLP_PARAMS,)
        _check(lib().csmv_mlp_set_params(self._h, _ptr(p)), "csmv_mlp_set_params")

    def grads(self) -> np.ndarray:
        out = np.empty(MLP_PARAMS, np.float32)
        _check(lib().csmv_mlp_get_grads(self._h, _ptr(out)), "csmv_mlp_get_grads")
        return out

    def forward(self, n: int, dev_x: int, dev_p: int) -> None:
        _check(lib().csmv_mlp_forward(self._h, n, dev_x, dev_p), "csmv_mlp_forward")

    def grad(self, n: int, dev_x: int, dev_y: int) -> float:
        loss = C.c_float()
        _check(lib().csmv_mlp_grad(self._h, n, dev_x, dev_y, C.byref(loss)), "csmv_mlp_grad")
        return loss.value

    def adam_step(self, lr: float) -> None:
        _check(lib().csmv_mlp_adam_step(self._h, lr), "csmv_mlp_adam_step")


# ---------------------------------------------------------------------------------------------
# learned conflict scheduler
# ---------------------------------------------------------------------------------------------

def sched_config(**kw) -> SchedConfig:
    cfg = SchedConfig()
    lib().csmv_sched_config_default(C.byref(cfg))
    for k, v in kw.items():
        if not hasattr(cfg, k):
            raise KeyError(f"unknown scheduler config field {k}")
        setattr(cfg, k, v)
    return cfg


class Scheduler:
    """The learned conflict scheduler (csmv_sched_*) in front of a Bank. Chunks are device
    streams (BankStream with device pointers)."""

    def __init__(self, cfg: SchedConfig | None = None, **kw):
        self.cfg = cfg if cfg is not None else sched_config(**kw)
        h = C.c_void_p()
        _check(lib().csmv_sched_create(C.byref(self.cfg), C.byref(h)), "csmv_sched_create")
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None) is not None:
            lib().csmv_sched_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _call(self, name: str, bank: Bank, dev_stream: BankStream) -> SchedReport:
        rep = SchedReport()
        rc = getattr(lib(), name)(self._h, bank._h, C.byref(dev_stream), C.byref(rep))
        bank.last_stats = {"csmv_sched_probe": rep.probe,
                           "csmv_sched_serial_run": rep.serial}.get(name, rep.planned)
        _check(rc, name)
        return rep

    def run(self, bank: Bank, dev_stream: BankStream) -> SchedReport:
        return self._call("csmv_sched_run", bank, dev_stream)

    def probe(self, bank: Bank, dev_stream: BankStream) -> SchedReport:
        return self._call("csmv_sched_probe", bank, dev_stream)

    def plan_run(self, bank: Bank, dev_stream: BankStream) -> SchedReport:
        return self._call("csmv_sched_plan_run", bank, dev_stream)

    def serial_run(self, bank: Bank, dev_stream: BankStream) -> SchedReport:
        return self._call("csmv_sched_serial_run", bank, dev_stream)

    def plan(self, n: int):
        """(perm, probe_rounds, split_round) of the last planned run."""
        perm = np.empty(max(1, n), np.uint32)
        pr, sp = C.c_uint32(), C.c_uint32()
        _check(lib().csmv_sched_read_plan(self._h, _ptr(perm), max(1, n), C.byref(pr), C.byref(sp)),
               "csmv_sched_read_plan")
        n1 = n - 32 * pr.value
        return perm[:n1], pr.value, sp.value


def autotune(stream: Stream, repeats: int = 3, init: np.ndarray | None = None, **base):
    """Pick the engine's launch shape for a workload (csmv_bank_autotune). Returns (best
    BankConfig, list of trial dicts)."""
    cfg = bank_config(**base)
    res = TuneResult()
    s = stream.c_struct()
    init_p = None
    if init is not None:
        init = np.ascontiguousarray(init, dtype=np.int32)
        init_p = _ptr(init)
    _check(lib().csmv_bank_autotune(C.byref(cfg), C.byref(s), init_p, repeats, C.byref(res)),
           "csmv_bank_autotune")
    trials = [{n: getattr(t, n) for n, _ in TuneTrial._fields_} for t in res.trials[:res.n_trials]]
    return res.best, trials


def memcd_autotune(sample: Requests, fill: Requests | None = None, repeats: int = 3,
                   tick: int = 2, **base):
    """Pick the cache's launch shape (csmv_memcd_autotune): `fill` runs first on each fresh
    candidate (tick 1), then `sample` is timed. Returns (best MemcdConfig, trial dicts; tx_per_s
    is requests/s)."""
    cfg = memcd_config(**base)
    res = MemcdTuneResult()
    def batch(r, t):
        return MemcdBatch(r.n_req, t, _ptr(r.kind), _ptr(r.key), _ptr(r.val), None, None)
    fb = batch(fill, 1) if fill is not None else None
    sb = batch(sample, tick)
    _check(lib().csmv_memcd_autotune(C.byref(cfg), C.byref(fb) if fb is not None else None,
                                     C.byref(sb), repeats, C.byref(res)), "csmv_memcd_autotune")
    trials = [{n: getattr(t, n) for n, _ in TuneTrial._fields_} for t in res.trials[:res.n_trials]]
    return res.best, trials


class AtomicRates(C.Structure):
    _fields_ = [("same_word_per_s", C.c_double), ("spread_per_s", C.c_double),
                ("cas_chain_ns", C.c_double), ("kernel_ms", C.c_double)]


def measure_atomics(device: int = 0) -> dict:
    """The device's L2 atomic rates (csmv_measure_atomics)."""
    r = AtomicRates()
    _check(lib().csmv_measure_atomics(device, C.byref(r)), "csmv_measure_atomics")
    return {n: getattr(r, n) for n, _ in AtomicRates._fields_}


def cuda_device_present() -> bool:
    """True when a CUDA device is visible (checked through the library, no torch needed)."""
    try:
        cfg = bank_config(n_accounts=64, max_txn=32, ctas=1, client_warps=1)
        Bank(cfg).close()
        return True
    except CsmvError as e:
        return e.status not in (6,)
    except RuntimeError:
        return False


