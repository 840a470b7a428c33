"""Benchmark of the CSMV commit path on GB300 (contract: one JSON line from rank 0).

Workload (the configuration the headline metric is quoted on): the contended bank at scale -
2^20 int32 accounts at 1000, Zipf(0.99) account choice, transfers that read 4 and write 2
accounts (skipped when funds are short), 20 % read-only rounds summing 32 accounts. The stream
is 2^24 transactions, seeded; a step is one batch of 2^20 consecutive transactions of it
(batch i = transactions [i 2^20, (i+1) 2^20)), so warm-up and timed steps see different
transactions and the account state carries over between steps. Stream arrays are larger than
L2 (28 MB per batch), so no L2 flush is needed between steps.

value = the learned arm: the learned conflict scheduler (csmv_sched_run) in front of the commit
engine in group-commit mode. The scheduler probes 2 % of a batch's rounds in stream order, trains
its network on the probe's conflicts (aborts and lock waits), and reorders and groups the rest:
transfers it flags are sorted by the hot accounts they touch into rounds of 32, each hot
account's rounds spread over the batch, with a per-transaction retry backoff. EVERY transaction
of the batch then goes through the engine: its warp takes the write locks, the CTA's commit
server draws the timestamps, every read of an account the group does not lock is validated, and
the versions are installed - nothing bypasses validation. GPU-resident inputs; wall time of the
step between device synchronisations.
e2e = the same through host buffers: the batch's op/off arrays and address range are copied from
pinned memory inside the timed region, and each run's per-transaction outcomes and read-only
results are copied back.

Comparison arms on the same batches (reported beside the headline, not in it):
  plain              the engine alone in stream order with the reference's commit method
                     (per-transaction validation, intra-warp pre-validation, CTA-batched
                     timestamps: batchedAtrInsert), the method the benchmark spec calls plain
  group_stream       the engine's group commit in stream order, no scheduler
  dataflow_lane      the earlier path: the scheduler deferring flagged transfers to the dataflow
                     lane, which executes them in stream order WITHOUT locks or validation
                     (labelled as such; not CSMV)
Extra sections: "hotspot" (learned vs plain on a shifting hotspot), "uniform", "c1" (the small
bank of the reference's own configuration), "variants" (the engine's validation / batching /
write-back / cluster modes on uniform and Zipf banks), "alternatives" (another STM on the same
batches: the reference's naive JVSTM-style baseline), "memcd", "serving", "atomics" (the L2
atomic rates of the GPU, the engine's roofline).

--impl reference runs the reference arm: the path's CPU execution (the oracle port, striped
locks on every host core) on the same batches, generated by the oracle's own generator.
--case NAME runs one small invocation of one kernel for profiling (engine, group, serial, flow,
mlp, memcd, sched). Multi-GPU: replicas only (no collective on the path); each rank runs its own
instance on its own GPU, value sums the ranks' transactions over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "csmv-gpu-stm_gb300"))

N_ACCOUNTS = 1 << 20
STREAM_TXN = 1 << 24
BATCH = 1 << 20
WORKLOAD = dict(seed=2026, pr_read_pct=20, ro_reads=32, up_reads=4, amt_lo=1, amt_hi=10,
                zipf_theta=0.99)
B_UPDATE = 16 * 4 + 12 * 2   # algorithmic bytes of a transfer: 4 versioned reads, 2 writes
B_RO = 16 * 32               # a 32-account read-only scan
ENGINE = dict(prevalidate=3, max_reads=4)          # group commit, kernels for <= 4 reads
SCHED = dict(plan=1, probe_rounds_pct=2, probe_every=3)
PLAIN = dict(prevalidate=1, max_reads=4)           # the reference's commit method
FLOW = dict(plan=0, serial_lane=2, defer_threshold=0.0, probe_every=3, probe_rounds_pct=2)
TRIPS_PER_HOLD = 4  # dependent L2 round trips of a contended lock's hand-off and hold: the lock
                    # CAS, the timestamp draw, the validation load, the releasing store


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="csmv", choices=["csmv", "reference"])
    ap.add_argument("--batch", type=int, default=BATCH)
    ap.add_argument("--dist", default="zipf", choices=["zipf", "uniform", "hotspot"])
    ap.add_argument("--client-warps", type=int, default=int(os.environ.get("CSMV_CLIENT_WARPS", 1)))
    ap.add_argument("--ctas", type=int, default=int(os.environ.get("CSMV_CTAS", 152)))
    ap.add_argument("--depth", type=int, default=int(os.environ.get("CSMV_DEPTH", 8)))
    ap.add_argument("--case", default=None,
                    choices=["engine", "group", "serial", "flow", "mlp", "memcd", "sched"])
    ap.add_argument("--case-txn", type=int, default=1 << 18)
    ap.add_argument("--no-extras", action="store_true", help="skip the extra sections")
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner (use the flags)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


T_START = time.perf_counter()


def progress(msg: str) -> None:
    print(f"[bench {time.perf_counter() - T_START:7.1f} s] {msg}", file=sys.stderr, flush=True)


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def reduce_max(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device, self.rows, self._stop = device, [], threading.Event()
        self._t = threading.Thread(target=self._run, daemon=True)

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits"], capture_output=True,
                                     text=True, timeout=5).stdout.strip()
                if out:
                    self.rows.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4)
                          if len(r) > 3 + i and r[3 + i].strip() == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(self.rows)}


def peaks():
    try:
        return json.loads((ROOT / "MEASURED_PEAKS.json").read_text()), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def generate_batches(dist: str, batch: int, count: int, pinned: bool = True, seed: int = None,
                     **over):
    """The first `count` batches of a seeded stream (the generator is counter-based, so a prefix
    of the stream holds the same transactions as the whole stream)."""
    import csmv_gb300 as cg
    d = dict(WORKLOAD)
    if seed is not None:
        d["seed"] = seed
    d.update(over)
    dist_id = {"zipf": cg.DIST_ZIPF, "uniform": cg.DIST_UNIFORM, "hotspot": cg.DIST_HOTSPOT}[dist]
    w = cg.bank_workload(N_ACCOUNTS, batch * count, dist=dist_id, kind=cg.KIND_TRANSFER, **d)
    s = cg.generate(w, pinned=pinned)
    return s, [cg.Stream(s.op[i * batch:(i + 1) * batch], s.off[i * batch:(i + 1) * batch], s.addr)
               for i in range(count)]


class DevBatch:
    """A batch's op/off arrays staged in device memory (the address array is shared)."""

    def __init__(self, torch, b):
        self.t = [torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda()
                  for a in (b.op, b.off)]
        self.n = b.n_txn

    def stream(self, cg, addr_dev, n_addr):
        return cg.BankStream(self.n, self.t[0].data_ptr(), self.t[1].data_ptr(),
                             addr_dev.data_ptr(), n_addr)


def launches_learned(rep) -> int:
    """Kernels the scheduler and the engine launched for one chunk (sched_engine.cu, plan 1)."""
    n = 1  # access counts
    if rep.n_probe:
        n += 1 + 1 + 2 + 4  # features, probe engine run, labels + rates, 2 x (grad + adam)
    n += 2 + 2  # features and network forward; read-only flags and scan
    if rep.n_planned:
        # hot flags, 3-kernel scan, keys, 3-kernel scan, cold flags, 3-kernel scan, scatter,
        # round buckets, 3-kernel scan, round scatter, expand, read-only list, emit, backoff
        n += 1 + 3 + 1 + 3 + 1 + 3 + 1 + 1 + 3 + 1 + 1 + 1 + 1 + 1
        n += 1 if rep.planned.commits else 0  # the planned engine run
    return n


def new_bank(cg, args, local, max_txn, **over):
    kw = dict(n_accounts=N_ACCOUNTS, version_depth=args.depth, client_warps=args.client_warps,
              ctas=args.ctas, max_txn=max_txn, log_commits=1, device=local, **ENGINE)
    kw.update(over)
    bank = cg.Bank(**kw)
    bank.load()
    return bank


def plan_lock_rounds(op, off, addr, order):
    """Largest number of rounds (32 consecutive transactions of `order`) that write one account:
    the length of the busiest account's lock chain in this plan."""
    n = (len(order) // 32) * 32
    o = np.asarray(order[:n]).reshape(-1, 32)
    upd = (op[o[:, 0]] & 3) != 0
    o = o[upd]
    w = np.stack([addr[off[o]], addr[off[o] + 1]], 2).reshape(o.shape[0], 64).astype(np.int64)
    w.sort(axis=1)
    first = np.ones_like(w, dtype=bool)
    first[:, 1:] = w[:, 1:] != w[:, :-1]
    counts = np.bincount(w[first], minlength=1)
    top = int(np.argmax(counts))
    return int(counts[top]), top, int(o.shape[0])


# ---------------------------------------------------------------------------------------------
# arms
# ---------------------------------------------------------------------------------------------

def run_engine(cg, dev, addr_dev, n_addr, args, local, batches, **over):
    """The engine alone on device batches (stream order); device time from the engine's events."""
    bank = new_bank(cg, args, local, args.batch, **over)
    res = dict(ms=0.0, commits=0, aborts=0, ro=0, upd=0, steps=0)
    for j, i in enumerate(batches):
        st = bank.run_device(dev[i].stream(cg, addr_dev, n_addr))
        if j == 0:
            continue  # warm-up
        res["ms"] += st.kernel_ms
        res["commits"] += st.commits
        res["aborts"] += st.aborts
        res["ro"] += st.commits_readonly
        res["upd"] += st.commits_update + st.commits_nowrite
        res["steps"] += 1
    info = bank.device_info()
    bank.close()
    res["tx_s"] = res["commits"] / (res["ms"] * 1e-3) if res["ms"] else 0.0
    res["abort_rate"] = res["aborts"] / max(1, res["aborts"] + res["commits"])
    return res, info


def run_learned(torch, cg, dev, addr_dev, n_addr, args, local, warm, timed, sched_cfg=SCHED,
                bank_over=None):
    bank = new_bank(cg, args, local, args.batch, **(bank_over or {}))
    sched = cg.Scheduler(n_accounts=N_ACCOUNTS, max_txn=args.batch, device=local, **sched_cfg)
    res = dict(wall=0.0, commits=0, aborts=0, launches=0, plan_ms=0.0, train_ms=0.0,
               engine_ms=0.0, serial_ms=0.0, serial_txn=0, flagged=0, ww=0, rw=0, age=0,
               device_ms=0.0, rounds=0)
    last = None
    for i in range(warm + timed):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rep = sched.run(bank, dev[i].stream(cg, addr_dev, n_addr))
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        if i >= warm:
            res["wall"] += dt
            res["commits"] += rep.commits
            res["aborts"] += rep.aborts
            res["launches"] += launches_learned(rep)
            res["plan_ms"] += rep.plan_ms
            res["train_ms"] += rep.train_ms
            res["engine_ms"] += rep.probe.kernel_ms + rep.planned.kernel_ms
            res["serial_ms"] += rep.serial.kernel_ms
            res["serial_txn"] += rep.n_serial
            res["flagged"] += rep.n_flagged
            res["device_ms"] += rep.kernel_ms + rep.plan_ms + rep.train_ms
            res["rounds"] += rep.probe.rounds + rep.planned.rounds
            for part in (rep.probe, rep.planned):
                res["ww"] += part.aborts_write_write
                res["rw"] += part.aborts_read_write
                res["age"] += part.aborts_data_age
            last = (i, rep)
    i, rep = last
    perm, probe_rounds, _ = sched.plan(dev[i].n)
    sched.close()
    bank.close()
    res["tx_s"] = res["commits"] / res["wall"]
    res["abort_rate"] = res["aborts"] / max(1, res["aborts"] + res["commits"])
    res["last_plan"] = (i, perm)
    return res


def tune_learned(torch, cg, dev, addr_dev, n_addr, args, local):
    """Client warps per CTA x versions per account for the learned arm: each candidate runs the
    whole arm (probe, plan, group commit) on batch 0 (warm-up) and batch 1 (timed); the fastest
    is kept in args. The grid stays one CTA per SM (at most 15 client warps beside the commit
    server in its 512 threads)."""
    trials = []
    for cw, depth in ((2, 8), (4, 8), (8, 8), (12, 8), (15, 8), (12, 4)):
        args.client_warps, args.depth = cw, depth
        r = run_learned(torch, cg, dev, addr_dev, n_addr, args, local, 1, 1)
        trials.append({"client_warps": cw, "version_depth": depth, "tx_s": r["tx_s"]})
    best = max(trials, key=lambda t: t["tx_s"])
    args.client_warps, args.depth = best["client_warps"], best["version_depth"]
    return {"client_warps": best["client_warps"], "ctas": args.ctas,
            "version_depth": best["version_depth"], "trials": trials,
            "sample": "the learned arm on batches 0 (warm-up) and 1"}


def e2e_learned(torch, cg, host, s_addr, args, local, warm, timed):
    """Host buffers through the public calls: each step copies the batch's op/off arrays and its
    range of the address array from pinned host memory, runs the scheduler's probe and planned
    runs, and copies every transaction's outcome and read-only result back to the host; timed on
    the host clock."""
    bank = new_bank(cg, args, local, args.batch)
    sched = cg.Scheduler(n_accounts=N_ACCOUNTS, max_txn=args.batch, device=local, **SCHED)
    n = args.batch
    d_op = torch.empty(n, dtype=torch.int32, device="cuda")
    d_off = torch.empty(n, dtype=torch.int32, device="cuda")
    d_addr = torch.empty(s_addr.shape[0], dtype=torch.int32, device="cuda")
    h_addr = torch.from_numpy(s_addr.view(np.int32))
    commits, wall, h2d, d2h, checksum = 0, 0.0, 0, 0, 0
    for i in range(warm + timed):
        b = host[i]
        lo = int(b.off[0])
        hi = int(b.off[-1]) + int((b.op[-1] >> 2) & 63)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        d_op.copy_(torch.from_numpy(b.op.view(np.int32)), non_blocking=True)
        d_off.copy_(torch.from_numpy(b.off.view(np.int32)), non_blocking=True)
        d_addr[lo:hi].copy_(h_addr[lo:hi], non_blocking=True)
        torch.cuda.synchronize()
        ds = cg.BankStream(n, d_op.data_ptr(), d_off.data_ptr(), d_addr.data_ptr(),
                           int(s_addr.shape[0]))
        r1 = sched.probe(bank, ds)
        out_bytes = 0
        if r1.n_probe:
            o1, res1 = bank.results(r1.n_probe)
            out_bytes += o1.nbytes + res1.nbytes
            checksum ^= int(res1.view(np.uint32).sum(dtype=np.uint64))
        r2 = sched.plan_run(bank, ds)
        o2, res2 = bank.results(r2.n_planned)
        out_bytes += o2.nbytes + res2.nbytes
        checksum ^= int(res2.view(np.uint32).sum(dtype=np.uint64))
        dt = time.perf_counter() - t0
        if i >= warm:
            wall += dt
            commits += r1.probe.commits + r2.planned.commits
            h2d += b.op.nbytes + b.off.nbytes + (hi - lo) * 4
            d2h += out_bytes + 2 * 80  # results and the two runs' statistics
    sched.close()
    bank.close()
    return commits, wall, h2d // max(1, timed), d2h // max(1, timed)


def hotspot_section(torch, cg, args, local):
    """Learned vs plain on the shifting hotspot: batches of 2^20 transactions. Arms: plain (the
    reference's commit method, stream order), group commit in stream order, the learned
    scheduler with group commit (probing and training on every third chunk, as in the headline
    arm), and two ablations of it (the raw sketch-count score instead of the network; no
    backoff); tx/s on the host clock with planning and training included."""
    chunk, count = 1 << 20, 6
    s, bs = generate_batches("hotspot", chunk, count, pinned=False, seed=3, pr_read_pct=10,
                             ro_reads=8, up_reads=2, hot_frac=0.01, hot_prob=0.3,
                             shift_every=1 << 20)
    addr = torch.from_numpy(s.addr.view(np.int32)).cuda()
    dev = [DevBatch(torch, b) for b in bs]
    out = {}
    probe = dict(probe_rounds_pct=SCHED["probe_rounds_pct"], probe_every=SCHED["probe_every"])
    for arm, over, learned in (("plain", PLAIN, False), ("group_stream", ENGINE, False),
                               ("learned", ENGINE, probe),
                               ("learned_sketch_score", ENGINE, dict(probe, score=1)),
                               ("learned_no_backoff", ENGINE, dict(probe, backoff_ns=0))):
        bank = cg.Bank(n_accounts=N_ACCOUNTS, version_depth=8, client_warps=2, ctas=152,
                       max_txn=chunk, log_commits=0, device=local, **over)
        bank.load()
        sched = cg.Scheduler(n_accounts=N_ACCOUNTS, max_txn=chunk, device=local, plan=1,
                             **learned) if learned is not False else None
        c = a = 0
        t = 0.0
        for j, d in enumerate(dev):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            if sched is None:
                st = bank.run_device(d.stream(cg, addr, s.addr.shape[0]))
                c, a = c + st.commits, a + st.aborts
            else:
                r = sched.run(bank, d.stream(cg, addr, s.addr.shape[0]))
                c, a = c + r.commits, a + r.aborts
            torch.cuda.synchronize()
            if j == 0:  # warm-up
                c = a = 0
                continue
            t += time.perf_counter() - t0
        if sched is not None:
            sched.close()
        bank.close()
        out[arm] = {"tx_s": c / t, "abort_rate": a / (a + c)}
    out["workload"] = ("2^20 accounts, 1% hot set drawing 30% of the accesses, moving every 2^20 "
                       "txn; 90% 2-account transfers, 10% read-only sums of 8; batches of 2^20, "
                       "one warm-up and 5 timed")
    return out


def uniform_section(torch, cg, args, local):
    s, bs = generate_batches("uniform", args.batch, 4, pinned=False)
    addr = torch.from_numpy(s.addr.view(np.int32)).cuda()
    dev = [DevBatch(torch, b) for b in bs]
    out = {}
    for name, over in (("plain", PLAIN), ("group_commit", ENGINE)):
        res, _ = run_engine(cg, dev, addr, s.addr.shape[0], args, local, [0, 1, 2, 3],
                            log_commits=0, **over)
        out[name] = {"tx_s": res["tx_s"], "abort_rate": res["abort_rate"]}
    out["workload"] = "same bank, uniform account choice, engine alone, 3 batches of 2^20"
    return out


def alternatives_section(torch, cg, dev, addr_dev, n_addr, args, local):
    """Another STM on the same batches: the reference's naive baseline (bank/baseline, JVSTM
    style: snapshot reads, validation against the commit records written since, one global
    commit section; csmv_bank_run_baseline_device) on the Zipf bench batches and on uniform
    batches; committed tx/s on device time and abort rate, at the learned arm's launch shape.
    Each runs a warm-up on 2^12 transactions of its first batch, then a prefix of each later
    batch sized to about half a second at the warm-up's rate (at most the whole batch)."""
    def run(batches, addr, n_a, order):
        bank = new_bank(cg, args, local, args.batch, log_commits=0)

        def prefix(b, n):
            return cg.BankStream(n, b.t[0].data_ptr(), b.t[1].data_ptr(), addr.data_ptr(), n_a)
        st = bank.run_baseline_device(prefix(batches[order[0]], 1 << 12))
        rate = st.commits / max(st.kernel_ms * 1e-3, 1e-6)
        n = min(batches[order[0]].n, max(1 << 12, int(rate * 0.5) // 32 * 32))
        ms = commits = aborts = 0
        for i in order[1:]:
            st = bank.run_baseline_device(prefix(batches[i], n))
            ms += st.kernel_ms
            commits += st.commits
            aborts += st.aborts
        bank.close()
        return {"tx_s": commits / (ms * 1e-3), "abort_rate": aborts / max(1, aborts + commits),
                "txn_per_batch": n}

    out = {"method": "the reference's naive baseline STM (no commit server; validation against "
                     "commit records; one global commit section, taken once per warp)",
           "workload": "2^20 accounts r4/w2, 20% read-only scans of 32, batches of 2^20; "
                       f"{args.client_warps} client warps x {args.ctas} CTAs, depth {args.depth}"}
    out["zipf"] = run(dev, addr_dev, n_addr, [0, 1])
    s, bs = generate_batches("uniform", args.batch, 3, pinned=False)
    addr = torch.from_numpy(s.addr.view(np.int32)).cuda()
    out["uniform"] = run([DevBatch(torch, b) for b in bs], addr, int(s.addr.shape[0]), [0, 1, 2])
    return out


def c1_section(cg, local):
    """The small bank of the reference's configuration: 4096 accounts at 1000, 8 blocks x 128
    client threads, 256 transactions per thread (90 % two-account transfers of 1..10, 10 %
    read-only sums of 8), version depth 4; host buffers, device time of the commit kernel."""
    n = 8 * 128 * 256
    w = cg.bank_workload(4096, n, seed=1, pr_read_pct=10, ro_reads=8, up_reads=2,
                         kind=cg.KIND_TRANSFER, amt_lo=1, amt_hi=10, dist=cg.DIST_UNIFORM)
    s = cg.generate(w)
    out = {"workload": "4096 accounts, 8 x 128 client threads x 256 txn, 90/10, depth 4"}
    for name, over in (("plain", dict(prevalidate=1)), ("group_commit", dict(prevalidate=3))):
        with cg.Bank(n_accounts=4096, version_depth=4, ctas=8, client_warps=4, max_txn=n,
                     log_commits=0, device=local, **over) as bank:
            ms = []
            for _ in range(4):
                bank.load()
                st = bank.run(s)
                ms.append(st.kernel_ms)
            ms = sorted(ms[1:])[1]
            out[name] = {"tx_s": n / (ms * 1e-3), "abort_rate": st.abort_rate, "kernel_ms": ms}
    # the same stream on the whole GPU: the autotuner's launch shape and commit method
    best, trials = cg.autotune(s, repeats=2, n_accounts=4096, init_value=1000, device=local,
                               max_txn=n)
    with cg.Bank(best) as bank:
        ms = []
        for _ in range(4):
            bank.load()
            st = bank.run(s)
            ms.append(st.kernel_ms)
        ms = sorted(ms[1:])[1]
    out["tuned"] = {"tx_s": n / (ms * 1e-3), "abort_rate": st.abort_rate, "kernel_ms": ms,
                    "client_warps": best.client_warps, "ctas": best.ctas,
                    "version_depth": best.version_depth, "prevalidate": best.prevalidate,
                    "max_reads": best.max_reads, "candidates": len(trials)}
    return out


VARIANT_CELLS = {
    "stamp-cta-prevalidate": dict(validate=0, batch=2, prevalidate=1),
    "stamp-warp-prevalidate": dict(validate=0, batch=1, prevalidate=1),
    "stamp-lane-serverwb": dict(validate=0, batch=0, writeback=1, prevalidate=1),
    "stamp-cta-chain": dict(validate=0, batch=2, prevalidate=2),
    "stamp-cta-group": dict(validate=0, batch=2, prevalidate=3),
    "stamp-cluster2": dict(validate=0, batch=3, cluster_size=2, prevalidate=1),
    "stamp-cluster4": dict(validate=0, batch=3, cluster_size=4, prevalidate=1),
    "stamp-cluster8": dict(validate=0, batch=3, cluster_size=8, prevalidate=1),
    "stamp-cluster2-group": dict(validate=0, batch=3, cluster_size=2, prevalidate=3),
    "ring-cta-client": dict(validate=1, batch=2, prevalidate=1),
    "ring-warp-serverwb": dict(validate=1, batch=1, writeback=1, prevalidate=1),
    "ring-lane-serverwb": dict(validate=1, batch=0, writeback=1, prevalidate=1),
    "ringlane-warp-client": dict(validate=2, batch=1, prevalidate=1),
    "ringlane-cta-client": dict(validate=2, batch=2, prevalidate=1),
}


def variants_section(cg, local):
    """The engine's commit variants (the reference's sh / gb / ts storage forms map to the stamp
    and ring protocols and the cluster form; vanilla / batchedAtrInsert / clientWriteback /
    collabValidation to lane / warp / CTA batches, server write-back and the collaborative ring
    scan) on the uniform bank (2^18 transactions) and the Zipf bank (2^15): committed tx/s
    (device time) and abort rate per cell, 2 client warps per CTA, depth 8, host buffers."""
    out = {"workload": "2^20 accounts r4/w2, 20% read-only scans of 32; uniform 2^18 txn, "
                       "Zipf(0.99) 2^15 txn; 2 client warps x 152 CTAs (clusters: 4 warps)"}
    for dist, n in (("uniform", 1 << 18), ("zipf", 1 << 15)):
        s, bs = generate_batches(dist, n, 2, pinned=False)
        rows = {}
        for name, cell in VARIANT_CELLS.items():
            cw = 4 if cell.get("batch") == 3 and cell.get("cluster_size", 2) <= 8 else 2
            ctas = 152 if cell.get("batch") != 3 else 0
            try:
                with cg.Bank(n_accounts=N_ACCOUNTS, version_depth=8, client_warps=cw, ctas=ctas,
                             max_txn=n, log_commits=0, device=local, max_reads=4, **cell) as bank:
                    bank.load()
                    # warm-up on 2^12 transactions; the timed run is sized to about 0.3 s of
                    # this cell's rate (the slow ring-scan cells run a shorter prefix)
                    st = bank.run(cg.Stream(bs[0].op[:4096], bs[0].off[:4096], bs[0].addr))
                    rate = 4096 / max(st.kernel_ms * 1e-3, 1e-6)
                    m = int(min(n, max(4096, rate * 0.3))) // 32 * 32
                    st = bank.run(cg.Stream(np.ascontiguousarray(bs[1].op[:m]),
                                            np.ascontiguousarray(bs[1].off[:m]), bs[1].addr))
                    rows[name] = {"tx_s": m / (st.kernel_ms * 1e-3), "abort_rate": st.abort_rate,
                                  "txn": m}
            except Exception as e:
                rows[name] = {"error": f"{type(e).__name__}: {e}"}
        out[dist] = rows
    return out


def memcd_section(cg, local, n_batches=40):
    """Cache: 2^20 sets x 8 ways, Zipf(0.99) keys over 4 M ids, 99 % GET rounds, 64 K-request
    batches through csmv_memcd_run (host buffers); latency = wall time of one batch call."""
    n = 1 << 16
    cache = cg.Memcd(n_sets=1 << 20, client_warps=4, max_req=n, log_commits=0, device=local)
    for i in range(8):  # fill
        cache.run(cg.memcd_generate(cg.memcd_workload(1 << 22, n, seed=500 + i, get_pct=0)))
    reqs = [cg.memcd_generate(cg.memcd_workload(1 << 22, n, seed=1000 + i, get_pct=99), pinned=True)
            for i in range(n_batches)]
    lat, kern, aborts, commits = [], [], 0, 0
    for r in reqs:
        _, _, st = cache.run(r)
        lat.append(st.total_ms)
        kern.append(st.kernel_ms)
        aborts += st.aborts
        commits += st.commits
    cache.close()
    lat, kern = np.array(lat[4:]), np.array(kern[4:])
    return {"req_s": n * len(lat) / (lat.sum() * 1e-3),
            "kernel_req_s": n * len(kern) / (kern.sum() * 1e-3),
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "abort_rate": aborts / max(1, aborts + commits),
            "workload": "2^20 sets x 8 ways, 16 B keys / 32 B values, Zipf(0.99) over 4M keys, "
                        "99% GET rounds, 64K-request batches, host buffers"}


def serve_section(cg, local, loads=(0.1, 0.25, 0.5, 0.75, 1.0), per_load_s=1.5):
    """Serving loop under open-loop Poisson arrivals: 2^20 sets x 8 ways, batches of U[1K, 64K]
    requests (multiples of 32), 95 % GET rounds, Zipf(0.99) keys over 4 M. The peak is the
    closed-loop throughput of the loop with overlapping batches (submit as fast as admission
    allows); each offered load is a fraction of it. Latency of a batch = completion seen by the
    host - its scheduled arrival. The same arrivals go through the loop with one batch on the
    device at a time (serial_batches: "p50_ms", "p99_ms"), the loop with overlapping batches
    ("overlap_*") and the plain form - one synchronous batch call at a time ("plain_*")."""
    rng = np.random.default_rng(7)
    pool_n = 1 << 21
    pool = cg.memcd_generate(cg.memcd_workload(1 << 22, pool_n, seed=77, get_pct=95))
    def draw():
        n = int(rng.integers(1024 // 32, 65536 // 32 + 1)) * 32
        lo = int(rng.integers(0, (pool_n - n) // 32 + 1)) * 32
        return cg.requests_slice(pool, lo, lo + n)
    out = {"workload": "2^20 sets x 8 ways, batches U[1K,64K] requests, 95% GET rounds, "
                       "Zipf(0.99) over 4M keys, open-loop Poisson arrivals, host ring"}
    def deadline_check(t_end, what):
        if time.perf_counter() > t_end:
            raise TimeoutError(f"serving: {what} exceeded its time budget")

    # one launch shape for every form: the cache autotuner's pick on a 32 K-request sample
    fill = cg.memcd_generate(cg.memcd_workload(1 << 22, 1 << 16, seed=5, get_pct=0))
    best, trials = cg.memcd_autotune(cg.requests_slice(pool, 0, 1 << 15), fill, repeats=2,
                                     n_sets=1 << 20, device=local)
    shape = dict(client_warps=best.client_warps, ctas=best.ctas)
    out["tuned"] = dict(shape, candidates=len(trials))
    progress(f"serving: tuned shape {shape}")

    def new_server(serial):
        srv = cg.Server(n_sets=1 << 20, arena_requests=1 << 19, max_inflight_sets=1 << 16,
                        idle_timeout_ms=5000, device=local, serial_batches=serial, **shape)
        srv.start()  # a session of fills; the measured session starts from the table it leaves
        t_end = time.perf_counter() + 30
        for _ in range(8):
            b = None
            while b is None:
                b = srv.submit(fill)
                deadline_check(t_end, "fill")
            while srv.poll(b, results=False) is None:
                deadline_check(t_end, "fill")
        srv.stop()
        srv.start()
        return srv

    def closed_loop(srv):
        inflight, n_done, t0 = [], 0, time.perf_counter()
        t_end = t0 + 30
        while time.perf_counter() - t0 < 1.0:
            req = draw()
            b = srv.submit(req)
            if b is not None:
                inflight.append((b, req.n_req))
            while inflight and srv.poll(inflight[0][0], results=False) is not None:
                n_done += inflight.pop(0)[1]
        while inflight:
            deadline_check(t_end, "closed loop")
            if srv.poll(inflight[0][0], results=False) is not None:
                n_done += inflight.pop(0)[1]
        return n_done / (time.perf_counter() - t0)

    def open_loop(srv, arrivals, reqs, what):
        lat, dev_ns, pending, inflight, served = [], [], 0, [], 0
        n_b = len(reqs)
        t0 = time.perf_counter()
        t_end = t0 + per_load_s * 4 + 10
        while pending < n_b or inflight:
            deadline_check(t_end, what)
            now = time.perf_counter() - t0
            if pending < n_b and now >= arrivals[pending]:
                b = srv.submit(reqs[pending])
                if b is not None:
                    inflight.append((b, arrivals[pending], reqs[pending].n_req))
                    pending += 1
            i = 0
            while i < len(inflight):
                b, arr, n = inflight[i]
                r = srv.poll(b, results=False)
                if r is not None:
                    lat.append(time.perf_counter() - t0 - arr)
                    dev_ns.append(r[2])
                    served += n
                    inflight.pop(i)
                else:
                    i += 1
        span = time.perf_counter() - t0
        lat = np.array(lat) * 1e3
        dms = np.array(dev_ns) * 1e-6
        return {"achieved_req_s": served / span, "p50_ms": float(np.percentile(lat, 50)),
                "p99_ms": float(np.percentile(lat, 99)),
                "device_p50_ms": float(np.percentile(dms, 50)),
                "device_p99_ms": float(np.percentile(dms, 99))}

    # the capacity: the loop with overlapping batches, closed loop
    srv = new_server(0)
    peak = closed_loop(srv)
    progress(f"serving: closed-loop peak {peak:.3g} req/s")
    out["peak_req_s"] = peak
    mean_n = (1024 + 65536) / 2
    replay = []
    for load in loads:
        rate = load * peak / mean_n  # batches per second
        n_b = max(20, int(rate * per_load_s))
        replay.append((np.cumsum(rng.exponential(1.0 / rate, n_b)), [draw() for _ in range(n_b)]))
    rows = [{"offered_frac": load, "offered_req_s": load * peak, "batches": len(r[1])}
            for load, r in zip(loads, replay)]
    for row, (arrivals, reqs) in zip(rows, replay):
        r = open_loop(srv, arrivals, reqs, f"overlap load {row['offered_frac']}")
        row.update({"overlap_" + k: v for k, v in r.items()})
    st = srv.stop()
    srv.close()
    out["overlap_abort_rate"] = st.aborts / max(1, st.aborts + st.commits)
    # one batch on the device at a time
    srv = new_server(1)
    for row, (arrivals, reqs) in zip(rows, replay):
        row.update(open_loop(srv, arrivals, reqs, f"load {row['offered_frac']}"))
        progress(f"serving: load {row['offered_frac']}: p99 {row['p99_ms']:.3f} ms "
                 f"(overlapping {row['overlap_p99_ms']:.3f} ms)")
    st = srv.stop()
    srv.close()
    out["loads"] = rows
    out["abort_rate"] = st.aborts / max(1, st.aborts + st.commits)  # the measured session
    # the plain form at equal offered load: the same arrivals, one batch call at a time
    # (csmv_memcd_run with host buffers); a batch that arrives while another runs waits
    with cg.Memcd(n_sets=1 << 20, max_req=1 << 16, log_commits=0, device=local,
                  **shape) as cache:
        for _ in range(8):
            cache.run(fill)
        p_commits = p_aborts = 0
        for row, (arrivals, reqs) in zip(rows, replay):
            lat, kms, served, t0 = [], [], 0, time.perf_counter()
            t_end = t0 + per_load_s * 4 + 10
            for arr, req in zip(arrivals, reqs):
                if time.perf_counter() > t_end:
                    row["plain_saturated"] = True
                    break
                while time.perf_counter() - t0 < arr:
                    pass
                _, _, pst = cache.run(req)
                lat.append(time.perf_counter() - t0 - arr)
                kms.append(pst.kernel_ms)
                p_commits += pst.commits
                p_aborts += pst.aborts
                served += req.n_req
            lat = np.array(lat) * 1e3
            row["plain_p50_ms"] = float(np.percentile(lat, 50))
            row["plain_p99_ms"] = float(np.percentile(lat, 99))
            row["plain_kernel_p50_ms"] = float(np.percentile(kms, 50))
            row["plain_kernel_p99_ms"] = float(np.percentile(kms, 99))
            row["plain_achieved_req_s"] = served / (time.perf_counter() - t0)
            progress(f"serving: plain form at load {row['offered_frac']}: "
                     f"p99 {row['plain_p99_ms']:.3f} ms")
        out["plain_abort_rate"] = p_aborts / max(1, p_aborts + p_commits)
    return out


def cpu_baseline(bs, sample_txn=1 << 21):
    """The oracle's CPU executions of a bounded sample of the same batches: striped locks on
    every host core (reported) and one thread in stream order (for comparison)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as orc
    op = np.concatenate([b.op for b in bs])[:sample_txn]
    off = np.concatenate([b.off for b in bs])[:sample_txn]
    addr = bs[0].addr
    init = np.full(N_ACCOUNTS, 1000, np.int32)
    threads = orc.cpu_threads()
    best = min(orc.locked(op, off, addr, N_ACCOUNTS, init, threads)[1] for _ in range(3))
    ser = min(orc.serial(op, off, addr, N_ACCOUNTS, init)[1] for _ in range(2))
    n = op.shape[0]
    return {"value": n / (best * 1e-9), "unit": "committed tx/s", "cores": threads, "kind": "port",
            "sample": f"first {n} transactions of the stream, striped-lock threads on all cores, "
                      f"best of 3", "single_thread_stream_order_tx_s": n / (ser * 1e-9)}


def workload_name(args):
    return (f"bank {args.dist}(0.99) 2^20 int32 accounts, transfers r4/w2, 20% read-only scans "
            f"of 32; 2^24-txn stream in batches of {args.batch}")


def oracle_batches(args, count):
    """The same batches from the oracle's own generator (so this arm loads no library of the
    product)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as orc
    dist_id = {"uniform": 0, "zipf": 1, "hotspot": 2}[args.dist]
    d = dict(WORKLOAD)
    w = orc.Workload(seed=d["seed"], n_accounts=N_ACCOUNTS, n_txn=args.batch * count,
                     pr_read_pct=d["pr_read_pct"], ro_reads=d["ro_reads"],
                     up_reads=d["up_reads"], kind=1, amt_lo=d["amt_lo"], amt_hi=d["amt_hi"],
                     dist=dist_id, zipf_theta=d["zipf_theta"], hot_frac=0.01, hot_prob=0.3,
                     shift_every=1 << 20)
    op, off, addr = orc.generate(w)
    b = args.batch
    return [(op[i * b:(i + 1) * b], off[i * b:(i + 1) * b], addr) for i in range(count)]


def run_reference(args, rank, world):
    """Reference arm: the path's CPU execution (oracle port, striped locks, all host threads)."""
    if rank != 0:
        return
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as orc
    bs = oracle_batches(args, args.warmup + args.steps)
    vals = np.full(N_ACCOUNTS, 1000, np.int32)
    threads = orc.cpu_threads()
    t, commits = 0.0, 0
    for i, (op, off, addr) in enumerate(bs):
        vals, ns = orc.locked(op, off, addr, N_ACCOUNTS, vals, threads)
        if i >= args.warmup:
            t += ns * 1e-9
            commits += op.shape[0]
    v = commits / t
    print(json.dumps({
        "impl": "reference", "metric": "committed tx/s", "value": v, "unit": "committed tx/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": {"workload": workload_name(args)},
        "cpu_baseline": {"value": v, "unit": "committed tx/s", "cores": threads, "kind": "port",
                         "sample": f"{args.batch} transactions per step, striped-lock threads"},
        "e2e": {"value": v, "unit": "committed tx/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0}}))


# ---------------------------------------------------------------------------------------------
# profiling cases: one small invocation of one kernel (run under ncu)
# ---------------------------------------------------------------------------------------------

def run_case(args, local):
    import torch

    import csmv_gb300 as cg
    torch.cuda.set_device(local)
    n = args.case_txn
    if args.case in ("engine", "group", "serial", "flow", "sched"):
        dist = "uniform" if args.case == "engine" else "zipf"
        s, bs = generate_batches(dist, n, 2, pinned=False)
        addr = torch.from_numpy(s.addr.view(np.int32)).cuda()
        dev = [DevBatch(torch, b) for b in bs]
        over = PLAIN if args.case == "engine" else {}
        bank = new_bank(cg, args, local, n, log_commits=0, **over)
        if args.case in ("sched", "group"):
            sched = cg.Scheduler(n_accounts=N_ACCOUNTS, max_txn=n, device=local,
                                 **dict(SCHED, probe_every=1))
            for d in dev:  # a warm-up chunk, then the profiled one
                r = sched.run(bank, d.stream(cg, addr, s.addr.shape[0]))
            sched.close()
            out = {"case": args.case, "commits": r.commits, "planned_ms": r.planned.kernel_ms}
        else:
            run = {"engine": bank.run_device, "serial": bank.run_serial_device,
                   "flow": bank.run_flow_device}[args.case]
            for d in dev:  # a warm-up launch, then the profiled one
                st = run(d.stream(cg, addr, s.addr.shape[0]))
            out = {"case": args.case, "commits": st.commits, "kernel_ms": st.kernel_ms}
        bank.close()
    elif args.case == "mlp":
        rng = np.random.default_rng(0)
        x = (rng.random((n, 64)) < 0.2).astype(np.float32)
        bits = (x.view(np.uint32) >> 16).astype(np.uint16).view(np.int16)  # 0/1 exact in bf16
        dx = torch.from_numpy(bits).cuda()
        dp = torch.zeros(n, dtype=torch.float32, device="cuda")
        with cg.Mlp(seed=1, device=local) as m:
            m.forward(n, dx.data_ptr(), dp.data_ptr())
            m.forward(n, dx.data_ptr(), dp.data_ptr())
        out = {"case": "mlp", "mean_p": float(dp.mean())}
    else:
        n = 1 << 16
        with cg.Memcd(n_sets=1 << 20, client_warps=4, max_req=n, log_commits=0, device=local) as c:
            c.run(cg.memcd_generate(cg.memcd_workload(1 << 22, n, seed=5, get_pct=0)))
            _, _, st = c.run(cg.memcd_generate(cg.memcd_workload(1 << 22, n, seed=6, get_pct=99)))
        out = {"case": "memcd", "commits": st.commits}
    print(json.dumps(out))


# ---------------------------------------------------------------------------------------------

def main():
    args = parse()
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.case:
        run_case(args, local)
        return
    import torch

    import csmv_gb300 as cg

    torch.cuda.set_device(local)
    warm, timed = args.warmup, args.steps
    s, host = generate_batches(args.dist, args.batch, warm + timed, pinned=True)
    addr_dev = torch.from_numpy(np.asarray(s.addr).view(np.int32).copy()).cuda()
    n_addr = int(s.addr.shape[0])
    dev = [DevBatch(torch, b) for b in host]

    tuned = None
    if not args.no_tune:  # the learned arm's launch shape, measured on the first two batches
        progress("tune")
        tuned = tune_learned(torch, cg, dev, addr_dev, n_addr, args, local)
    atomics = cg.measure_atomics(local)
    barrier(world)
    progress("learned arm")
    with ClockSampler(local) as clk:
        learned = run_learned(torch, cg, dev, addr_dev, n_addr, args, local, warm, timed)
    barrier(world)
    t_learned = reduce_max(learned["wall"], world)
    value = learned["commits"] * world / t_learned
    progress("e2e")
    e_commits, e_wall, h2d, d2h = e2e_learned(torch, cg, host, np.asarray(s.addr), args, local,
                                              warm, timed)
    e2e = e_commits * world / reduce_max(e_wall, world)
    progress("comparison arms")
    n_cmp = min(warm + timed, 4)
    group_stream, info = run_engine(cg, dev, addr_dev, n_addr, args, local, list(range(n_cmp)),
                                    log_commits=0)
    plain, _ = run_engine(cg, dev, addr_dev, n_addr, args, local, list(range(min(n_cmp, 3))),
                          log_commits=0, **PLAIN)
    # ablations of the learned arm, one warm-up and two timed batches each (no probe falls in
    # that window, so "learned" is the arm itself timed the same way): the raw sketch-count
    # score instead of the network, no backoff, no heat classes (plain account lock order),
    # rounds keyed by the hottest accounts touched rather than written
    ablations = {}
    for name, over in (("learned", {}), ("sketch_score", dict(score=1)),
                       ("no_backoff", dict(backoff_ns=0)),
                       ("no_heat_classes", dict(hot_last=0)), ("key_touched", dict(key_written=0))):
        r = run_learned(torch, cg, dev, addr_dev, n_addr, args, local, 1, 2,
                        sched_cfg=dict(SCHED, **over))
        ablations[name] = {"tx_s": r["tx_s"], "abort_rate": r["abort_rate"],
                           "flagged_per_step": r["flagged"] / 2}
    if rank != 0:
        return
    pk, pk_kind = peaks()
    # roofline of the engine on this workload (the bounds of the survey's measurement row):
    #  - throughput bound min(BW_eff / B_tx, R_atomic / A_tx): HBM bytes of a transaction's
    #    versioned reads and writes, and the atomics a committed transfer needs (a lock CAS per
    #    written account, plus the group's timestamp draw and completion bits per 32)
    #  - chain bound: the busiest account's lock passes through L_max rounds of the plan, each
    #    with at least TRIPS_PER_HOLD dependent L2 round trips of cas_chain_ns each
    i_last, perm = learned["last_plan"]
    b = host[i_last]
    probe_n = b.n_txn - len(perm)
    order = np.concatenate([np.arange(probe_n), perm.astype(np.int64)])
    l_max, hot_acct, upd_rounds = plan_lock_rounds(b.op, b.off, b.addr, order)
    l_plain, _, _ = plan_lock_rounds(b.op, b.off, b.addr, np.arange(b.n_txn))
    steps_t = timed
    per_step_txn = learned["commits"] / steps_t
    frac_upd = 0.8
    a_tx = 2.0 * frac_upd + 3.0 / 32.0
    b_tx = frac_upd * B_UPDATE + (1 - frac_upd) * B_RO
    bound_atomic = atomics["spread_per_s"] / a_tx
    bound_hbm = pk["hbm_gbs"] * 1e9 / b_tx
    bound_tp = min(bound_atomic, bound_hbm)
    chain_s = l_max * TRIPS_PER_HOLD * atomics["cas_chain_ns"] * 1e-9
    bound_chain = per_step_txn / chain_s
    achieved_atomic = value * a_tx
    traffic = None
    tr = ROOT / "profiles" / "traffic.json"
    if tr.exists():
        try:
            traffic = json.loads(tr.read_text()).get("bank_kernel_learned_bytes_per_launch")
        except Exception:
            traffic = None
    line = {
        "metric": "committed tx/s", "value": value, "unit": "committed tx/s", "n_gpus": world,
        "steps": timed, "warmup": warm, "ms_per_step": t_learned / timed * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded generator with the configured shapes)",
        "config": {"workload": workload_name(args), "l2": "inputs larger than L2 (28 MB/batch)",
                   "ctas": info["ctas"], "threads_per_cta": info["threads_per_cta"],
                   "version_depth": args.depth, "engine": ENGINE, "autotuned": tuned,
                   "scheduler": SCHED, "parallelism": f"replicas x{world}"},
        "abort_rate": learned["abort_rate"],
        "learned": {"tx_s": value, "abort_rate": learned["abort_rate"],
                    "engine_validated": "every transaction: locks, server timestamps, validation",
                    "flagged_per_step": learned["flagged"] / timed,
                    "aborts_by_kind": {"write_write_lock_held": learned["ww"],
                                       "read_validation": learned["rw"],
                                       "data_age": learned["age"]},
                    "plan_ms_per_step": learned["plan_ms"] / timed,
                    "train_ms_per_step": learned["train_ms"] / timed,
                    "engine_ms_per_step": learned["engine_ms"] / timed,
                    "device_ms_per_step": learned["device_ms"] / timed},
        "plain": {"tx_s": plain["tx_s"] * world, "abort_rate": plain["abort_rate"],
                  "method": "reference commit method: per-transaction validation, pre-validation, "
                            "CTA-batched timestamps", "steps": plain["steps"]},
        "group_stream": {"tx_s": group_stream["tx_s"] * world,
                         "abort_rate": group_stream["abort_rate"], "steps": group_stream["steps"],
                         "method": "group commit in stream order, no scheduler"},
        "ablations": ablations,
        "roofline": {"bound": "l2_atomic", "achieved": achieved_atomic,
                     "peak": atomics["spread_per_s"], "unit": "atomic/s",
                     "frac": achieved_atomic / atomics["spread_per_s"], "traffic": traffic,
                     "peak_source": "measured by csmv_measure_atomics in this run",
                     "kernel": "bank_kernel (group commit)", "atomics_per_txn": a_tx,
                     "throughput_bound_tx_s": bound_tp,
                     "throughput_frac": value / bound_tp,
                     "hbm": {"bytes_per_txn": b_tx, "achieved_gbs": value * b_tx / 1e9,
                             "peak_gbs": pk["hbm_gbs"], "frac": value * b_tx / 1e9 / pk["hbm_gbs"],
                             "peak_source": pk_kind},
                     "chain": {"busiest_account": hot_acct, "rounds_locking_it": l_max,
                               "rounds_locking_it_stream_order": l_plain,
                               "update_rounds": upd_rounds, "trips_per_hold": TRIPS_PER_HOLD,
                               "cas_round_trip_ns": atomics["cas_chain_ns"],
                               "bound_tx_s": bound_chain, "frac": value / bound_chain}},
        "atomics": atomics,
        "e2e": {"value": e2e, "unit": "committed tx/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": learned["launches"],
        "clocks": clk.summary(),
    }
    if not args.no_extras:
        sections = [("hotspot", lambda: hotspot_section(torch, cg, args, local)),
                    ("uniform", lambda: uniform_section(torch, cg, args, local)),
                    ("c1", lambda: c1_section(cg, local)),
                    ("dataflow_lane", lambda: dataflow_section(torch, cg, dev, addr_dev, n_addr,
                                                               args, local)),
                    ("variants", lambda: variants_section(cg, local)),
                    ("alternatives", lambda: alternatives_section(torch, cg, dev, addr_dev,
                                                                  n_addr, args, local)),
                    ("memcd", lambda: memcd_section(cg, local)),
                    ("serving", lambda: serve_section(cg, local))]
        for name, fn in sections:
            progress(name)
            try:
                line[name] = fn()
            except Exception as e:  # a section's failure is reported, not fatal to the line
                line[name] = {"error": f"{type(e).__name__}: {e}"}
    if not args.no_cpu_baseline:
        progress("cpu baseline")
        line["cpu_baseline"] = cpu_baseline(host)
    print(json.dumps(line))


def dataflow_section(torch, cg, dev, addr_dev, n_addr, args, local):
    """The earlier learned path, kept as a labelled comparison: transfers the scheduler flags are
    deferred to the dataflow lane, which executes them in stream order WITHOUT locks, server
    timestamps or validation (exact by construction, not CSMV); the rest go through the engine."""
    timed = min(3, len(dev) - 1)
    res = run_learned(torch, cg, dev, addr_dev, n_addr, args, local, 1, timed,
                      sched_cfg=FLOW, bank_over=dict(flow_warps=8, log_commits=0))
    return {"tx_s": res["tx_s"], "abort_rate": res["abort_rate"],
            "lane_txn_per_step": res["serial_txn"] / timed,
            "lane_ms_per_step": res["serial_ms"] / timed,
            "validated": "no: the lane's transactions bypass the engine's validation"}


if __name__ == "__main__":
    main()
