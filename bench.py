"""Benchmark of the CSMV commit path on GB300 (contract: one JSON line from rank 0).

Workload (the configuration the headline metric is quoted on): the contended bank at scale -
2^20 int32 accounts at 1000, Zipf(0.99) account choice, transfers that read 4 and write 2
accounts (skipped when funds are short), 20 % read-only rounds summing 32 accounts. The stream
is 2^24 transactions, seeded; a step is one batch of 2^20 consecutive transactions of it
(batch i = transactions [i 2^20, (i+1) 2^20)), so warm-up and timed steps see different
transactions and the account state carries over between steps. Stream arrays are larger than
L2 (28 MB per batch), so no L2 flush is needed between steps.

Two arms run the same batches on separate banks:
  plain    the commit engine alone (csmv_bank_run_device): every transfer through the stamp
           protocol, client warps + per-CTA commit server on every SM
  learned  the learned conflict scheduler in front of the same engine (csmv_sched_run): a probe
           slice in stream order trains the conflict predictor, the predictor routes likely-
           conflicting transfers to the dataflow lane (run after the rest, each transfer as
           soon as the transfers it depends on have run) and spaces the rest
value = the learned arm's committed tx/s (GPU time of the whole step, inputs resident in HBM);
e2e = the same through host buffers (pinned -> device copies and the statistics read inside
the timed region). Both arms' throughput and abort rate are in "plain" / "learned".

Extra sections: "hotspot" (1 % hot set drawing 30 % of the accesses, moving every 2^20
transactions: learned vs plain), "uniform" (the same bank with uniform accounts, plain engine),
"memcd" (8-way cache of 2^20 sets, Zipf(0.99) keys over 4 M, 99 % GET rounds, 64 K-request
batches through the batch call: throughput and p50/p99 batch latency) and "serving" (the same
cache behind the serving loop under open-loop Poisson arrivals at 10-100 % of its closed-loop
peak, batches of 1 K-64 K requests, 95 % GET rounds: achieved req/s and p50/p99 latency).

--impl reference runs the reference arm: the path's CPU execution (the oracle port, striped
locks on every host core) on the same batches. --case NAME runs one small invocation of one
kernel for profiling (engine, serial, flow, mlp, memcd, sched). Multi-GPU: replicas only (no
collective on the path); each rank runs its own instance on its own GPU, value sums the ranks'
transactions over the slowest rank's time.
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
SCHED = dict(serial_lane=2, defer_threshold=0.0, probe_every=3, probe_rounds_pct=2)
FLOW_WARPS = 8  # warps of the dataflow lane's execution CTA


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="csmv", choices=["csmv", "reference"])
    ap.add_argument("--batch", type=int, default=BATCH)
    ap.add_argument("--dist", default="zipf", choices=["zipf", "uniform", "hotspot"])
    ap.add_argument("--client-warps", type=int, default=int(os.environ.get("CSMV_CLIENT_WARPS", 2)))
    ap.add_argument("--ctas", type=int, default=int(os.environ.get("CSMV_CTAS", 152)))
    ap.add_argument("--depth", type=int, default=int(os.environ.get("CSMV_DEPTH", 8)))
    ap.add_argument("--case", default=None,
                    choices=["engine", "serial", "flow", "mlp", "memcd", "sched"])
    ap.add_argument("--no-extras", action="store_true", help="skip hotspot/uniform/memcd sections")
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
    """Kernels the scheduler and the engine launched for one chunk (see sched_engine.cu)."""
    n = 1  # access counts
    if rep.n_probe:
        n += 1 + 1 + 2 + 4  # features, probe engine run, labels + rates, 2 x (grad + adam)
    n += 2 + 2  # features and network forward; read-only flags and scan
    if rep.n_planned:
        n += 6  # keys, buckets, scan, scatter, read-only list, emit
        n += 1 if rep.planned.commits else 0  # concurrent engine run
        if rep.n_serial:                      # dataflow lane: analysis, sort, run, commit
            n += 17 + 5 * (((N_ACCOUNTS - 1).bit_length() + 7) // 8)
    return n


def new_bank(cg, args, local, max_txn, **over):
    kw = dict(n_accounts=N_ACCOUNTS, version_depth=args.depth, client_warps=args.client_warps,
              ctas=args.ctas, max_txn=max_txn, log_commits=0, device=local, flow_warps=FLOW_WARPS)
    kw.update(over)
    bank = cg.Bank(**kw)
    bank.load()
    return bank


# ---------------------------------------------------------------------------------------------
# arms
# ---------------------------------------------------------------------------------------------

def run_plain(cg, dev, addr_dev, n_addr, args, local, warm, timed):
    bank = new_bank(cg, args, local, args.batch)
    res = dict(ms=0.0, commits=0, aborts=0, ro=0, upd=0)
    for i in range(warm + timed):
        st = bank.run_device(dev[i].stream(cg, addr_dev, n_addr))
        if i >= warm:
            res["ms"] += st.kernel_ms
            res["commits"] += st.commits
            res["aborts"] += st.aborts
            res["ro"] += st.commits_readonly
            res["upd"] += st.commits_update + st.commits_nowrite
    info = bank.device_info()
    bank.close()
    return res, info


def run_learned(torch, cg, dev, addr_dev, n_addr, args, local, warm, timed):
    bank = new_bank(cg, args, local, args.batch)
    sched = cg.Scheduler(n_accounts=N_ACCOUNTS, max_txn=args.batch, device=local, **SCHED)
    res = dict(wall=0.0, commits=0, aborts=0, launches=0, serial_ms=0.0, serial_txn=0,
               plan_ms=0.0, train_ms=0.0)
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
            res["serial_ms"] += rep.serial.kernel_ms
            res["serial_txn"] += rep.n_serial
            res["plan_ms"] += rep.plan_ms
            res["train_ms"] += rep.train_ms
    sched.close()
    bank.close()
    return res


def e2e_learned(torch, cg, host, s_addr, args, local, warm, timed):
    """Host buffers through the public calls: each step copies the batch's op/off arrays and its
    range of the address array from pinned host memory, runs the scheduler (which returns the
    statistics to the host) and is timed on the host clock."""
    bank = new_bank(cg, args, local, args.batch)
    sched = cg.Scheduler(n_accounts=N_ACCOUNTS, max_txn=args.batch, device=local, **SCHED)
    n = args.batch
    d_op = torch.empty(n, dtype=torch.int32, device="cuda")
    d_off = torch.empty(n, dtype=torch.int32, device="cuda")
    d_addr = torch.empty(s_addr.shape[0], dtype=torch.int32, device="cuda")
    h_addr = torch.from_numpy(s_addr.view(np.int32))
    commits, wall, h2d = 0, 0.0, 0
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
        rep = sched.run(bank, ds)
        dt = time.perf_counter() - t0
        if i >= warm:
            wall += dt
            commits += rep.commits
            h2d += b.op.nbytes + b.off.nbytes + (hi - lo) * 4
    sched.close()
    bank.close()
    return commits, wall, h2d // max(1, timed)


def hotspot_section(torch, cg, local):
    """Learned vs plain on the shifting hotspot: 8 batches of 2^18 transactions."""
    chunk, count = 1 << 18, 8
    s, bs = generate_batches("hotspot", chunk, count, pinned=False, seed=3, pr_read_pct=10,
                             ro_reads=8, up_reads=2, hot_frac=0.01, hot_prob=0.3,
                             shift_every=1 << 20)
    addr = torch.from_numpy(s.addr.view(np.int32)).cuda()
    dev = [DevBatch(torch, b) for b in bs]
    out = {}
    for arm in ("plain", "learned"):
        bank = cg.Bank(n_accounts=N_ACCOUNTS, version_depth=8, client_warps=2, ctas=152,
                       max_txn=chunk, log_commits=0, device=local)
        bank.load()
        sched = cg.Scheduler(n_accounts=N_ACCOUNTS, max_txn=chunk, device=local) \
            if arm == "learned" else None
        c = a = 0
        t = 0.0
        for d in dev:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            if sched is None:
                st = bank.run_device(d.stream(cg, addr, s.addr.shape[0]))
                c, a = c + st.commits, a + st.aborts
            else:
                r = sched.run(bank, d.stream(cg, addr, s.addr.shape[0]))
                c, a = c + r.commits, a + r.aborts
            torch.cuda.synchronize()
            t += time.perf_counter() - t0
        if sched is not None:
            sched.close()
        bank.close()
        out[arm] = {"tx_s": c / t, "abort_rate": a / (a + c)}
    out["workload"] = ("2^20 accounts, 1% hot set drawing 30% of the accesses, moving every 2^20 "
                       "txn; 90% 2-account transfers, 10% read-only sums of 8; 8 batches of 2^18")
    return out


def uniform_section(torch, cg, args, local):
    s, bs = generate_batches("uniform", args.batch, 4, pinned=False)
    addr = torch.from_numpy(s.addr.view(np.int32)).cuda()
    dev = [DevBatch(torch, b) for b in bs]
    res, _ = run_plain(cg, dev, addr, s.addr.shape[0], args, local, 1, 3)
    return {"tx_s": res["commits"] / (res["ms"] * 1e-3),
            "abort_rate": res["aborts"] / (res["aborts"] + res["commits"]),
            "workload": "same bank, uniform account choice, plain engine, 3 batches of 2^20"}


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
    closed-loop throughput (submit as fast as admission allows); each offered load is a fraction
    of it. Latency of a batch = completion seen by the host - its scheduled arrival. The same
    arrivals then go through the plain form - one synchronous batch call at a time - for the
    p50/p99 at equal offered load ("plain_*" in each row)."""
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

    with cg.Server(n_sets=1 << 20, client_warps=4, arena_requests=1 << 19,
                   max_inflight_sets=1 << 16, idle_timeout_ms=5000, device=local) as srv:
        srv.start()
        fill = cg.memcd_generate(cg.memcd_workload(1 << 22, 1 << 16, seed=5, get_pct=0))
        t_end = time.perf_counter() + 30
        for _ in range(8):
            b = None
            while b is None:
                b = srv.submit(fill)
                deadline_check(t_end, "fill")
            while srv.poll(b, results=False) is None:
                deadline_check(t_end, "fill")
        progress("serving: table filled")
        # closed loop: keep the ring full
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
        peak = n_done / (time.perf_counter() - t0)
        progress(f"serving: closed-loop peak {peak:.3g} req/s")
        out["peak_req_s"] = peak
        mean_n = (1024 + 65536) / 2
        rows, replay = [], []
        for load in loads:
            rate = load * peak / mean_n  # batches per second
            n_b = max(20, int(rate * per_load_s))
            arrivals = np.cumsum(rng.exponential(1.0 / rate, n_b))
            reqs = [draw() for _ in range(n_b)]
            lat, pending, inflight = [], 0, []
            served = 0
            t0 = time.perf_counter()
            t_end = t0 + per_load_s * 4 + 10
            while pending < n_b or inflight:
                deadline_check(t_end, f"load {load}")
                now = time.perf_counter() - t0
                if pending < n_b and now >= arrivals[pending]:
                    b = srv.submit(reqs[pending])
                    if b is not None:
                        inflight.append((b, arrivals[pending], reqs[pending].n_req))
                        pending += 1
                i = 0
                while i < len(inflight):
                    b, arr, n = inflight[i]
                    if srv.poll(b, results=False) is not None:
                        lat.append(time.perf_counter() - t0 - arr)
                        served += n
                        inflight.pop(i)
                    else:
                        i += 1
            span = time.perf_counter() - t0
            lat = np.array(lat) * 1e3
            rows.append({"offered_frac": load, "offered_req_s": load * peak,
                         "achieved_req_s": served / span, "p50_ms": float(np.percentile(lat, 50)),
                         "p99_ms": float(np.percentile(lat, 99)), "batches": n_b})
            replay.append((arrivals, reqs))
            progress(f"serving: load {load}: p50 {rows[-1]['p50_ms']:.3f} ms")
        st = srv.stop()
        out["loads"] = rows
        out["abort_rate"] = st.aborts / max(1, st.aborts + st.commits)
    # the plain form at equal offered load: the same arrivals, one batch call at a time
    # (csmv_memcd_run with host buffers); a batch that arrives while another runs waits
    with cg.Memcd(n_sets=1 << 20, client_warps=4, max_req=1 << 16, log_commits=0,
                  device=local) as cache:
        for _ in range(8):
            cache.run(fill)
        for row, (arrivals, reqs) in zip(rows, replay):
            lat, served, t0 = [], 0, time.perf_counter()
            t_end = t0 + per_load_s * 4 + 10
            for arr, req in zip(arrivals, reqs):
                if time.perf_counter() > t_end:
                    row["plain_saturated"] = True
                    break
                while time.perf_counter() - t0 < arr:
                    pass
                cache.run(req)
                lat.append(time.perf_counter() - t0 - arr)
                served += req.n_req
            lat = np.array(lat) * 1e3
            row["plain_p50_ms"] = float(np.percentile(lat, 50))
            row["plain_p99_ms"] = float(np.percentile(lat, 99))
            row["plain_achieved_req_s"] = served / (time.perf_counter() - t0)
            progress(f"serving: plain form at load {row['offered_frac']}: "
                     f"p99 {row['plain_p99_ms']:.3f} ms")
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


def run_reference(args, rank, world):
    """Reference arm: the path's CPU execution (oracle port, striped locks, all host threads)."""
    if rank != 0:
        return
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as orc
    s, bs = generate_batches(args.dist, args.batch, args.warmup + args.steps, pinned=False)
    vals = np.full(N_ACCOUNTS, 1000, np.int32)
    threads = orc.cpu_threads()
    t, commits = 0.0, 0
    for i, b in enumerate(bs):
        vals, ns = orc.locked(b.op, b.off, b.addr, N_ACCOUNTS, vals, threads)
        if i >= args.warmup:
            t += ns * 1e-9
            commits += b.n_txn
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
    if args.case in ("engine", "serial", "flow", "sched"):
        dist = "uniform" if args.case == "engine" else "zipf"
        n = (1 << 15) if args.case == "serial" else (1 << 18)
        s, bs = generate_batches(dist, n, 2, pinned=False)
        addr = torch.from_numpy(s.addr.view(np.int32)).cuda()
        dev = [DevBatch(torch, b) for b in bs]
        bank = new_bank(cg, args, local, n)
        if args.case == "sched":
            sched = cg.Scheduler(n_accounts=N_ACCOUNTS, max_txn=n, device=local, **SCHED)
            for d in dev:
                r = sched.run(bank, d.stream(cg, addr, s.addr.shape[0]))
            sched.close()
            out = {"case": "sched", "commits": r.commits}
        else:
            run = {"engine": bank.run_device, "serial": bank.run_serial_device,
                   "flow": bank.run_flow_device}[args.case]
            for d in dev:  # a warm-up launch, then the profiled one
                st = run(d.stream(cg, addr, s.addr.shape[0]))
            out = {"case": args.case, "commits": st.commits, "kernel_ms": st.kernel_ms}
        bank.close()
    elif args.case == "mlp":
        n = 1 << 18
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
    if not args.no_tune:  # the engine's launch shape for this workload, measured on a sample
        progress("autotune")
        sample = cg.Stream(np.ascontiguousarray(host[0].op[:1 << 16]),
                           np.ascontiguousarray(host[0].off[:1 << 16]), host[0].addr)
        best, trials = cg.autotune(sample, repeats=2, n_accounts=N_ACCOUNTS, init_value=1000,
                                   device=local)
        args.client_warps, args.ctas, args.depth = best.client_warps, best.ctas, best.version_depth
        tuned = {"client_warps": best.client_warps, "ctas": best.ctas,
                 "version_depth": best.version_depth, "candidates": len(trials),
                 "sample_txn": 1 << 16}
    barrier(world)
    progress("plain arm")
    plain, info = run_plain(cg, dev, addr_dev, n_addr, args, local, warm, timed)
    barrier(world)
    progress("learned arm")
    with ClockSampler(local) as clk:
        learned = run_learned(torch, cg, dev, addr_dev, n_addr, args, local, warm, timed)
    barrier(world)
    progress("e2e")
    t_learned = reduce_max(learned["wall"], world)
    value = learned["commits"] * world / t_learned
    t_plain = reduce_max(plain["ms"] * 1e-3, world)
    e_commits, e_wall, h2d = e2e_learned(torch, cg, host, np.asarray(s.addr), args, local, warm,
                                         timed)
    e2e = e_commits * world / reduce_max(e_wall, world)
    if rank != 0:
        return
    pk, pk_kind = peaks()
    # roofline of the dominant part of the learned step, the dataflow lane (its execution
    # kernel holds nearly all of the lane's device time): algorithmic bytes of the transfers it
    # committed over the lane's device time
    s_ms = learned["serial_ms"]
    achieved = learned["serial_txn"] * B_UPDATE / (s_ms * 1e-3) / 1e9 if s_ms > 0 else 0.0
    traffic = None
    tr = ROOT / "profiles" / "traffic.json"
    if tr.exists():
        try:
            traffic = json.loads(tr.read_text()).get("flow_exec_kernel_bytes_per_launch")
        except Exception:
            traffic = None
    plain_gbs = (plain["upd"] * B_UPDATE + plain["ro"] * B_RO) / (plain["ms"] * 1e-3) / 1e9
    l_abort = learned["aborts"] / max(1, learned["aborts"] + learned["commits"])
    line = {
        "metric": "committed tx/s", "value": value, "unit": "committed tx/s", "n_gpus": world,
        "steps": timed, "warmup": warm, "ms_per_step": t_learned / timed * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded generator with the configured shapes)",
        "config": {"workload": workload_name(args), "l2": "inputs larger than L2 (28 MB/batch)",
                   "ctas": info["ctas"], "threads_per_cta": info["threads_per_cta"],
                   "version_depth": args.depth, "autotuned": tuned, "scheduler": SCHED,
                   "parallelism": f"replicas x{world}"},
        "abort_rate": l_abort,
        "learned": {"tx_s": value, "abort_rate": l_abort,
                    "dataflow_lane_txn_per_step": learned["serial_txn"] // timed,
                    "dataflow_lane_ms_per_step": learned["serial_ms"] / timed,
                    "plan_ms_per_step": learned["plan_ms"] / timed,
                    "train_ms_per_step": learned["train_ms"] / timed},
        "plain": {"tx_s": plain["commits"] * world / t_plain,
                  "abort_rate": plain["aborts"] / max(1, plain["aborts"] + plain["commits"]),
                  "roofline_frac_of_measured_hbm": plain_gbs / pk["hbm_gbs"]},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / pk["hbm_gbs"], "traffic": traffic,
                     "kernel": "flow_exec_kernel (dataflow lane)", "peak_source": pk_kind,
                     "bytes_per_txn": B_UPDATE},
        "e2e": {"value": e2e, "unit": "committed tx/s", "h2d_bytes_per_step": h2d,
                # per engine or lane run: statistics (80 B) + commit-order words (768 B); up to
                # three runs per step, the scheduler's 16 B of plan sizes and loss, and the
                # dataflow lane's 8 B of access count and widest transfer
                "d2h_bytes_per_step": 3 * (80 + 768) + 16 + 8},
        "gpu_launches": learned["launches"],
        "clocks": clk.summary(),
    }
    if not args.no_extras:
        sections = [("hotspot", lambda: hotspot_section(torch, cg, local)),
                    ("uniform", lambda: uniform_section(torch, cg, args, local)),
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


if __name__ == "__main__":
    main()
