"""Benchmark of the CSMV commit path on GB300 (contract: one JSON line from rank 0).

Workload (the configuration the headline metric is quoted on): contended bank at scale -
2^20 int32 accounts, Zipf(0.99) account choice, transfers read 4 / write 2, 20% read-only scans
of 32 accounts, 2^24 transactions per step, persistent kernel over every SM. One step = one run
of the whole stream through the engine; the account state carries over between steps.

  value   committed tx/s with the stream resident in HBM (csmv_bank_run_device), device time of
          the persistent kernel from CUDA events on the engine's own stream
  e2e     committed tx/s through csmv_bank_run with pinned HOST buffers: host->device copy of the
          stream and device->host read of the statistics inside the timed region
  roofline  algorithmic bytes per committed transaction (16 B per versioned read, 12 B per
          written item: 88 B per transfer, 512 B per 32-account scan) / kernel time vs the
          measured HBM copy bandwidth (MEASURED_PEAKS.json)
  cpu_baseline  the oracle's host-threaded lock-based execution of a bounded sample of the
          same stream on this host's cores (the reference has no CPU implementation)

--impl reference runs that CPU execution as the reference arm (the reference's own code is
GPU-only; its CPU semantics are the oracle port). Multi-GPU: replicas only (no collective in the
path); each rank runs its own instance, value sums the ranks' transactions over the max time.
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
N_TXN = 1 << 24
WORKLOAD = dict(seed=2026, pr_read_pct=20, ro_reads=32, up_reads=4, amt_lo=1, amt_hi=10,
                zipf_theta=0.99)
B_UPDATE = 16 * 4 + 12 * 2
B_RO = 16 * 32


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="csmv", choices=["csmv", "reference"])
    ap.add_argument("--n-txn", type=int, default=N_TXN)
    ap.add_argument("--dist", default="zipf", choices=["zipf", "uniform", "hotspot"])
    ap.add_argument("--client-warps", type=int, default=int(os.environ.get("CSMV_CLIENT_WARPS", 2)))
    ap.add_argument("--ctas", type=int, default=int(os.environ.get("CSMV_CTAS", 152)))
    ap.add_argument("--depth", type=int, default=int(os.environ.get("CSMV_DEPTH", 8)))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def dist_id(name):
    import csmv_gb300 as cg
    return {"zipf": cg.DIST_ZIPF, "uniform": cg.DIST_UNIFORM, "hotspot": cg.DIST_HOTSPOT}[name]


def workload(args):
    import csmv_gb300 as cg
    return cg.bank_workload(N_ACCOUNTS, args.n_txn, dist=dist_id(args.dist), kind=cg.KIND_TRANSFER,
                            **WORKLOAD)


def dist_env():
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    return rank, world, local


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


def cpu_baseline(stream, args, sample_txn=1 << 21):
    """Oracle's host-threaded lock-based execution of the first sample_txn transactions."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as orc
    n = min(sample_txn, stream.n_txn)
    op, off = stream.op[:n], stream.off[:n]
    init = np.full(N_ACCOUNTS, 1000, np.int32)
    threads = orc.cpu_threads()
    best = None
    for _ in range(3):
        _, ns = orc.locked(op, off, stream.addr, N_ACCOUNTS, init, threads)
        best = ns if best is None else min(best, ns)
    return {"value": n / (best * 1e-9), "unit": "committed tx/s", "cores": threads, "kind": "port",
            "sample": f"first {n} transactions of the stream, striped-lock threads, best of 3"}


def run_reference(args, rank, world):
    """Reference arm: the CPU execution of the path on the host cores (oracle port)."""
    if rank != 0:
        return
    import csmv_gb300 as cg  # generator only (host code)
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as orc
    sample = min(args.n_txn, 1 << 21)
    w = workload(args)
    w.n_txn = sample
    s = cg.generate(w)
    init = np.full(N_ACCOUNTS, 1000, np.int32)
    threads = orc.cpu_threads()
    for _ in range(args.warmup):
        orc.locked(s.op, s.off, s.addr, N_ACCOUNTS, init, threads)
    t = 0
    for _ in range(args.steps):
        _, ns = orc.locked(s.op, s.off, s.addr, N_ACCOUNTS, init, threads)
        t += ns * 1e-9
    v = sample * args.steps / t
    line = {"impl": "reference", "metric": "committed tx/s", "value": v, "unit": "committed tx/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int32", "data": "synthetic",
            "config": {"workload": f"bank {args.dist}(0.99) 2^20 accounts r4/w2, 20% RO scans of 32",
                       "sample_txn": sample},
            "cpu_baseline": {"value": v, "unit": "committed tx/s", "cores": threads, "kind": "port",
                             "sample": f"{sample} transactions per step, striped-lock threads"},
            "e2e": {"value": v, "unit": "committed tx/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    args = parse()
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    import torch

    import csmv_gb300 as cg

    torch.cuda.set_device(local)
    w = workload(args)
    s = cg.generate(w, pinned=True)
    n = s.n_txn
    h2d = (s.op.nbytes + s.off.nbytes + s.addr.nbytes)
    dev = [torch.from_numpy(np.asarray(a).view(np.int32).copy()).cuda() for a in (s.op, s.off, s.addr)]
    ds = cg.BankStream(n, dev[0].data_ptr(), dev[1].data_ptr(), dev[2].data_ptr(), s.addr.shape[0])
    bank = cg.Bank(n_accounts=N_ACCOUNTS, version_depth=args.depth, client_warps=args.client_warps,
                   ctas=args.ctas, max_txn=n, log_commits=0, device=local)
    bank.load()
    for _ in range(args.warmup):
        bank.run_device(ds)
    torch.cuda.synchronize()
    barrier(world)
    totals = dict(ms=0.0, commits=0, ro=0, aborts=0, upd=0)
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            st = bank.run_device(ds)
            totals["ms"] += st.kernel_ms
            totals["commits"] += st.commits
            totals["ro"] += st.commits_readonly
            totals["upd"] += st.commits_update + st.commits_nowrite
            totals["aborts"] += st.aborts
    torch.cuda.synchronize()
    barrier(world)
    t_dev = reduce_max(totals["ms"] * 1e-3, world)
    value = totals["commits"] * world / t_dev
    # e2e: host buffers through the public call (copies inside the timed region)
    barrier(world)
    t0 = time.perf_counter()
    e_commits = 0
    for _ in range(args.steps):
        st = bank.run(s)
        e_commits += st.commits
    t_e2e = reduce_max(time.perf_counter() - t0, world)
    e2e = e_commits * world / t_e2e
    info = bank.device_info()
    bank.close()
    if rank != 0:
        return
    pk, pk_kind = peaks()
    bytes_per_tx = (totals["upd"] * B_UPDATE + totals["ro"] * B_RO) / max(1, totals["commits"])
    achieved = bytes_per_tx * totals["commits"] / (totals["ms"] * 1e-3) / 1e9
    traffic = None
    prof = ROOT / "profiles" / "traffic.json"
    if prof.exists():
        try:
            traffic = json.loads(prof.read_text()).get("bytes_per_launch_scaled")
        except Exception:
            traffic = None
    line = {
        "metric": "committed tx/s", "value": value, "unit": "committed tx/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": totals["ms"] / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic",
        "config": {"workload": f"bank {args.dist}(0.99), 2^20 int32 accounts, transfers r4/w2, "
                               f"20% read-only scans of 32, {n} txn/step, depth {args.depth}",
                   "l2": "inputs larger than L2 (stream ~%d MB)" % (h2d >> 20),
                   "ctas": info["ctas"], "threads_per_cta": info["threads_per_cta"],
                   "parallelism": f"replicas x{world}"},
        "abort_rate": totals["aborts"] / max(1, totals["aborts"] + totals["commits"]),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / pk["hbm_gbs"], "traffic": traffic,
                     "peak_source": pk_kind,
                     "bytes_per_tx": bytes_per_tx},
        "e2e": {"value": e2e, "unit": "committed tx/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": 2 * 8 * 9 + 640},
        "gpu_launches": args.steps,
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(s, args)
    print(json.dumps(line))


if __name__ == "__main__":
    main()
