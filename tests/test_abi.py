"""CPU tests of the C-ABI boundary: the libraries load, export every declared symbol, validate
their arguments, and report a missing GPU as a status (never a crash). No compute calls."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import pytest

import csmv_gb300 as cg
from csmv_gb300 import build as b

ROOT = Path(__file__).resolve().parent.parent


def declared(header: Path) -> set[str]:
    text = re.sub(r"/\*.*?\*/", "", header.read_text(), flags=re.S)
    return set(re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(csmv_\w+)\s*\(", text, flags=re.M))


def exported(lib: Path) -> set[str]:
    out = subprocess.run(["nm", "-D", "--defined-only", str(lib)], capture_output=True, text=True,
                         check=True).stdout
    return {ln.split()[-1] for ln in out.splitlines() if ln.strip()}


def test_every_declared_symbol_is_exported():
    names = declared(ROOT / "include" / "csmv.h")
    assert {"csmv_bank_create", "csmv_bank_run", "csmv_bank_read_log", "csmv_last_error",
            "csmv_memcd_create", "csmv_memcd_run", "csmv_memcd_read_table"} <= names
    missing = names - exported(b.LIB)
    assert not missing, missing


def test_library_loads_and_reports_version():
    L = cg.lib()
    assert L.csmv_abi_version() == 3
    assert L.csmv_status_str(4) == b"bounded device wait timed out"


def test_config_validation_is_a_status():
    for bad in (dict(version_depth=3), dict(ring_size=100), dict(client_warps=0),
                dict(client_warps=16), dict(validate=1, batch=0, writeback=0), dict(max_txn=33),
                dict(spin_limit_log2=2), dict(n_accounts=1), dict(batch=9),
                dict(batch=3, validate=1, writeback=1), dict(batch=3, cluster_size=3),
                dict(batch=3, cluster_size=4, client_warps=15), dict(flow_warps=17),
                dict(prevalidate=4), dict(prevalidate=3, validate=1, batch=1),
                dict(max_reads=5)):
        with pytest.raises(cg.CsmvError) as e:
            cg.Bank(cg.bank_config(**bad))
        assert e.value.status == 1, bad


def test_memcd_config_validation_is_a_status():
    for bad in (dict(n_ways=4), dict(version_depth=4), dict(client_warps=0),
                dict(client_warps=16), dict(batch=cg.BATCH_LANE), dict(max_req=33),
                dict(n_sets=0), dict(spin_limit_log2=40)):
        with pytest.raises(cg.CsmvError) as e:
            cg.Memcd(cg.memcd_config(**bad))
        assert e.value.status == 1, bad
    for bad in (dict(n_req=33), dict(get_pct=101), dict(dist=cg.DIST_HOTSPOT), dict(n_keys=0)):
        kw = dict(n_keys=100, n_req=64)
        kw.update(bad)
        with pytest.raises(cg.CsmvError) as e:
            cg.memcd_generate(cg.memcd_workload(**kw))
        assert e.value.status == 1, bad


def test_workload_validation_is_a_status():
    for bad in (dict(n_txn=33), dict(up_reads=1), dict(amt_lo=0), dict(amt_hi=5000),
                dict(pr_read_pct=101), dict(kind=0), dict(dist=7),
                dict(n_accounts=3, up_reads=4)):  # four distinct accounts out of three
        kw = dict(n_accounts=100, n_txn=64)
        kw.update(bad)
        with pytest.raises(cg.CsmvError) as e:
            cg.generate(cg.bank_workload(**kw))
        assert e.value.status == 1, bad


def test_null_handles_are_rejected():
    L = cg.lib()
    assert L.csmv_bank_load(None, None) == 1
    assert L.csmv_bank_run(None, None, None) == 1
    assert L.csmv_bank_read_values(None, None) == 1
    L.csmv_bank_destroy(None)
    assert L.csmv_memcd_clear(None) == 1
    assert L.csmv_memcd_run(None, None, None) == 1
    assert L.csmv_memcd_read_table(None, None, None) == 1
    L.csmv_memcd_destroy(None)


@pytest.mark.skipif(cg.cuda_device_present(), reason="a GPU is present")
def test_create_without_gpu_is_no_device():
    with pytest.raises(cg.CsmvError) as e:
        cg.Bank(n_accounts=64, max_txn=64)
    assert e.value.status == 6


def test_driver_keeps_reference_cli():
    exe = b.BIN / "csmv_bank"
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0 and "argument order" in out.stdout and "8) verbose" in out.stdout


def test_memcd_driver_keeps_reference_cli():
    exe = b.BIN / "csmv_memcd"
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0 and "argument order" in out.stdout and "10) verbose" in out.stdout


def test_devtest_library_exports():
    names = exported(b.DEVTEST_LIB)
    assert {"csmv_devtest_read", "csmv_devtest_prevalidate", "csmv_devtest_writeback",
            "csmv_devtest_bounded_wait"} <= names
    C.CDLL(str(b.DEVTEST_LIB))


# the binding's ctypes mirrors of the header's structs
MIRRORS = {
    "BankWorkload": "csmv_bank_workload", "BankStream": "csmv_bank_stream",
    "BankConfig": "csmv_bank_config", "Stats": "csmv_stats",
    "MemcdWorkload": "csmv_memcd_workload", "MemcdBatch": "csmv_memcd_batch",
    "MemcdConfig": "csmv_memcd_config", "TuneTrial": "csmv_tune_trial",
    "TuneResult": "csmv_tune_result", "MemcdTuneResult": "csmv_memcd_tune_result",
    "ServeConfig": "csmv_serve_config", "SchedConfig": "csmv_sched_config",
    "SchedReport": "csmv_sched_report", "AtomicRates": "csmv_atomic_rates",
}


def test_binding_structs_match_the_header(tmp_path):
    """Every ctypes struct of the binding has the size, field offsets and field sizes of its C
    struct, as a C compiler lays it out from include/csmv.h (a field added to one side only
    would shift every later field the library reads)."""
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "csmv.h"', "int main(void) {"]
    for py, c in MIRRORS.items():
        cls = getattr(cg, py)
        lines.append(f'  printf("{py} . %zu 0\\n", sizeof({c}));')
        for name, *_ in cls._fields_:
            lines.append(f'  printf("{py} {name} %zu %zu\\n", offsetof({c}, {name}), '
                         f"sizeof((({c}*)0)->{name}));")
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    seen = 0
    for ln in out.splitlines():
        py, name, a, bsz = ln.split()
        cls = getattr(cg, py)
        if name == ".":
            assert C.sizeof(cls) == int(a), (py, C.sizeof(cls), int(a))
        else:
            f = getattr(cls, name)
            assert (f.offset, f.size) == (int(a), int(bsz)), (py, name, f.offset, f.size, a, bsz)
        seen += 1
    assert seen == sum(len(getattr(cg, py)._fields_) + 1 for py in MIRRORS)
