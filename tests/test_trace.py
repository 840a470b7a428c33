"""On-disk streams and commit logs (csmv_stream_* / csmv_log_*): round trips, the checks that
refuse a damaged or foreign file, capacity errors, byte layout, and a CPU replay of a stream
read back from its file."""
import struct

import numpy as np
import pytest

import csmv_gb300 as cg
import oracle as orc


def _stream(seed=3, n=32 * 64):
    return cg.generate(cg.bank_workload(512, n, seed=seed, pr_read_pct=20, ro_reads=8,
                                        up_reads=4, dist=cg.DIST_ZIPF))


def test_stream_round_trip(tmp_path):
    s = _stream()
    p = tmp_path / "a.stream"
    cg.save_stream(p, s)
    t = cg.load_stream(p)
    for a, b in ((s.op, t.op), (s.off, t.off), (s.addr, t.addr)):
        np.testing.assert_array_equal(a, b)


def test_stream_layout_is_little_endian_with_header(tmp_path):
    s = _stream(n=32)
    p = tmp_path / "b.stream"
    cg.save_stream(p, s)
    raw = p.read_bytes()
    assert raw[:8] == b"CSMVSTRM"
    version, n_txn, n_addr = struct.unpack_from("<IIQ", raw, 8)
    assert (version, n_txn, n_addr) == (1, 32, s.addr.shape[0])
    assert len(raw) == 32 + 8 * n_txn + 4 * n_addr
    assert struct.unpack_from("<I", raw, 32)[0] == int(s.op[0])
    # FNV-1a 64 of the payload
    h = 0xcbf29ce484222325
    for byte in raw[32:]:
        h = ((h ^ byte) * 0x100000001b3) & 0xFFFFFFFFFFFFFFFF
    assert struct.unpack_from("<Q", raw, 24)[0] == h


@pytest.mark.parametrize("damage", ["payload", "truncate", "magic", "version", "extra"])
def test_damaged_stream_files_are_refused(tmp_path, damage):
    s = _stream()
    p = tmp_path / "c.stream"
    cg.save_stream(p, s)
    raw = bytearray(p.read_bytes())
    if damage == "payload":
        raw[-5] ^= 0x40
    elif damage == "truncate":
        raw = raw[:-4]
    elif damage == "magic":
        raw[0:8] = b"CSMVXXXX"
    elif damage == "version":
        raw[8] = 2
    else:
        raw += b"\0\0\0\0"
    p.write_bytes(bytes(raw))
    with pytest.raises(cg.CsmvError) as e:
        cg.load_stream(p)
    assert e.value.status == 8


def test_missing_file_and_capacity(tmp_path):
    with pytest.raises(cg.CsmvError) as e:
        cg.load_stream(tmp_path / "none.stream")
    assert e.value.status == 8
    s = _stream()
    p = tmp_path / "d.stream"
    cg.save_stream(p, s)
    L = cg.lib()
    op = np.empty(s.n_txn, np.uint32)
    off = np.empty(s.n_txn, np.uint32)
    addr = np.empty(s.addr.shape[0], np.uint32)
    rc = L.csmv_stream_load(str(p).encode(), op.ctypes.data, off.ctypes.data, addr.ctypes.data,
                            s.n_txn - 32, addr.shape[0])
    assert rc == 5  # CSMV_ERR_CAPACITY
    rc = L.csmv_stream_load(str(p).encode(), op.ctypes.data, off.ctypes.data, addr.ctypes.data,
                            s.n_txn, addr.shape[0] - 1)
    assert rc == 5


def test_log_round_trip_and_damage(tmp_path):
    rng = np.random.default_rng(1)
    log_txn = rng.integers(0, 1 << 20, 300, dtype=np.uint32)
    log_txn[::7] = cg.HOLE
    outcome = rng.integers(0, 1 << 32, 256, dtype=np.uint64).astype(np.uint32)
    result = rng.integers(-(1 << 31), 1 << 31, 256, dtype=np.int64).astype(np.int32)
    p = tmp_path / "a.log"
    cg.save_log(p, 1234, log_txn, outcome, result)
    base, lt, oc, rs = cg.load_log(p)
    assert base == 1234
    np.testing.assert_array_equal(lt, log_txn)
    np.testing.assert_array_equal(oc, outcome)
    np.testing.assert_array_equal(rs, result)
    raw = bytearray(p.read_bytes())
    assert raw[:8] == b"CSMVCLOG"
    raw[40] ^= 1
    p.write_bytes(bytes(raw))
    with pytest.raises(cg.CsmvError) as e:
        cg.load_log(p)
    assert e.value.status == 8


def test_empty_log(tmp_path):
    p = tmp_path / "e.log"
    cg.save_log(p, 0, np.zeros(0, np.uint32), np.zeros(0, np.uint32), np.zeros(0, np.int32))
    base, lt, oc, rs = cg.load_log(p)
    assert base == 0 and lt.size == 0 and oc.size == 0 and rs.size == 0


def test_cpu_replay_of_a_stream_file_matches_the_original(tmp_path):
    """A stream read back from its file runs to the same balances in the oracle's stream-order
    execution as the stream it was written from."""
    s = _stream(seed=8, n=32 * 256)
    p = tmp_path / "f.stream"
    cg.save_stream(p, s)
    t = cg.load_stream(p)
    init = np.full(512, 1000, np.int32)
    a, _ = orc.serial(s.op, s.off, s.addr, 512, init)
    b, _ = orc.serial(t.op, t.off, t.addr, 512, init)
    np.testing.assert_array_equal(a, b)
