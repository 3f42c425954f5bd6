"""The archive reader (host code only): record scanning and recovery from a record
cut short by an interrupted write."""
import ctypes
import struct

import numpy as np

from rebound_gb300 import _lib


def record(t, N, whfast=False, version=1):
    cfg = _lib.Config()
    _lib.load().rgpu_config_default(ctypes.byref(cfg))
    cfg.t = t
    cfg_bytes = bytes(cfg)
    head_wo_cfg = 8 + 4 + 4 + 8 + 8 + 4 + 4 + 8 + 8 + 8 + 40
    header_bytes = head_wo_cfg + len(cfg_bytes)
    payload = np.arange(N * (11 + (7 if whfast else 0)), dtype=np.float64).tobytes()
    rec_bytes = header_bytes + len(payload)
    head = b"RGPUSNAP" + struct.pack("<IIQQII", version, header_bytes, rec_bytes, N, 4 if whfast else 0,
                                     len(cfg_bytes))
    head += struct.pack("<ddq5d", t, 0.0, 0, 0, 0, 0, 0, 0)
    return head + cfg_bytes + payload


def scan(path):
    L = _lib.load()
    n = ctypes.c_size_t(0)
    L.rgpu_archive_scan(str(path).encode(), None, None, 0, ctypes.byref(n))
    t = np.zeros(n.value)
    off = np.zeros(n.value, dtype=np.int64)
    if n.value:
        assert L.rgpu_archive_scan(str(path).encode(), t.ctypes.data, off.ctypes.data, n.value,
                                   ctypes.byref(n)) == 0
    return t, off


def test_scan_records_and_stop_at_a_cut_record(tmp_path):
    path = tmp_path / "a.bin"
    recs = [record(0.0, 3), record(10.5, 3, whfast=True), record(20.25, 5)]
    blob = b"".join(recs)
    path.write_bytes(blob)
    t, off = scan(path)
    assert list(t) == [0.0, 10.5, 20.25]
    assert list(off) == [0, len(recs[0]), len(recs[0]) + len(recs[1])]
    path.write_bytes(blob + recs[1][: len(recs[1]) // 2])        # interrupted append
    assert list(scan(path)[0]) == [0.0, 10.5, 20.25]
    path.write_bytes(recs[0] + b"garbage!" + recs[1])             # a bad record ends the list
    assert list(scan(path)[0]) == [0.0]
    path.write_bytes(record(1.0, 2, version=7))                  # another layout version is not read
    assert len(scan(path)[0]) == 0


def test_missing_archive_is_an_error(tmp_path):
    L = _lib.load()
    n = ctypes.c_size_t(0)
    assert L.rgpu_archive_scan(str(tmp_path / "none.bin").encode(), None, None, 0, ctypes.byref(n)) != 0


def test_archive_index_by_time(tmp_path):
    # Simulationarchive's bookkeeping (rebound/simulationarchive.py:110-177): length,
    # tmin / tmax, and the snapshot at or before a requested time
    from rebound_gb300 import Simulationarchive
    path = tmp_path / "a.bin"
    path.write_bytes(b"".join(record(t, 2) for t in (0.0, 10.25, 20.5, 30.75)))
    sa = Simulationarchive(path)
    assert len(sa) == 4 and sa.tmin == 0.0 and sa.tmax == 30.75
    assert [sa._snapshot_index(t) for t in (0.0, 5.0, 10.25, 20.49, 29.0, 30.75)] == [0, 0, 1, 1, 2, 3]
    for bad in (-1.0, 31.0):
        try:
            sa._snapshot_index(bad)
        except ValueError:
            pass
        else:
            raise AssertionError("time outside the archive accepted")
    try:
        sa[4]
    except IndexError:
        pass
    else:
        raise AssertionError("index past the end accepted")
