"""The MatrixMarket reader's binary CSR cache (<file>.fapcsr beside the
file; fap/utils/readMatFile.h:66-173 is the reader it replaces): the first
read parses the text (on several threads) and writes the cache, later reads
of the unchanged file load it, and a changed file, another reading mode or a
damaged cache falls back to the parse.  Every read is checked against the
oracle's restatement of the reference reader.  No GPU."""
import os
import time

import numpy as np
import pytest

from fastapsp_gb300 import graphs


def _same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


@pytest.fixture
def mtx(tmp_path):
    g = graphs.road_like(30000, seed=5)
    path = tmp_path / "road.mtx"
    graphs.write_mtx(g, str(path))
    return path, g


def test_cache_written_and_used(fap_lib, oracle_lib, mtx):
    path, g = mtx
    cache = path.with_name(path.name + ".fapcsr")
    ref = oracle_lib.mtx_read(path, False, True)
    t0 = time.perf_counter()
    first = fap_lib.mtx_read(str(path), False, True)
    t1 = time.perf_counter()
    assert _same(first, ref)
    assert cache.exists()
    second = fap_lib.mtx_read(str(path), False, True)
    t2 = time.perf_counter()
    assert _same(second, ref)
    print(f"parse {1e3 * (t1 - t0):.1f} ms, cached {1e3 * (t2 - t1):.1f} ms")
    # the cache is what the second read returned: a planted change shows up ...
    raw = bytearray(cache.read_bytes())
    raw[-4:] = np.float32(123.5).tobytes()
    cache.write_bytes(bytes(raw))
    st = path.stat()
    os.utime(path, ns=(st.st_atime_ns, st.st_mtime_ns))  # keep the stamp the cache records
    planted = fap_lib.mtx_read(str(path), False, True)
    assert planted[2][-1] == np.float32(123.5)
    # ... until the file changes (new stamp): parsed again, cache rewritten
    os.utime(path, ns=(st.st_atime_ns, st.st_mtime_ns + 1_000_000))
    assert _same(fap_lib.mtx_read(str(path), False, True), ref)
    assert _same(fap_lib.mtx_read(str(path), False, True), ref)


def test_other_reading_mode_and_damaged_cache(fap_lib, oracle_lib, mtx):
    path, g = mtx
    cache = path.with_name(path.name + ".fapcsr")
    und = fap_lib.mtx_read(str(path), False, True)
    dire = fap_lib.mtx_read(str(path), True, True)  # same file read as directed: its own CSR
    assert _same(dire, oracle_lib.mtx_read(path, True, True))
    assert _same(fap_lib.mtx_read(str(path), False, True), und)
    cache.write_bytes(cache.read_bytes()[:100])  # truncated
    assert _same(fap_lib.mtx_read(str(path), False, True), oracle_lib.mtx_read(path, False, True))


def test_cache_can_be_turned_off(fap_lib, oracle_lib, mtx, monkeypatch):
    path, g = mtx
    monkeypatch.setenv("FAP_MTX_CACHE", "0")
    assert _same(fap_lib.mtx_read(str(path), False, True), oracle_lib.mtx_read(path, False, True))
    assert not path.with_name(path.name + ".fapcsr").exists()
