"""The allocation-free SSSP entry point (fap_sssp_noalloc).

It exists for callers that cannot call cudaMalloc -- code running under a
memory pool or arena it does not own, plugin request paths that forbid
allocation, real-time paths -- so it takes every piece of scratch from a
fixed static device array instead.  These tests call it through the C ABI:

* twice in a row on graph arrays the test owns, each result checked against
  the allocating entry point fap_sssp (distances and predecessors bit for
  bit: the same kernel runs on both);
* in a fresh process that never creates an engine (so nothing else has set
  up the SSSP kernels on the device), checked against the oracle's Dijkstra;
* with a graph beyond the static array, which must be rejected.

The file sorts last so that a run stopping at the first failure has already
run every other test."""
import json
import os
import subprocess
import sys
import textwrap
from pathlib import Path

import numpy as np
import pytest
import torch

from fastapsp_gb300 import graphs
from fastapsp_gb300._lib import FAP_ERR_RANGE, FAP_OK, lib

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]


def _device_csr(g, int_weights):
    ro = torch.from_numpy(g.row_offset).cuda()
    col = torch.from_numpy(g.col_val).cuda()
    if int_weights:
        w = torch.from_numpy(g.weight.astype(np.int32)).cuda()
    else:
        w = torch.from_numpy(g.weight).cuda()
    # in-edge CSR (sources ascending per target), for the predecessors
    src = np.repeat(np.arange(g.n), np.diff(g.row_offset))
    order = np.lexsort((src, g.col_val))
    iro = np.zeros(g.n + 1, np.int64)
    np.add.at(iro, g.col_val + 1, 1)
    iro = np.cumsum(iro).astype(np.int32)
    icol = src[order].astype(np.int32)
    iw = g.weight[order]
    iw = iw.astype(np.int32) if int_weights else iw.astype(np.float32)
    return ro, col, w, torch.from_numpy(iro).cuda(), torch.from_numpy(icol).cuda(), torch.from_numpy(iw).cuda()


@pytest.mark.parametrize("kind", ["grid_i32", "road_f32"])
def test_noalloc_sssp_matches_allocating_entry_point_twice(gpu, kind):
    if kind == "grid_i32":
        g, dtype = graphs.grid_graph(60, 60, seed=3), gpu.DTYPE_I32
    else:
        g, dtype = graphs.road_like(6000, seed=4), gpu.DTYPE_F32
    rng = np.random.default_rng(1)
    src = np.ascontiguousarray(rng.choice(g.n, size=77, replace=False).astype(np.int32))
    dt = torch.int32 if dtype == gpu.DTYPE_I32 else torch.float32
    with gpu.Engine(g.n, g.row_offset, g.col_val, g.weight, 2, dtype=dtype) as eng:
        ref_d = torch.empty((len(src), g.n), dtype=dt, device="cuda")
        ref_p = torch.empty((len(src), g.n), dtype=torch.int32, device="cuda")
        eng.sssp(src, ref_d, ref_p)
    torch.cuda.synchronize()
    ro, col, w, iro, icol, iw = _device_csr(g, dtype == gpu.DTYPE_I32)
    for call in range(2):
        d = torch.full((len(src), g.n), 7, dtype=dt, device="cuda")
        p = torch.full((len(src), g.n), 7, dtype=torch.int32, device="cuda")
        rc = lib().fap_sssp_noalloc(dtype, g.n, g.m, ro.data_ptr(), col.data_ptr(), w.data_ptr(),
                                    iro.data_ptr(), icol.data_ptr(), iw.data_ptr(),
                                    src.ctypes.data, len(src), d.data_ptr(), p.data_ptr(), g.n, None)
        assert rc == FAP_OK, lib().fap_last_error()
        torch.cuda.synchronize()
        assert torch.equal(d, ref_d), f"distances differ on call {call}"
        assert torch.equal(p, ref_p), f"predecessors differ on call {call}"


# Runs in a fresh interpreter: loads the library, never creates an engine or a
# context object, calls fap_sssp_noalloc twice and saves what it returned.
_CHILD = textwrap.dedent("""
    import json, sys
    import numpy as np, torch
    sys.path.insert(0, {root!r})
    sys.path.insert(0, {tests!r})
    from fastapsp_gb300 import graphs
    from fastapsp_gb300._lib import lib
    from test_zz_no_alloc import _device_csr
    g = graphs.grid_graph(40, 40, seed=9)
    src = np.arange(0, g.n, 97, dtype=np.int32)
    torch.cuda.init()
    ro, col, w, iro, icol, iw = _device_csr(g, True)
    out = {{}}
    for call in range(2):
        d = torch.full((len(src), g.n), 7, dtype=torch.int32, device="cuda")
        p = torch.full((len(src), g.n), 7, dtype=torch.int32, device="cuda")
        rc = lib().fap_sssp_noalloc(1, g.n, g.m, ro.data_ptr(), col.data_ptr(), w.data_ptr(),
                                    iro.data_ptr(), icol.data_ptr(), iw.data_ptr(),
                                    src.ctypes.data, len(src), d.data_ptr(), p.data_ptr(), g.n, None)
        out[call] = dict(rc=rc, err=(lib().fap_last_error() or b"").decode())
        torch.cuda.synchronize()
        np.save({out!r} + f".d{{call}}.npy", d.cpu().numpy())
        np.save({out!r} + f".p{{call}}.npy", p.cpu().numpy())
    print(json.dumps(out))
""")


def test_noalloc_sssp_in_a_process_without_an_engine(gpu, oracle_lib, tmp_path):
    out = str(tmp_path / "res")
    code = _CHILD.format(root=str(ROOT), tests=str(ROOT / "tests"), out=out)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600,
                       env=dict(os.environ))
    assert r.returncode == 0, r.stdout + r.stderr
    status = json.loads(r.stdout.strip().splitlines()[-1])
    g = graphs.grid_graph(40, 40, seed=9)
    src = np.arange(0, g.n, 97, dtype=np.int32)
    for call in ("0", "1"):
        assert status[call]["rc"] == FAP_OK, status[call]["err"]
        d = np.load(out + f".d{call}.npy")
        p = np.load(out + f".p{call}.npy")
        for i, s in enumerate(src):
            rd, rp = oracle_lib.dijkstra_path(int(s), g.row_offset, g.col_val, g.weight)
            ref = np.where(rd >= 1e8, 1 << 30, rd).astype(np.int64)
            assert np.array_equal(d[i].astype(np.int64), ref), f"call {call}, source {s}: distances"
            assert np.array_equal(p[i], rp), f"call {call}, source {s}: predecessors"


def test_noalloc_rejects_graphs_beyond_the_static_scratch(gpu):
    # Real device buffers of the declared sizes (an edgeless graph), so that
    # no argument could fault even if the size check moved after a launch.
    n = 1_000_000  # needs about 140 MB of scratch, above the 64 MiB array
    ro = torch.zeros(n + 1, dtype=torch.int32, device="cuda")
    src = np.zeros(1, np.int32)
    d = torch.empty((1, n), dtype=torch.int32, device="cuda")
    rc = lib().fap_sssp_noalloc(gpu.DTYPE_I32, n, 0, ro.data_ptr(), None, None, None, None, None,
                                src.ctypes.data, 1, d.data_ptr(), None, n, None)
    assert rc == FAP_ERR_RANGE
    assert "static scratch" in lib().fap_last_error().decode()
