"""The drop-in C++ fap::fapGraph (include/fap/fap.h) driven by the example
application with the reference's command line, against the reference's own
outputs (golden fixtures)."""
import subprocess

import numpy as np
import pytest
from conftest import ROOT, load_golden

from fastapsp_gb300 import graphs

pytestmark = pytest.mark.gpu

APP = ROOT / "fastapsp_gb300" / "fap_single_node"


@pytest.mark.parametrize("name,version", [("knn300_dir_int", "false"), ("grid12_tree", "true"),
                                          ("road300_f32", "true")])
def test_example_app_matches_reference(gpu, tmp_path, name, version):
    z, g = load_golden(name)
    typ = ("weight-" if g.weighted else "unweight-") + ("directed" if g.directed else "undirected")
    (tmp_path / "graph" / typ).mkdir(parents=True)
    graphs.write_mtx(g, str(tmp_path / "graph" / typ / f"{name}.mtx"))
    out = tmp_path / "out"
    out.mkdir()
    r = subprocess.run([str(APP), "-f", name, "-k", str(int(z["K"])), "-direct",
                        "true" if g.directed else "false", "-weight", "true" if g.weighted else "false",
                        "-partitioner", "metis", "-version", version, "-dump", str(out)],
                       cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "subGraph is right" in r.stdout
    n = g.n
    assert np.array_equal(np.fromfile(out / "mapping.i32", "<i4"), z["mapping"])
    d = np.fromfile(out / "dist.f32", "<f4").reshape(n, n)
    if name.endswith("f32"):
        fin = z["dist"] < 1e8
        assert np.array_equal(fin, d < 1e8)
        assert np.max(np.abs(d[fin] - z["dist"][fin]) / np.maximum(z["dist"][fin], 1e-30)) <= 1e-6
    else:
        assert np.array_equal(d, z["dist"])


def test_example_app_rejects_unknown_partitioner(gpu, tmp_path):
    (tmp_path / "graph" / "unweight-undirected").mkdir(parents=True)
    graphs.write_mtx(graphs.grid_graph(4, 4), str(tmp_path / "graph" / "unweight-undirected" / "g.mtx"))
    r = subprocess.run([str(APP), "-f", "g", "-k", "2", "-partitioner", "nope"], cwd=tmp_path,
                       capture_output=True, text=True)
    assert r.returncode == 2 and "Invalid partitioner" in r.stderr
