"""The multi-GPU task layer of the drop-in API (fap::fapGraphMoreTask,
include/fap/fap_more_task.h; reference fapGraphMoreTaskMPI,
fap/fap_more_task_mpi.h:23-50): cost-balanced assignment of parts to
processes, metadata broadcast through the caller's collective, and solves of
every process's parts on its own engine."""
import subprocess

import pytest
from conftest import ROOT

LIB = ROOT / "fastapsp_gb300"


def _build(tmp_path):
    exe = tmp_path / "more_task_check"
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", str(ROOT / "include"),
                        str(ROOT / "tests" / "more_task_check.cpp"), "-L", str(LIB), "-lfastapsp",
                        f"-Wl,-rpath,{LIB}", "-pthread", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_more_task_assignment_and_broadcast(tmp_path):
    if not (LIB / "libfastapsp.so").exists():
        pytest.skip("library not built")
    r = subprocess.run([str(_build(tmp_path)), "cpu"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "OK" in r.stdout, r.stdout + r.stderr


@pytest.mark.gpu
def test_more_task_solve_matches_single_solve(gpu, tmp_path):
    r = subprocess.run([str(_build(tmp_path)), "gpu"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "OK" in r.stdout, r.stdout + r.stderr
