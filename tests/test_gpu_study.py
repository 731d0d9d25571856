"""The Study-compatible profiling driver (python -m pascal_btdma_gb300.study)
against the reference Study's CSV schemas (Study/README.md:133-148, writer
Study/example_cuda_cxx_btdma_profile.cu:76-160, 230-289) and its recorded
solution signatures (tests/golden/signatures.json, copied from
Study/result/btdma_solution_signature_260702_193138.csv).

Each case runs the driver as the Study scripts do (a child process with the
positional arguments n1 n2 n3 m iters) and checks: the timing header and
column order, one row per iteration, compute_s_max = local + reduced + update
and communication_s_max = forward + backward exchange, total >= compute; the
signature file's header and the row of the first solve against the
reference's row for the same (m, n3, nseg, nsys) -- sums at 1e-9 relative
(the reference's own spread across rank counts), samples at 1e-14."""
import csv
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]
GOLDEN = json.loads((ROOT / "tests" / "golden" / "signatures.json").read_text())

# The two CSV schemas of Study/README.md:133-148 (an interface: the Study's
# analysis scripts read these columns by name and position).
TIMING_HEADER = ("solver,variant,implementation,nranks,n1,n2,n3,m,nsys,nrow_min,nrow_max,iter,iterations,"
                 "mpi_mode,total_s_max,total_s_avg,local_compute_s_max,forward_exchange_s_max,"
                 "reduced_compute_s_max,backward_exchange_s_max,update_compute_s_max,compute_s_max,"
                 "communication_s_max")
SIGNATURE_HEADER = ("solver,variant,implementation,nranks,n1,n2,n3,m,nsys,nrow_min,nrow_max,mpi_mode,"
                    "solution_sum,solution_l2,solution_linf,sample_z0,sample_zmid,sample_zlast")


def golden_row(m, n3, nseg, nsys):
    for r in GOLDEN["rows"]:
        if (r["m"], r["n3"], r["nseg"], r["nsys"]) == (m, n3, nseg, nsys):
            return r
    raise KeyError((m, n3, nseg, nsys))


@pytest.mark.parametrize("m,n3,nseg", [(2, 128, 1), (3, 128, 1), (5, 128, 1), (8, 128, 1), (5, 2048, 8),
                                       (2, 2048, 8)])
def test_study_driver_schema_and_signature(cuda, tmp_path, m, n3, nseg):
    n1 = n2 = 32
    iters = 3
    sig = tmp_path / "sig.csv"
    env = dict(os.environ, PYTHONPATH=str(ROOT))
    res = subprocess.run([sys.executable, "-m", "pascal_btdma_gb300.study", str(n1), str(n2), str(n3), str(m),
                          str(iters), "--nseg", str(nseg), "--signature-out", str(sig)],
                         cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr
    lines = [ln for ln in res.stdout.splitlines() if ln.strip()]
    assert lines[0] == TIMING_HEADER
    rows = list(csv.DictReader(lines))
    assert len(rows) == iters
    for it, r in enumerate(rows):
        assert list(r) == TIMING_HEADER.split(",")
        assert (r["solver"], r["variant"], r["mpi_mode"]) == ("btdma", "noncyclic", "device")
        assert int(r["iter"]) == it and int(r["iterations"]) == iters
        assert (int(r["nranks"]), int(r["n1"]), int(r["n2"]), int(r["n3"]), int(r["m"]), int(r["nsys"])) == \
            (nseg, n1, n2, n3, m, n1 * n2)
        lo, hi = n3 // nseg, -(-n3 // nseg)
        assert (int(r["nrow_min"]), int(r["nrow_max"])) == (lo, hi)
        v = {k: float(r[k]) for k in TIMING_HEADER.split(",")[14:]}
        assert v["total_s_max"] == v["total_s_avg"] and v["total_s_max"] > 0
        comp = v["local_compute_s_max"] + v["reduced_compute_s_max"] + v["update_compute_s_max"]
        comm = v["forward_exchange_s_max"] + v["backward_exchange_s_max"]
        assert v["compute_s_max"] == pytest.approx(comp, rel=1e-9, abs=1e-12)
        assert v["communication_s_max"] == pytest.approx(comm, rel=1e-9, abs=1e-12)
        assert v["total_s_max"] >= comp * (1 - 1e-6)
        if nseg == 1:
            assert v["reduced_compute_s_max"] == 0.0 and v["update_compute_s_max"] == 0.0
        else:
            assert v["reduced_compute_s_max"] > 0 and v["update_compute_s_max"] > 0
    sig_lines = sig.read_text().splitlines()
    assert sig_lines[0] == SIGNATURE_HEADER and len(sig_lines) == 2
    got = next(csv.DictReader(sig_lines))
    ref = golden_row(m, n3, nseg, n1 * n2)
    for key in ("solution_sum", "solution_l2"):
        assert float(got[key]) == pytest.approx(ref[key], rel=1e-9)
    for key in ("solution_linf", "sample_z0", "sample_zmid", "sample_zlast"):
        assert float(got[key]) == pytest.approx(ref[key], rel=1e-14, abs=1e-15)
