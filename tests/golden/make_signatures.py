"""Regenerate tests/golden/signatures.json from the reference's own recorded
first-solve signatures (Study/result/btdma_solution_signature_260702_193138.csv
of PaScaL_BTDMA).  Run in a checkout where the reference is mounted:

    python tests/golden/make_signatures.py /path/to/PaScaL_BTDMA

Each row was written by the reference CUDA C++ port
(Study/example_cuda_cxx_btdma_profile.cu:76-160) after one non-cyclic solve of
the diagonal workload A = 0.25 I, B = 2 I, C = 0.25 I, d = 1 on nsys = n1*n2
systems of n3 block rows split over `nranks` MPI ranks.  The JSON keeps the
shape, the rank count (= nseg here) and the six signature numbers.
"""
import csv
import json
import sys
from pathlib import Path

src = Path(sys.argv[1]) / "Study/result/btdma_solution_signature_260702_193138.csv"
rows = []
with open(src) as f:
    for r in csv.DictReader(f):
        if r["mpi_mode"] != "device":
            continue
        rows.append({
            "nseg": int(r["nranks"]), "n1": int(r["n1"]), "n2": int(r["n2"]), "n3": int(r["n3"]),
            "m": int(r["m"]), "nsys": int(r["nsys"]),
            "solution_sum": float(r["solution_sum"]), "solution_l2": float(r["solution_l2"]),
            "solution_linf": float(r["solution_linf"]), "sample_z0": float(r["sample_z0"]),
            "sample_zmid": float(r["sample_zmid"]), "sample_zlast": float(r["sample_zlast"]),
        })
out = Path(__file__).resolve().parent / "signatures.json"
out.write_text(json.dumps({"source": "Study/result/btdma_solution_signature_260702_193138.csv",
                           "workload": "A=0.25I, B=2I, C=0.25I, d=1", "rows": rows}, indent=1) + "\n")
print(f"wrote {len(rows)} rows to {out}")
