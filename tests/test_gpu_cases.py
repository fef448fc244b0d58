"""The named cases that the ncu summaries under profiles/ are captured on
(python -m proxpde_gb300.cases) run and report their workload."""
import json
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case,n,elements", [("p1tet", 4, 384), ("p2tet", 3, 162), ("q1hex", 5, 125),
                                             ("q2hex", 3, 27)])
def test_assembly_cases(engine, case, n, elements):
    from proxpde_gb300 import cases

    out = cases.run_assembly(case, n, warmup=1, reps=2)
    assert out["case"] == case and out["elements"] == elements and out["ms"] > 0 and out["nnz"] > out["ndof"]


def test_batch_case_cli(engine):
    r = subprocess.run([sys.executable, "-m", "proxpde_gb300.cases", "batch", "--n", "2", "--warmup", "1",
                        "--reps", "1"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["problems"] == 4 and out["ms"] > 0 and out["kernel"] == "kBatchSolve"
