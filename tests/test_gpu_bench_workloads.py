"""Every bench.py workload runs end to end on a small batch: the process exits 0 and prints one JSON
line with a positive value, and the workloads that check their results against the oracle report
equality (guards the bench paths that no other test drives)."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
WORKLOADS = ["affine_dna_100k", "linear_dna_1024x150", "protein_local_tb_20k", "banded_reads_1m", "xdrop_reads_1m",
             "extend_reads_250k", "waterman_eggert_10k", "waterman_eggert_banded_10k", "banded_chain_20k",
             "sam_records_1m", "fasta_reads_2m", "dynamic_dna_tb_100k", "bam_records_1m"]


@pytest.mark.parametrize("workload", WORKLOADS)
def test_workload_runs(engine, workload):
    cmd = [sys.executable, "bench.py", "--workload", workload, "--pairs", "2000", "--steps", "1", "--warmup", "3",
           "--no-cpu-baseline", "--no-plain", "--no-serving"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1])
    assert line["value"] > 0
    for key in ("parity_vs_oracle", "parity_first_300_vs_oracle"):
        if key in line:
            assert line[key] is True, key
    if isinstance(line.get("parity"), dict):
        assert line["parity"].get("equal") is True
