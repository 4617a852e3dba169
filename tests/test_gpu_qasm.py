"""The QASM front end on the GPU: a script's MeasZ probabilities against the oracle running
the same gates, with operand names mapped to positions in order of first use."""
import math
import subprocess
import sys

import numpy as np
import pytest

import oracle
from conftest import REPO

pytestmark = pytest.mark.gpu

SCRIPT = """qubit a
.malloc 4
H a
CNOT a,b
T b
H c
Tdag c
S a
CNOT c,d
X d
H b
PrepZ a
MeasZ a
MeasZ b
MeasZ c
MeasZ d
.free
.malloc 2
H d
MeasZ a
.free
"""


def test_qasm_script_matches_oracle():
    sys.path.insert(0, str(REPO / "intel-qs_gb300"))
    import iqsg_build
    exe = iqsg_build.build_qasm()
    r = subprocess.run([str(exe)], input=SCRIPT, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.splitlines()
    probs = [float(l.strip("()").split(",")[0]) for l in lines if l.startswith("(")]
    o = oracle.OracleRegister(4, "base", 0)
    o.ApplyHadamard(0)
    o.ApplyCPauliX(0, 1)
    o.ApplyT(1)
    o.ApplyHadamard(2)
    o.ApplyRotationZ(2, -0.785398163397448)
    o.ApplyPauliSqrtZ(0)
    o.ApplyCPauliX(2, 3)
    o.ApplyPauliX(3)
    o.ApplyHadamard(1)
    want = [o.GetProbability(q) for q in range(4)]
    assert len(probs) == 5
    assert np.max(np.abs(np.asarray(probs[:4]) - want)) <= 1e-6  # printed with 6 significant digits
    # second register: 2 qubits, "d" is position 3 -> out of range, "a" still position 0
    assert "Qasm Op failed - [H]" in r.stderr
    assert probs[4] == 0.0
    assert lines.count("Allocated [4] qubits.") == 1 and lines.count("Qubits successfully free.") == 2
