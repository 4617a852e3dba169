"""The QASM front end (intel-qs_gb300/qasm/iqsg_qasm.cpp) without a GPU: commands that need no
register, argument errors, unknown operations and the end-of-input rule."""
import subprocess
import sys

from conftest import REPO


def qasm(text):
    sys.path.insert(0, str(REPO / "intel-qs_gb300"))
    import iqsg_build
    iqsg_build.build()  # no-op when libiqsg.so is current
    exe = iqsg_build.build_qasm()
    return subprocess.run([str(exe)], input=text, capture_output=True, text=True, timeout=60)


def test_commands_without_a_register():
    r = qasm(".iversion\n.version\nqubit q0\ncbit c0\n")
    assert r.returncode == 0
    out = r.stdout.splitlines()
    assert out[0] == "RC-1.1.0" and out[1].startswith("iqs_gb300 ")
    assert out[2:] == ["Qubit (scaffold syntax): q0", "Cbit (scaffold syntax): c0"]
    assert r.stderr == ""


def test_errors_are_reported_and_skipped():
    r = qasm(".free\nFOO x\n.malloc abc\n.malloc 0\n.malloc 44\nH q0\nCNOT q0,q1\n")
    assert r.returncode == 0
    err = r.stderr.splitlines()
    assert "Harmless attempt to .free before .malloc. Nothing done." in err
    for op in (".free", "FOO", ".malloc", "H", "CNOT"):
        assert f"Qasm Op failed - [{op}]" in err
    assert ".malloc (size) - size parameter was not an integer." in err
    assert err.count(".malloc (size) - allocations in the range from 1..43 only.") == 3
    # gates are echoed before they run, as in the reference; without a register they then fail
    assert r.stdout.splitlines() == ["H [q0]", "CNOT [q0,q1]"]


def test_empty_line_ends_the_program():
    r = qasm(".iversion\n\n.iversion\n")
    assert r.stdout.splitlines() == ["RC-1.1.0"]
