"""Entropy, GoogleStats, Print, ExportAmplitudes and dumpbin against the reference's own
outputs (tests/golden/state_io.npz, made by tests/golden/make_state_io.py): the statistics
to rounding, the printed and exported text character for character."""
import json

import numpy as np
import pytest

from conftest import REPO

pytestmark = pytest.mark.gpu

FIX = REPO / "tests" / "golden" / "state_io.npz"


def cases():
    z = np.load(FIX)
    return sorted({k.split("/")[0] for k in z.files})


def register(name):
    import iqs_gb300 as iqs
    z = np.load(FIX)
    meta = json.loads(str(z[f"{name}/meta"]))
    r = iqs.QubitRegister(meta["n"], "base", 0, precision=meta["precision"])
    r.SetStateVector(z[f"{name}/init"])
    if meta["perm"] is not None:
        r.PermuteQubits(meta["perm"])
    return r, meta, {k.split("/", 1)[1]: z[k] for k in z.files if k.startswith(name + "/")}


@pytest.mark.parametrize("name", cases())
def test_stats_match_reference(name):
    r, meta, d = register(name)
    tol = 1e-12 if meta["precision"] == "DP" else 2e-5
    got = np.asarray(r.GoogleStats())
    want = d["stats"]
    assert got.shape == want.shape
    assert np.max(np.abs(got - want) / np.maximum(1.0, np.abs(want))) <= tol
    assert abs(r.Entropy() - meta["entropy"]) <= tol * max(1.0, meta["entropy"])


@pytest.mark.parametrize("name", cases())
def test_print_and_export_text_match_reference(name, capsys, tmp_path):
    r, meta, d = register(name)
    r.Print(name)
    assert capsys.readouterr().out == str(d["print"])
    f = tmp_path / "amps.json"
    r.ExportAmplitudes(str(f))
    assert f.read_text() == str(d["export"])


def test_dumpbin_round_trip(tmp_path, capsys):
    r, meta, d = register("dp5_perm")
    f = tmp_path / "state.bin"
    r.dumpbin(str(f))
    assert capsys.readouterr().out.startswith(f"Dumping state to {f} took ")
    assert np.array_equal(np.fromfile(f, dtype=np.complex128), r.GetStateVector())
