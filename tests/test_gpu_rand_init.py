"""Initialize("rand") against the reference's own random states (tests/golden/rand_init.npz,
made by tests/golden/make_rand_init.py): same seeds, same streams, the same numbers."""
import json

import numpy as np
import pytest

from conftest import REPO

pytestmark = pytest.mark.gpu

FIX = REPO / "tests" / "golden" / "rand_init.npz"


def cases():
    return sorted({k.split("/")[0] for k in np.load(FIX).files})


@pytest.mark.parametrize("name", cases())
def test_random_states_match_reference(name):
    import iqs_gb300 as iqs
    z = np.load(FIX)
    meta = json.loads(str(z[f"{name}/meta"]))
    r = iqs.QubitRegister(meta["n"], "base", 0, precision=meta["precision"])
    rng = iqs.RandomNumberGenerator()
    rng.SetSeedStreamPtrs(meta["seed"])
    r.SetRngPtr(rng)
    for _ in range(meta["times"]):
        r.Initialize("rand", meta["base_index"])
    tol = 1e-14 if meta["precision"] == "DP" else 1e-6
    assert np.max(np.abs(r.GetStateVector() - z[f"{name}/state"])) <= tol
    stream = "pool" if meta["base_index"] == 0 else "local"
    counts = {"pool": rng.GetNumGeneratedOrSkippedPoolNumbers(), "local": rng.GetNumGeneratedOrSkippedLocalNumbers()}
    assert counts[stream] == 2 * (1 << meta["n"]) * meta["times"]


def test_random_init_requires_a_seeded_generator():
    import iqs_gb300 as iqs
    r = iqs.QubitRegister(4, "base", 0)
    with pytest.raises(ValueError):
        r.Initialize("rand", 0)
    rng = iqs.RandomNumberGenerator()
    r.SetRngPtr(rng)
    with pytest.raises(ValueError):  # seed 0, which the reference asserts against
        r.Initialize("rand", 0)
    rng.SetSeedStreamPtrs(5)
    with pytest.raises(ValueError):
        r.Initialize("rand", 2)
    r.Initialize("rand", 0)
    assert abs(r.ComputeNorm() - 1.0) <= 1e-14
