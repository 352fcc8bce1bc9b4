"""The oracle against its frozen outputs (tests/golden/oracle_small.npz, made
by tests/golden/make_golden.py): residuals, limited gradients and a four-step
trajectory on five small seeded cases, bit for bit.  The GPU parity tests
compare the engine with the oracle; this keeps the oracle itself from moving
unnoticed.  The fixture was made on x86-64 and is checked on this machine
type only (libm's pow may differ in the last bit between architectures)."""
import os
import platform

import numpy as np
import pytest

from tests.golden import make_golden as G

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = os.path.join(HERE, "golden", "oracle_small.npz")

pytestmark = pytest.mark.skipif(platform.machine() not in ("x86_64", "AMD64"),
                                reason="fixture made on x86-64")


@pytest.fixture(scope="module")
def golden():
    return np.load(FIX)


@pytest.mark.parametrize("name", sorted(G.CASES))
def test_oracle_matches_golden(golden, name):
    c = G.CASES[name]()
    assert np.array_equal(c.cv, golden[f"{name}/cv0"]), "case generator changed"
    got = G.compute(c)
    for k, v in got.items():
        want = golden[f"{name}/{k}"]
        assert v.shape == want.shape, (name, k)
        assert np.array_equal(v, want, equal_nan=True), (name, k)
