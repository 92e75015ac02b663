"""The oracle reproduces the committed golden fixture (tests/golden/).

The fixture was written by tests/golden/make_golden.py; a change to the
oracle or to the seeded generators that moves any number shows up here."""
import os

import numpy as np
import pytest

from tests.golden import make_golden

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "oracle_small.npz")

INT_KEYS = ("nneighpn", "pairs", "seed")


@pytest.fixture(scope="module")
def fresh(orc):
    return make_golden.make(orc)


def test_fixture_keys(fresh):
    g = np.load(GOLDEN)
    assert sorted(g.files) == sorted(fresh)


@pytest.mark.parametrize("key", sorted(np.load(GOLDEN).files))
def test_oracle_reproduces_fixture(fresh, key):
    ref = np.load(GOLDEN)[key]
    got = np.asarray(fresh[key])
    assert got.shape == ref.shape
    if _is_input(key) or key.endswith(INT_KEYS):
        assert np.array_equal(got, ref), key          # generated inputs and integers: exact
    else:
        scale = max(np.abs(ref).max(), 1e-300)
        assert np.abs(got - ref).max() <= 1e-12 * scale, key


def _is_input(key):
    """Seeded inputs: the UTotal cases' positions and the integrators' start."""
    group, name = key.split("/")
    return name in ("ro0", "rod0") or (name == "ro" and group not in ("bd", "md"))
