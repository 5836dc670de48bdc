"""The oracle still reproduces the committed golden vectors (tests/golden/)."""
import os

import numpy as np
import pytest

from golden.make_golden import cases

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def fresh():
    return cases()


@pytest.mark.parametrize("name", ["nufft1d", "nufft2d", "nufft2d_kw6", "nufft3d", "sense", "sho", "haar", "bfista"])
def test_oracle_matches_golden(fresh, name):
    stored = np.load(os.path.join(HERE, f"{name}.npz"))
    for k, v in fresh[name].items():
        np.testing.assert_allclose(np.asarray(v), stored[k], rtol=1e-10, atol=1e-12, err_msg=f"{name}.{k}")
