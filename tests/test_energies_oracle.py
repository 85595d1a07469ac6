"""Pinning of the template-energy oracle against numpy itself (CPU)."""
import numpy as np
import pytest

from oracle.energies import pairwise_sum, template_energies


@pytest.mark.parametrize("L", list(range(1, 20)) + [64, 127, 128, 129, 135, 255, 256, 257, 600,
                                                    801, 1200, 4097])
def test_pairwise_sum_is_numpy_sum(L):
    rng = np.random.default_rng(L)
    x = (rng.standard_normal((6, L)) * np.exp(rng.uniform(-4, 4, (6, L)))).astype(np.float32)
    for row in x:
        assert pairwise_sum(row ** 2) == np.sum(row ** 2)


def test_template_energies_4d():
    rng = np.random.default_rng(1)
    t = rng.standard_normal((3, 4, 2, 601)).astype(np.float32)
    assert np.array_equal(template_energies(t), np.sum(t ** 2, axis=-1))
