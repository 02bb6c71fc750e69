"""
Equivalent sources on the CPU: the estimator's host logic (checks of
``depth``, default depth, memory estimate, unsupported options) mirroring
test/test_eq_sources_cartesian.py of the reference.
"""

import numpy as np
import numpy.testing as npt
import pytest

from harmonica_gb300.equivalent_sources import EquivalentSources, EquivalentSourcesSph


def test_invalid_depth():
    """test/test_eq_sources_cartesian.py:462-470."""
    with pytest.raises(ValueError, match="Found invalid 'depth' value equal to 'blabla'"):
        EquivalentSources(depth="blabla")


def test_zero_depth():
    """test/test_eq_sources_cartesian.py:472-480."""
    with pytest.raises(ValueError, match="Depth value cannot be zero"):
        EquivalentSources(depth=0)


def test_default_depth_and_points():
    """Sources 4.5 x the mean nearest-neighbour distance below the data
    (cartesian.py:283-324), checked by brute force."""
    rng = np.random.default_rng(3)
    e, n = rng.uniform(0, 1e4, 60), rng.uniform(0, 1e4, 60)
    u = rng.uniform(100, 300, 60)
    eqs = EquivalentSources()
    pts = eqs._build_points((e, n, u))
    d = np.hypot(e[:, None] - e[None, :], n[:, None] - n[None, :])
    np.fill_diagonal(d, np.inf)
    npt.assert_allclose(eqs.depth_, 4.5 * d.min(axis=1).mean(), rtol=1e-12)
    npt.assert_allclose(pts[2], u - eqs.depth_)
    eqs = EquivalentSources(depth=500)
    npt.assert_allclose(eqs._build_points((e, n, u))[2], u - 500)


def test_memory_estimation():
    """test/test_eq_sources_cartesian.py:484-498 and the docstring example
    (cartesian.py:193-234): n_data x n_points x itemsize."""
    rng = np.random.default_rng(42)
    coords = (rng.uniform(-1e3, 3e3, 100), rng.uniform(2e3, 5e3, 100), np.full(100, 100.0))
    assert EquivalentSources().estimate_required_memory(coords) == 80000
    assert EquivalentSources(dtype="float32").estimate_required_memory(coords) == 40000
    sph = EquivalentSourcesSph()
    assert sph.estimate_required_memory(coords) == 80000


def test_unsupported_options():
    with pytest.raises(NotImplementedError, match="block_size"):
        EquivalentSources(block_size=100)._build_points((np.zeros(2), np.zeros(2), np.zeros(2)))
    with pytest.raises(NotImplementedError):
        EquivalentSources().grid((0, 1, 0, 1))


def test_predict_before_fit():
    with pytest.raises(ValueError, match="not fitted yet"):
        EquivalentSources().predict((np.zeros(1), np.zeros(1), np.zeros(1)))
