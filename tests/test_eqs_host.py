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


def _verde_least_squares(jacobian, data, weights, damping):
    """verde's least-squares step, stated with the scikit-learn classes it
    is built on: features scaled by their standard deviation (no centring),
    an ordinary least-squares or ridge regression without intercept fitted
    with the sample weights, then the coefficients divided by the scales."""
    from sklearn.linear_model import LinearRegression, Ridge
    from sklearn.preprocessing import StandardScaler

    scaler = StandardScaler(copy=True, with_mean=False, with_std=True)
    scaled = scaler.fit_transform(jacobian)
    if damping is None:
        regr = LinearRegression(fit_intercept=False)
    else:
        regr = Ridge(alpha=damping, fit_intercept=False)
    regr.fit(scaled, data.ravel(), sample_weight=weights)
    return regr.coef_ / scaler.scale_


@pytest.mark.parametrize("damping", [None, 1e-3, 10.0])
@pytest.mark.parametrize("weighted", [False, True])
def test_least_squares_matches_verde_algorithm(damping, weighted):
    """The fit's solver (torch, run here on CPU tensors) against the
    scikit-learn statement of verde's least squares, on a 1/distance
    Jacobian of sources below scattered data with noise in the data."""
    pytest.importorskip("sklearn")
    import torch

    from harmonica_gb300.equivalent_sources import _least_squares

    rng = np.random.default_rng(42)
    n_data, n_src = 120, 40
    data_xyz = np.stack([rng.uniform(0, 5e3, n_data), rng.uniform(0, 5e3, n_data),
                         rng.uniform(0, 50, n_data)])
    src_xyz = np.stack([rng.uniform(0, 5e3, n_src), rng.uniform(0, 5e3, n_src),
                        np.full(n_src, -1e3)])
    jac = 1 / np.linalg.norm(data_xyz[:, :, None] - src_xyz[:, None, :], axis=0)
    data = jac @ rng.normal(0, 1e5, n_src) + rng.normal(0, 1.0, n_data)
    weights = rng.uniform(0.5, 2.0, n_data) if weighted else None
    expected = _verde_least_squares(jac, data, weights, damping)
    got = _least_squares(torch.from_numpy(jac), torch.from_numpy(data),
                         None if weights is None else torch.from_numpy(weights), damping)
    # ridge: torch solves the normal equations, scikit-learn a Cholesky of
    # the same matrix; cond(scaled Jacobian) ~1e4 here, so 1e-8 leaves room
    # for the squared condition number (measured: 2e-10 at damping 1e-3)
    npt.assert_allclose(got.numpy(), expected, rtol=0, atol=1e-8 * np.abs(expected).max())
    npt.assert_allclose(jac @ got.numpy(), jac @ expected, rtol=0,
                        atol=1e-11 * np.abs(data).max())


def test_least_squares_constant_column():
    """A column with zero spread keeps a scale of one (no division by zero),
    as the standard scaler does."""
    pytest.importorskip("sklearn")
    import torch

    from harmonica_gb300.equivalent_sources import _least_squares

    rng = np.random.default_rng(3)
    jac = rng.normal(size=(30, 5))
    jac[:, 2] = 0.7
    data = rng.normal(size=30)
    expected = _verde_least_squares(jac, data, None, 0.5)
    got = _least_squares(torch.from_numpy(jac), torch.from_numpy(data), None, 0.5)
    npt.assert_allclose(got.numpy(), expected, rtol=1e-10, atol=1e-12)


def test_oracle_matches_reference_golden():
    """The oracle against harmonica's own jacobian/predict loops and Green's
    functions run from the reference sources (tests/golden/make_eqs_golden.py):
    the Jacobians bit for bit, the predictions to the rounding of the sum
    order (the reference adds coefficient x Green's function source by
    source; the oracle uses a matrix product)."""
    import os

    from oracle import eqs_oracle

    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_eqs.npz"))
    for name, spherical in (("cart", False), ("sph", True)):
        data, src = g[f"{name}_data"], g[f"{name}_src"]
        npt.assert_array_equal(eqs_oracle.jacobian(data, src, spherical=spherical),
                               g[f"{name}_jacobian"])
        ref = g[f"{name}_predict"]
        npt.assert_allclose(eqs_oracle.predict(data, src, g["coefs"], spherical=spherical), ref,
                            rtol=0, atol=1e-14 * np.abs(ref).max())
