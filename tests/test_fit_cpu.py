"""Host logic of the training loops (gpjax/fit.py:44-361): the softplus
bijection of positive / non-negative parameters, the identity for real ones,
and convergence of fit_scipy / fit_lbfgs / fit on a torch objective (CPU)."""
import numpy as np
import pytest
import torch

import gpjax_gb300 as gpx
from gpjax_gb300 import fit as F
from gpjax_gb300.parameters import NonNegativeReal, PositiveReal, Real


class _Toy:
    def __init__(self):
        self.a = PositiveReal(2.0)
        self.inner = type("Inner", (), {})()
        self.inner.b = Real(np.array([0.5, -0.25]))
        self.inner.c = NonNegativeReal(0.3)


def _objective(model, data):
    a, b, c = model.a.value, model.inner.b.value, model.inner.c.value
    t = torch.as_tensor([-1.0, 2.0], dtype=torch.float64)
    return (a - 3.0) ** 2 + ((b - t) ** 2).sum() + (c - 0.7) ** 2 + (data.X.sum() * 0.0)


def _data():
    return gpx.Dataset(X=np.zeros((4, 1)), y=np.zeros((4, 1)), device="cpu")


def test_unconstrained_round_trip():
    m = _Toy()
    st = F._Unconstrained(m, torch.device("cpu"))
    x = st.flat()
    assert np.isclose(x[0], np.log(np.expm1(2.0)))      # softplus^-1 of the positive value
    assert np.allclose(x[1:3], [0.5, -0.25])            # identity for real values
    st.finish(x)
    assert np.isclose(float(m.a.value), 2.0) and np.isclose(float(m.inner.c.value), 0.3)
    # gradient in unconstrained coordinates = constrained gradient * sigmoid(u)
    _, g = st.value_and_grad(_objective, m, _data(), x)
    assert np.isclose(g[0], 2 * (2.0 - 3.0) * (1 / (1 + np.exp(-x[0]))))


@pytest.mark.parametrize("runner", ["scipy", "lbfgs", "adam"])
def test_loops_converge(runner):
    m = _Toy()
    if runner == "scipy":
        m, hist = F.fit_scipy(model=m, objective=_objective, train_data=_data(), verbose=False)
        assert hist[-1] < 1e-10 and hist[0] > hist[-1]
    elif runner == "lbfgs":
        m, final = F.fit_lbfgs(model=m, objective=_objective, train_data=_data())
        assert final < 1e-10
    else:
        m, hist = F.fit(model=m, objective=_objective, train_data=_data(), num_iters=3000,
                        learning_rate=0.05)
        assert hist[-1] < 1e-6
    assert np.isclose(float(m.a.value), 3.0, atol=1e-3)
    assert np.allclose(m.inner.b.value.numpy(), [-1.0, 2.0], atol=1e-3)
    assert np.isclose(float(m.inner.c.value), 0.7, atol=1e-3)
    assert not m.a.value.requires_grad


def test_fit_rejects_bad_arguments():
    with pytest.raises(ValueError):
        F.fit_scipy(model=_Toy(), objective=_objective, train_data=_data(), max_iters=0)
    with pytest.raises(TypeError):
        F.fit_scipy(model=_Toy(), objective=None, train_data=_data())
