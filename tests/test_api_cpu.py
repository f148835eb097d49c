"""Host-side pieces of the Python layer, on CPU: the Dataset container and the
parameter types behave as the reference's (gpjax/dataset.py:26-126,
gpjax/parameters.py:69-146; behaviours restated from tests/test_dataset.py and
tests/test_parameters.py of the reference), and the precision setting."""
import numpy as np
import pytest
import torch

import gpjax_gb300 as gpx
from gpjax_gb300 import config, parameters


@pytest.mark.parametrize("n", [1, 2, 10])
@pytest.mark.parametrize("in_dim", [1, 2, 10])
def test_dataset_shapes_and_kinds(n, in_dim):
    x, y = np.ones((n, in_dim)), np.ones((n, 1))
    D = gpx.Dataset(X=x, y=y, device="cpu")
    assert D.n == n and D.in_dim == in_dim
    assert repr(D) == f"Dataset(Number of observations: {n} - Input dimension: {in_dim})"
    assert D.is_supervised() and not D.is_unsupervised()
    U = gpx.Dataset(y=y, device="cpu")
    assert U.is_unsupervised() and not U.is_supervised() and U.X is None
    assert gpx.Dataset(X=x, device="cpu").y is None


@pytest.mark.parametrize("n1,n2", [(1, 2), (10, 1)])
def test_dataset_add_stacks_rows(n1, n2):
    a = gpx.Dataset(X=np.ones((n1, 3)), y=np.ones((n1, 1)), device="cpu")
    b = gpx.Dataset(X=2 * np.ones((n2, 3)), y=2 * np.ones((n2, 1)), device="cpu")
    c = a + b
    assert c.n == n1 + n2 and c.in_dim == 3
    assert torch.equal(c.X[n1:], b.X) and torch.equal(c.y[:n1], a.y)
    u = gpx.Dataset(y=np.ones((n1, 1)), device="cpu") + gpx.Dataset(y=np.ones((n2, 1)), device="cpu")
    assert u.is_unsupervised() and u.n == n1 + n2


def test_dataset_rejects_mismatched_rows():
    with pytest.raises(ValueError, match="same number of rows"):
        gpx.Dataset(X=np.ones((3, 2)), y=np.ones((4, 1)), device="cpu")


@pytest.mark.parametrize("dx,dy,warns", [(np.float32, np.float64, 1), (np.float64, np.float32, 1),
                                         (np.float32, np.float32, 2)])
def test_dataset_warns_on_low_precision(dx, dy, warns):
    with pytest.warns(UserWarning, match="not of type float64") as rec:
        D = gpx.Dataset(X=np.ones((4, 2), dtype=dx), y=np.ones((4, 1), dtype=dy), device="cpu")
    assert len(rec) == warns
    assert D.X.dtype == torch.float64 and D.y.dtype == torch.float64


def test_parameter_constraints():
    assert parameters.PositiveReal(0.5).value.item() == 0.5
    with pytest.raises(ValueError):
        parameters.PositiveReal(0.0)
    with pytest.raises(ValueError):
        parameters.PositiveReal(np.array([1.0, -2.0]))
    assert parameters.NonNegativeReal(0.0).value.item() == 0.0
    with pytest.raises(ValueError):
        parameters.NonNegativeReal(-1e-9)
    assert parameters.Real(-3.0).value.item() == -3.0
    p = parameters.PositiveReal(np.array([0.3, 2.0])).requires_grad_(True)
    assert p.value.requires_grad and p.value.dtype == torch.float64 and p.tag == "positive"


def test_softplus_inverse_round_trip():
    x = torch.tensor([1e-3, 0.5, 3.0, 20.0], dtype=torch.float64)
    y = parameters.softplus_inverse(x)
    assert torch.allclose(torch.nn.functional.softplus(y), x, rtol=1e-12, atol=0)


def test_precision_codes():
    from gpjax_gb300 import _lib
    assert config.precision_code("fp64") == _lib.PREC_FP64
    assert config.precision_code("mixed") == _lib.PREC_MIXED
    with pytest.raises(ValueError):
        config.precision_code("bf16")


# structured operators: the reference's dispatch (linalg/operations.py:22-222)
# answers these without a factorisation; restated from its tests/test_linalg.py
from gpjax_gb300 import linalg as la  # noqa: E402


def _t(v):
    return torch.tensor(v, dtype=torch.float64)


def test_structured_cholesky():
    L = la.lower_cholesky(la.Diagonal(_t([1.0, 4.0, 9.0])))
    assert isinstance(L, la.Diagonal) and torch.allclose(L.diagonal, _t([1.0, 2.0, 3.0]))
    eye = la.Identity(4, device="cpu")
    assert la.lower_cholesky(eye) is eye and eye.shape == (4, 4)


def test_structured_solve():
    b = _t([1.0, 2.0, 3.0])
    assert torch.allclose(la.solve(la.Identity(3, device="cpu"), b), b)
    x = la.solve(la.Diagonal(_t([2.0, 4.0, 5.0])), _t([2.0, 8.0, 10.0]))
    assert torch.allclose(x, _t([1.0, 2.0, 2.0]))
    X = la.solve(la.Diagonal(_t([2.0, 4.0])), _t([[2.0, 4.0], [8.0, 12.0]]))
    assert X.shape == (2, 2) and torch.allclose(X, _t([[1.0, 2.0], [2.0, 3.0]]))


def test_structured_logdet_and_diag():
    assert float(la.logdet(la.Identity(3, device="cpu"))) == 0.0
    d = _t([2.0, 3.0, 4.0])
    assert torch.isclose(la.logdet(la.Diagonal(d)), torch.log(d).sum())
    assert torch.allclose(la.diag(la.Identity(4, device="cpu")), torch.ones(4, dtype=torch.float64))
    assert torch.equal(la.diag(la.Diagonal(d)), d)


def test_add_jitter():
    K = _t([[1.0, 0.5], [0.5, 2.0]])
    J = la.add_jitter(K, 1e-3)
    assert torch.allclose(J, K + 1e-3 * torch.eye(2, dtype=torch.float64))
    assert torch.equal(K, _t([[1.0, 0.5], [0.5, 2.0]]))  # the input is not modified
    with pytest.raises(ValueError):
        la.add_jitter(_t([[1.0, 2.0, 3.0]]))


def test_theta_layout_and_model_parameters():
    """The theta vector that crosses the C ABI is [lengthscale..., variance,
    obs_stddev, mean constant] (include/gpk.h), and the posterior exposes its
    trainable parameters by name as the reference's model state does."""
    from gpjax_gb300.objectives import named_parameters
    ls = np.array([0.5, 1.5, 2.5])
    kern = gpx.kernels.Matern52(lengthscale=ls, variance=1.3)
    assert kern.n_ls == 3 and kern.kind == 2
    th = kern.theta_vector("cpu", torch.tensor(0.2, dtype=torch.float64),
                           torch.tensor(0.7, dtype=torch.float64))
    assert torch.allclose(th, _t([0.5, 1.5, 2.5, 1.3, 0.2, 0.7]))
    iso = gpx.kernels.RBF(lengthscale=0.9, variance=1.0)
    assert iso.n_ls == 1
    assert torch.allclose(iso.theta_vector("cpu"), _t([0.9, 1.0, 0.0, 0.0]))
    prior = gpx.gps.Prior(kernel=kern, mean_function=gpx.mean_functions.Constant(
        gpx.parameters.Real(0.7)))
    post = prior * gpx.likelihoods.Gaussian(num_datapoints=10, obs_stddev=0.2)
    names = named_parameters(post)
    assert any(k.endswith("lengthscale") for k in names)
    assert any(k.endswith("variance") for k in names)
    assert any(k.endswith("obs_stddev") for k in names)
    assert any(k.endswith("constant") for k in names)
