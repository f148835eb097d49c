"""GPU: gpk_conjugate_mll_batched — independent GPs of different sizes, input
dimensions and kernels in one call (float32 compute), each instance against the
float64 oracle (conjugate_mll, gpjax/objectives.py:36-107, and its torch float64
gradient).  Tolerances of the float32 form: 1e-4 relative on the MLL (measured
up to 2.2e-5 at n = 2048), 2e-3 on the gradient norm."""
import numpy as np
import pytest
import torch

from gpjax_gb300 import _lib
from gpjax_gb300.objectives import conjugate_mll_batched
from oracle import gp_oracle as O

pytestmark = pytest.mark.gpu

SPECS = [  # (kind, n, d, isotropic)
    (_lib.RBF, 64, 2, False), (_lib.MATERN32, 300, 5, False), (_lib.MATERN52, 777, 10, True),
    (_lib.RBF, 1500, 3, False), (_lib.MATERN32, 129, 8, True), (_lib.MATERN52, 2048, 4, False),
]


def _instance(spec, seed):
    kind, n, d, iso = spec
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1.0, 1.0, (n, d))
    ls = np.exp(rng.uniform(np.log(0.3), np.log(2.0), 1 if iso else d))
    var, sd, c = float(np.exp(rng.uniform(np.log(0.5), np.log(2.0)))), 0.1, 0.05
    y = np.sin(3 * x).sum(axis=1) + 0.1 * rng.standard_normal(n)
    theta = np.concatenate([ls, [var, sd, c]])
    return kind, x, y, ls, var, sd, c, theta


def _run(insts):
    dev = torch.device("cuda")
    xs = [torch.as_tensor(i[1], device=dev) for i in insts]
    ys = [torch.as_tensor(i[2], device=dev) for i in insts]
    ths = [torch.as_tensor(i[7], device=dev) for i in insts]
    mll, grads, info = conjugate_mll_batched([i[0] for i in insts], xs, ys, ths,
                                             [len(i[3]) for i in insts])
    torch.cuda.synchronize()
    return mll.cpu().numpy(), [g.cpu().numpy() for g in grads], info.cpu().numpy()


def test_batched_matches_oracle_per_instance(cuda_lib):
    insts = [_instance(s, 10 + k) for k, s in enumerate(SPECS)]
    mll, grads, info = _run(insts)
    assert np.all(info == 0)
    for k, (kind, x, y, ls, var, sd, c, _) in enumerate(insts):
        ref = O.conjugate_mll(kind, x, y[:, None], ls, var, sd, c)
        _, g = O.conjugate_mll_torch(kind, x, y[:, None], ls, var, sd, c, lu=False)
        gref = np.concatenate([np.atleast_1d(g["lengthscale"]),
                               [g["variance"], g["obs_stddev"], g["constant"]]])
        assert abs(mll[k] - ref) <= 1e-4 * abs(ref), (k, mll[k], ref)
        assert np.linalg.norm(grads[k] - gref) <= 2e-3 * np.linalg.norm(gref), (k, grads[k], gref)


def test_batched_repeatable(cuda_lib):
    insts = [_instance(s, 40 + k) for k, s in enumerate(SPECS[:4])]
    a = _run(insts)
    b = _run(insts)
    assert np.array_equal(a[0], b[0])
    assert all(np.array_equal(p, q) for p, q in zip(a[1], b[1]))
