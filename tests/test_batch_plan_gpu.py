"""GPU: the persistent batched plan (gpk_batch_plan_*) -- independent GPs of
different sizes, input dimensions and kernels evaluated by one persistent
launch, each instance against the float64 oracle (conjugate_mll,
gpjax/objectives.py:36-107, and its torch float64 gradient).

Tolerances of the float32 form (float64 pivots, float-float refinement of
alpha): 1e-4 relative on the MLL, 2e-3 relative on the gradient norm.  The
float32 rounding of Sigma's entries alone moves the log-determinant of the
Matern-5/2 n = 2048, d = 4 case (condition number 1.6e5) by 4.8e-5 of the MLL
(LAPACK's float32 Cholesky of the same matrix).  The same bounds hold for every
tile configuration (CUDA-core and tcgen05 split-TF32) forced in turn."""
import numpy as np
import pytest
import torch

from gpjax_gb300 import _lib
from gpjax_gb300.objectives import BatchPlan
from oracle import gp_oracle as O

pytestmark = pytest.mark.gpu

MLL_RTOL, GRAD_RTOL = 1e-4, 2e-3

SPECS = [  # (kind, n, d, isotropic)
    (_lib.RBF, 64, 2, False), (_lib.MATERN32, 300, 5, False), (_lib.MATERN52, 777, 10, True),
    (_lib.RBF, 1500, 3, False), (_lib.MATERN32, 129, 8, True), (_lib.MATERN52, 2048, 4, False),
    (_lib.MATERN12, 640, 6, False), (_lib.RBF, 128, 16, False), (_lib.MATERN52, 1, 3, False),
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


def _oracle(inst):
    kind, x, y, ls, var, sd, c, _ = inst
    ref = O.conjugate_mll(kind, x, y[:, None], ls, var, sd, c)
    _, g = O.conjugate_mll_torch(kind, x, y[:, None], ls, var, sd, c, lu=False)
    gref = np.concatenate([np.atleast_1d(g["lengthscale"]), [g["variance"], g["obs_stddev"],
                                                              g["constant"]]])
    return ref, gref


def _plan(insts, **kw):
    dev = torch.device("cuda")
    xs = [torch.as_tensor(i[1], device=dev) for i in insts]
    ys = [torch.as_tensor(i[2], device=dev) for i in insts]
    ths = [torch.as_tensor(i[7], device=dev) for i in insts]
    return BatchPlan([i[0] for i in insts], xs, ys, ths, [len(i[3]) for i in insts], **kw)


def test_plan_matches_oracle_per_instance(cuda_lib):
    insts = [_instance(s, 10 + k) for k, s in enumerate(SPECS)]
    plan = _plan(insts)
    mll, grads, info = plan.execute()
    torch.cuda.synchronize()
    mll, info = mll.cpu().numpy(), info.cpu().numpy()
    assert np.all(info == 0), info
    worst = 0.0
    for k, inst in enumerate(insts):
        ref, gref = _oracle(inst)
        g = grads[k].cpu().numpy()
        rel = abs(mll[k] - ref) / abs(ref)
        grel = np.linalg.norm(g - gref) / np.linalg.norm(gref)
        worst = max(worst, rel)
        assert rel <= MLL_RTOL, (k, SPECS[k], mll[k], ref, rel)
        assert grel <= GRAD_RTOL, (k, SPECS[k], g, gref, grel)
        print("instance", k, SPECS[k], "mll rel", rel, "grad rel", grel)
    print("worst MLL relative error", worst)
    plan.close()


def test_plan_is_repeatable_and_graph_capturable(cuda_lib):
    insts = [_instance(s, 40 + k) for k, s in enumerate(SPECS[:6])]
    plan = _plan(insts, autotune=False)
    a = [t.clone() for t in (plan.execute()[0],)] + [g.clone() for g in plan.grads]
    plan.execute()
    torch.cuda.synchronize()
    assert torch.equal(a[0], plan.mll)
    assert all(torch.equal(p, q) for p, q in zip(a[1:], plan.grads))
    plan.mll.fill_(0.0)
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            plan.execute()
    torch.cuda.current_stream().wait_stream(s)
    plan.mll.fill_(0.0)
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(a[0], plan.mll)
    plan.close()


def test_plan_reads_parameters_at_every_execution(cuda_lib):
    """Multi-start fits update theta in place between executions."""
    insts = [_instance(s, 70 + k) for k, s in enumerate(SPECS[:3])]
    plan = _plan(insts, autotune=False)
    plan.execute()
    for k, inst in enumerate(insts):
        plan.thetas[k][-2] = 0.3  # obs_stddev
    mll, grads, info = plan.execute()
    torch.cuda.synchronize()
    for k, inst in enumerate(insts):
        kind, x, y, ls, var, sd, c, th = inst
        ref = O.conjugate_mll(kind, x, y[:, None], ls, var, 0.3, c)
        assert abs(float(mll[k]) - ref) <= MLL_RTOL * abs(ref)
    plan.close()


def test_plan_reports_a_failed_instance_and_keeps_the_others(cuda_lib):
    insts = [_instance(s, 90 + k) for k, s in enumerate(SPECS[:4])]
    bad = list(insts[1])
    bad[7] = bad[7].copy()
    bad[7][-3] = -1.0  # negative variance: Sigma is not positive definite
    insts[1] = tuple(bad)
    plan = _plan(insts, autotune=False)
    mll, grads, info = plan.execute()
    torch.cuda.synchronize()
    info = info.cpu().numpy()
    assert info[1] > 0 and np.isnan(float(mll[1]))
    assert np.all(torch.isnan(plan.grads[1]).cpu().numpy())
    for k in (0, 2, 3):
        assert info[k] == 0
        ref, _ = _oracle(insts[k])
        assert abs(float(mll[k]) - ref) <= MLL_RTOL * abs(ref)
    plan.close()


def test_autotuner_picks_a_configuration_per_size(cuda_lib):
    insts = [_instance((_lib.RBF, n, 3, False), 120 + k) for k, n in enumerate([256, 256, 1024])]
    plan = _plan(insts, autotune=True)
    ncfg = BatchPlan.config_count()
    assert plan.config(256) in range(ncfg) and plan.config(1024) in range(ncfg)
    assert plan.config(5000) == -1
    plan.close()


@pytest.mark.parametrize("cfg", [0, 1, 2])
def test_every_configuration_matches_oracle(cuda_lib, cfg):
    """Each tile configuration forced on every instance (2: the products on the
    tcgen05 tensor cores in split TF32) meets the same tolerances, and going
    back to the tuned configurations changes no result beyond them."""
    insts = [_instance(s, 200 + k) for k, s in enumerate(SPECS)]
    plan = _plan(insts, autotune=False)
    plan.force_config(cfg)
    mll, grads, info = plan.execute()
    torch.cuda.synchronize()
    mll, info = mll.cpu().numpy().copy(), info.cpu().numpy()
    assert np.all(info == 0), info
    for k, inst in enumerate(insts):
        ref, gref = _oracle(inst)
        g = grads[k].cpu().numpy()
        rel = abs(mll[k] - ref) / abs(ref)
        grel = np.linalg.norm(g - gref) / np.linalg.norm(gref)
        assert rel <= MLL_RTOL, (cfg, k, SPECS[k], mll[k], ref, rel)
        assert grel <= GRAD_RTOL, (cfg, k, SPECS[k], g, gref, grel)
        print("cfg", cfg, "instance", k, SPECS[k], "mll rel", rel, "grad rel", grel)
    plan.force_config(-1)
    mll2, _, info2 = plan.execute()
    torch.cuda.synchronize()
    assert np.all(info2.cpu().numpy() == 0)
    np.testing.assert_allclose(mll2.cpu().numpy(), mll, rtol=2 * MLL_RTOL)
    with pytest.raises(_lib.GPKError):
        plan.force_config(BatchPlan.config_count())
    plan.close()


def test_plan_rational_quadratic_and_value_only(cuda_lib):
    """The rational quadratic (alpha in theta[n_ls + 3]) and a plan without
    gradients (no adjoint tiles: every instance finishes on its owner)."""
    dev = torch.device("cuda")
    rng = np.random.default_rng(7)
    insts, kinds = [], []
    for k, (n, d) in enumerate([(300, 3), (900, 5), (129, 2)]):
        x = rng.uniform(-1.0, 1.0, (n, d))
        ls = np.exp(rng.uniform(np.log(0.3), np.log(2.0), d))
        alpha = float(np.exp(rng.uniform(np.log(0.5), np.log(3.0))))
        y = np.sin(3 * x).sum(axis=1) + 0.1 * rng.standard_normal(n)
        insts.append((x, y, ls, 1.2, 0.1, 0.05, alpha))
        kinds.append(_lib.RATIONAL_QUADRATIC)
    xs = [torch.as_tensor(i[0], device=dev) for i in insts]
    ys = [torch.as_tensor(i[1], device=dev) for i in insts]
    ths = [torch.as_tensor(np.concatenate([i[2], [i[3], i[4], i[5], i[6]]]), device=dev)
           for i in insts]
    for want in (True, False):
        plan = BatchPlan(kinds, xs, ys, ths, [len(i[2]) for i in insts], want_grad=want,
                         autotune=False)
        mll, grads, info = plan.execute()
        torch.cuda.synchronize()
        assert np.all(info.cpu().numpy() == 0)
        for k, (x, y, ls, var, sd, c, alpha) in enumerate(insts):
            kern = O.rational_quadratic(alpha)
            ref = O.conjugate_mll(kern, x, y[:, None], ls, var, sd, c)
            assert abs(float(mll[k]) - ref) <= MLL_RTOL * abs(ref), (k, float(mll[k]), ref)
            if want:
                _, g = O.conjugate_mll_torch(kern, x, y[:, None], ls, var, sd, c, lu=False)
                gref = np.concatenate([np.atleast_1d(g["lengthscale"]),
                                       [g["variance"], g["obs_stddev"], g["constant"]]])
                gk = grads[k].cpu().numpy()[:len(gref)]
                assert np.linalg.norm(gk - gref) <= GRAD_RTOL * np.linalg.norm(gref)
        plan.close()


def test_tensor_core_wait_timeout_is_reported(cuda_lib):
    """A bounded wait that runs out (the self-test makes each CTA's first MMA
    wait also wait ~10 ms on a barrier nothing arrives on) is reported as
    info = -1 with NaN outputs; the context stays usable and the next
    execution without it is correct."""
    insts = [_instance(s, 300 + k) for k, s in enumerate(SPECS[:4])]
    plan = _plan(insts, autotune=False)
    plan.force_config(2)
    plan.selftest_stall(20_000_000)
    mll, grads, info = plan.execute()
    torch.cuda.synchronize()
    assert np.all(info.cpu().numpy() == -1), info
    assert np.all(np.isnan(mll.cpu().numpy()))
    plan.selftest_stall(0)
    mll, grads, info = plan.execute()
    torch.cuda.synchronize()
    assert np.all(info.cpu().numpy() == 0)
    for k, inst in enumerate(insts):
        ref, _ = _oracle(inst)
        assert abs(float(mll[k]) - ref) <= MLL_RTOL * abs(ref), (k, float(mll[k]), ref)
    with pytest.raises(_lib.GPKError):
        plan.selftest_stall(-1)
    plan.close()
