"""Objectives on the GPU: conjugate_mll and collapsed_elbo
(mirrors gpjax/objectives.py:33-416).

Each objective is a ``torch.autograd.Function``: one call of the C ABI returns
the value together with its gradient in the reference's constrained
coordinates (lengthscale, variance, obs_stddev, constant mean and, for the
collapsed ELBO, the inducing inputs); ``backward`` only scales the stored
gradient by the incoming cotangent.  This is the counterpart of the
reference's ``jax.value_and_grad`` over the objective (fit.py:160,233).
"""
from __future__ import annotations

import torch

from . import _lib
from .config import precision_code
from .gps import _mean_constant


class _ConjugateMLL(torch.autograd.Function):
    @staticmethod
    def forward(ctx, theta, x, y, kind, n_ls, jitter, prec):
        dev = _lib.require_cuda(x, y, theta)
        n, d = x.shape
        want_grad = bool(ctx.needs_input_grad[0])
        th = theta.detach().contiguous()
        xc, yc = x.detach().contiguous(), y.detach().reshape(-1).contiguous()
        out = torch.empty(1, dtype=torch.float64, device=dev)
        grad = torch.zeros(th.numel(), dtype=torch.float64, device=dev)  # n_ls + 3 (+ RQ alpha)
        info = torch.zeros(1, dtype=torch.int32, device=dev)
        nbytes = _lib.lib().gpk_conjugate_mll_workspace_bytes(n, d, prec)
        ws = _lib.workspace(nbytes, dev)
        _lib.call("gpk_conjugate_mll", kind, n, d, xc.data_ptr(), d, yc.data_ptr(), th.data_ptr(),
                  n_ls, float(jitter), prec, int(want_grad), out.data_ptr(), grad.data_ptr(),
                  info.data_ptr(), ws.data_ptr(), ws.numel(), _lib.stream_ptr(dev))
        ctx.save_for_backward(grad)
        ctx.info = info
        return out[0]

    @staticmethod
    def backward(ctx, g):
        (grad,) = ctx.saved_tensors
        return g * grad, None, None, None, None, None, None


def conjugate_mll(posterior, data, precision: str | None = None) -> torch.Tensor:
    """Marginal log-likelihood of a conjugate GP (objectives.py:36-107).

    Sigma = (K(x, x) + I*prior.jitter) + I*obs_stddev^2;
    returns log N(y; m(x), Sigma) as a 0-d float64 tensor that is
    differentiable w.r.t. the kernel, likelihood and mean parameters.
    """
    kernel = posterior.prior.kernel
    x = kernel.slice_input(data.X)
    dev = _lib.require_cuda(x)
    const = _mean_constant(posterior.prior.mean_function, dev)
    theta = kernel.theta_vector(dev, posterior.likelihood.obs_stddev.value, const)
    return _ConjugateMLL.apply(theta, x, data.y, kernel.kind, kernel.n_ls,
                               float(posterior.prior.jitter), precision_code(precision))


class _ConjugateLOOCV(torch.autograd.Function):
    @staticmethod
    def forward(ctx, theta, x, y, kind, n_ls, jitter):
        dev = _lib.require_cuda(x, y, theta)
        n, d = x.shape
        want_grad = bool(ctx.needs_input_grad[0])
        th = theta.detach().contiguous()
        xc, yc = x.detach().contiguous(), y.detach().reshape(-1).contiguous()
        out = torch.empty(1, dtype=torch.float64, device=dev)
        grad = torch.zeros(th.numel(), dtype=torch.float64, device=dev)  # n_ls + 3 (+ RQ alpha)
        info = torch.zeros(1, dtype=torch.int32, device=dev)
        ws = _lib.workspace(_lib.lib().gpk_conjugate_loocv_workspace_bytes(n, d), dev)
        _lib.call("gpk_conjugate_loocv", kind, n, d, xc.data_ptr(), d, yc.data_ptr(),
                  th.data_ptr(), n_ls, float(jitter), int(want_grad), out.data_ptr(),
                  grad.data_ptr(), info.data_ptr(), ws.data_ptr(), ws.numel(),
                  _lib.stream_ptr(dev))
        ctx.save_for_backward(grad)
        ctx.info = info
        return out[0]

    @staticmethod
    def backward(ctx, g):
        (grad,) = ctx.saved_tensors
        return g * grad, None, None, None, None, None


def conjugate_loocv(posterior, data) -> torch.Tensor:
    """Leave-one-out predictive log-probability of a conjugate GP
    (objectives.py:110-178), float64, differentiable w.r.t. the kernel,
    likelihood and mean parameters; maximise it (minimise its negative) like the
    marginal log-likelihood."""
    kernel = posterior.prior.kernel
    x = kernel.slice_input(data.X)
    dev = _lib.require_cuda(x)
    const = _mean_constant(posterior.prior.mean_function, dev)
    theta = kernel.theta_vector(dev, posterior.likelihood.obs_stddev.value, const)
    return _ConjugateLOOCV.apply(theta, x, data.y, kernel.kind, kernel.n_ls,
                                 float(posterior.prior.jitter))


def value_and_grad(objective, model, data, **kw):
    """(value, {name: grad}) of an objective, like jax.value_and_grad over the
    model's parameters (fit.py:160)."""
    params = named_parameters(model)
    for p in params.values():
        p.requires_grad_(True)
    val = objective(model, data, **kw)
    grads = torch.autograd.grad(val, [p.value for p in params.values()], allow_unused=True)
    out = {k: (g if g is not None else torch.zeros_like(p.value))
           for (k, p), g in zip(params.items(), grads)}
    return val.detach(), out


def named_parameters(model) -> dict:
    """The trainable Parameters of a posterior / variational family by dotted name."""
    from .parameters import Parameter
    found = {}

    def walk(obj, prefix, seen):
        if id(obj) in seen:
            return
        seen.add(id(obj))
        for k, v in vars(obj).items():
            name = f"{prefix}{k}"
            if isinstance(v, Parameter):
                found[name] = v
            elif hasattr(v, "__dict__") and not isinstance(v, (torch.Tensor, type)):
                walk(v, name + ".", seen)
    walk(model, "", set())
    return found


def shard_rows(n: int, world: int, rank: int) -> slice:
    """Rows of an n-row dataset that rank `rank` of `world` holds in a
    data-parallel collapsed ELBO: contiguous, sizes differing by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("need 0 <= rank < world")
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    return slice(start, start + base + (1 if rank < extra else 0))


def partition_instances(ns, world: int) -> list:
    """Independent GPs split over `world` ranks for a data-parallel batched
    evaluation (each rank builds a BatchPlan over its share; no collective but
    the gather of the results).  Cost of an instance ~ n^3: largest first, each
    to the rank with the least cost so far (ties to the lower rank).  Returns
    one sorted index list per rank; deterministic, so every rank computes the
    same split."""
    if world < 1:
        raise ValueError("need world >= 1")
    load = [0.0] * world
    parts = [[] for _ in range(world)]
    for i in sorted(range(len(ns)), key=lambda i: (-int(ns[i]), i)):
        r = min(range(world), key=lambda q: (load[q], q))
        parts[r].append(i)
        load[r] += float(ns[i]) ** 3
    return [sorted(p) for p in parts]


def gather_instance_results(mll: torch.Tensor, indices, count: int, group=None) -> torch.Tensor:
    """All ranks' per-instance MLL values into one [count] float64 tensor in
    the original order (torch.distributed.all_gather of each rank's share,
    padded to the longest share)."""
    import torch.distributed as dist

    world = dist.get_world_size(group)
    sizes = [None] * world
    dist.all_gather_object(sizes, (len(indices), list(indices)), group=group)
    width = max(s[0] for s in sizes) if sizes else 0
    buf = torch.full((width,), float("nan"), dtype=torch.float64, device=mll.device)
    buf[:len(indices)] = mll[:len(indices)]
    bufs = [torch.empty_like(buf) for _ in range(world)]
    dist.all_gather(bufs, buf, group=group)
    out = torch.full((count,), float("nan"), dtype=torch.float64, device=mll.device)
    for (k, idx), b in zip(sizes, bufs):
        if k:
            out[torch.as_tensor(idx, device=mll.device)] = b[:k]
    return out


def allreduce_callback(workspace: torch.Tensor, group=None):
    """The library's exchange hook for gpk_collapsed_elbo_sharded: sums the
    float64 region at a byte offset of `workspace` over the process group, in
    place (torch.distributed.all_reduce, ordered on the current stream).
    Returns the ctypes callback (keep a reference while the call runs)."""
    import torch.distributed as dist

    def fn(user, offset, count, stream):
        try:
            view = workspace.narrow(0, int(offset), int(count) * 8).view(torch.float64)
            dist.all_reduce(view, group=group)
            return 0
        except Exception:  # reported to the library as a failed exchange
            return 1
    return _lib.ALLREDUCE_FN(fn)


class _CollapsedELBO(torch.autograd.Function):
    @staticmethod
    def forward(ctx, theta, z, x, y, kind, n_ls, jitter, prec, group=None):
        dev = _lib.require_cuda(x, y, theta, z)
        n, d = x.shape
        m = z.shape[0]
        want = bool(ctx.needs_input_grad[0] or ctx.needs_input_grad[1])
        th = theta.detach().contiguous()
        xc, yc = x.detach().contiguous(), y.detach().reshape(-1).contiguous()
        zc = z.detach().to(torch.float64).contiguous()
        out = torch.empty(1, dtype=torch.float64, device=dev)
        grad = torch.zeros(th.numel(), dtype=torch.float64, device=dev)  # n_ls + 3 (+ RQ alpha)
        gz = torch.zeros((m, d), dtype=torch.float64, device=dev)
        info = torch.zeros(1, dtype=torch.int32, device=dev)
        nbytes = _lib.lib().gpk_collapsed_elbo_workspace_bytes(n, m, d, prec)
        ws = _lib.workspace(nbytes, dev)
        if group is None:
            _lib.call("gpk_collapsed_elbo", kind, n, m, d, xc.data_ptr(), d, yc.data_ptr(),
                      zc.data_ptr(), d, th.data_ptr(), n_ls, float(jitter), prec, int(want),
                      out.data_ptr(), grad.data_ptr(), gz.data_ptr(), info.data_ptr(),
                      ws.data_ptr(), ws.numel(), _lib.stream_ptr(dev))
        else:
            import torch.distributed as dist
            n_total = torch.tensor([n], dtype=torch.int64, device=dev)
            dist.all_reduce(n_total, group=group)
            cb = allreduce_callback(ws, group)
            _lib.call("gpk_collapsed_elbo_sharded", kind, n, int(n_total.item()), m, d,
                      xc.data_ptr(), d, yc.data_ptr(), zc.data_ptr(), d, th.data_ptr(), n_ls,
                      float(jitter), prec, int(want), out.data_ptr(), grad.data_ptr(),
                      gz.data_ptr(), info.data_ptr(), ws.data_ptr(), ws.numel(),
                      _lib.stream_ptr(dev), cb, None)
        ctx.save_for_backward(grad, gz)
        ctx.info = info
        return out[0]

    @staticmethod
    def backward(ctx, g):
        grad, gz = ctx.saved_tensors
        return g * grad, g * gz, None, None, None, None, None, None, None


def collapsed_elbo(variational_family, data, precision: str | None = None,
                   process_group=None) -> torch.Tensor:
    """SGPR collapsed evidence lower bound (objectives.py:321-416), differentiable
    w.r.t. the kernel, likelihood and mean parameters and the inducing inputs.

    With ``process_group`` (a torch.distributed group, one GPU per rank),
    ``data`` holds this rank's rows only (``shard_rows``): each rank forms its
    statistics, one all-reduce sums them, and every rank returns the ELBO and
    gradients of the whole dataset."""
    q = variational_family
    post = q.posterior
    kernel = post.prior.kernel
    x = kernel.slice_input(data.X)
    dev = _lib.require_cuda(x)
    z = kernel.slice_input(q.inducing_inputs.value.to(dev))
    const = _mean_constant(post.prior.mean_function, dev)
    theta = kernel.theta_vector(dev, post.likelihood.obs_stddev.value, const)
    return _CollapsedELBO.apply(theta, z, x, data.y, kernel.kind, kernel.n_ls, float(q.jitter),
                                precision_code(precision), process_group)


def cross_covariance_vjp(kind, n_ls, theta, x, y, G, need_x=False, need_y=False):
    """Cotangent of K(x, y) -> (d theta [n_ls + 3], d x, d y) through gpk_cross_covariance_vjp."""
    dev = _lib.require_cuda(x, y, G)
    n, m, d = x.shape[0], y.shape[0], x.shape[1]
    gth = torch.zeros(theta.numel(), dtype=torch.float64, device=dev)  # n_ls + 3 (+ RQ alpha)
    gx = torch.zeros((n, d), dtype=torch.float64, device=dev) if need_x else None
    gy = torch.zeros((m, d), dtype=torch.float64, device=dev) if need_y else None
    Gc = G.detach().to(torch.float64).contiguous()
    nbytes = _lib.lib().gpk_cross_covariance_vjp_workspace_bytes(n, m, d)
    ws = _lib.workspace(nbytes, dev)
    _lib.call("gpk_cross_covariance_vjp", kind, n, m, d, x.data_ptr(), d, y.data_ptr(), d,
              theta.data_ptr(), n_ls, Gc.data_ptr(), m, gth.data_ptr(), _lib.ptr(gx),
              _lib.ptr(gy), ws.data_ptr(), ws.numel(), _lib.stream_ptr(dev))
    return gth, gx, gy


class BatchPlan:
    """Many independent GPs of uneven n (conjugate_mll, gpjax/objectives.py:36-107,
    and its gradient per instance) evaluated by ONE persistent kernel launch per
    :meth:`execute`: the plan sorts the instances by n into a device queue, and
    one CTA per SM pulls instances from it and runs each to completion
    (``gpk_batch_plan_*`` in include/gpk.h).  With ``autotune`` the plan times
    the library's tile configurations on its own instances for every padded n
    not tuned before in this process.

    kinds: kernel codes; xs: [n_i, d_i] float64 CUDA tensors (n_i <= 4096,
    d_i <= 16); ys: [n_i]; thetas: the theta layout ``[lengthscale (n_ls[i]),
    variance, obs_stddev, constant]`` (``alpha`` last for RationalQuadratic).
    The tensors are read at every execution (update them in place between
    executions, e.g. for multi-start fits); results land in ``self.mll``,
    ``self.grads`` and ``self.info``.  ``execute`` is stream-ordered and can be
    captured in a CUDA graph.
    """

    def __init__(self, kinds, xs, ys, thetas, n_ls, jitter: float = 1e-6,
                 want_grad: bool = True, autotune: bool = True):
        import ctypes

        B = len(xs)
        dev = _lib.require_cuda(*xs)
        self.device = dev
        self.xs = [x.detach().contiguous() for x in xs]
        self.ys = [y.detach().reshape(-1).contiguous() for y in ys]
        self.thetas = [t.detach().contiguous() for t in thetas]
        self.mll = torch.full((B,), float("nan"), dtype=torch.float64, device=dev)
        self.grads = [torch.zeros(int(nl) + 3 + (1 if int(k) == _lib.RATIONAL_QUADRATIC else 0),
                                  dtype=torch.float64, device=dev)
                      for nl, k in zip(n_ls, kinds)]
        self.info = torch.zeros(B, dtype=torch.int32, device=dev)
        i32, i64, ptr = ctypes.c_int * B, ctypes.c_int64 * B, ctypes.c_void_p * B
        handle = ctypes.c_void_p()
        _lib.call("gpk_batch_plan_create", B, i32(*[int(k) for k in kinds]),
                  i64(*[x.shape[0] for x in self.xs]), i32(*[x.shape[1] for x in self.xs]),
                  ptr(*[x.data_ptr() for x in self.xs]), i64(*[x.shape[1] for x in self.xs]),
                  ptr(*[y.data_ptr() for y in self.ys]), ptr(*[t.data_ptr() for t in self.thetas]),
                  i32(*[int(v) for v in n_ls]), float(jitter), int(want_grad),
                  ptr(*[self.mll.data_ptr() + 8 * i for i in range(B)]),
                  ptr(*[g.data_ptr() for g in self.grads]), self.info.data_ptr(), int(autotune),
                  ctypes.byref(handle))
        self._handle = handle
        lib = _lib.lib()
        self.workspace = torch.empty(max(int(lib.gpk_batch_plan_workspace_bytes(handle)), 256),
                                     dtype=torch.uint8, device=dev)

    def config(self, n: int) -> int:
        """Tile configuration the autotuner chose for instances of size n."""
        return int(_lib.lib().gpk_batch_plan_config(self._handle, int(n)))

    @staticmethod
    def config_count() -> int:
        """Number of tile configurations (the last one runs on the tensor cores)."""
        return int(_lib.lib().gpk_batch_plan_config_count())

    def force_config(self, cfg: int):
        """Run every instance of later executions with configuration ``cfg``
        (``-1``: the tuned configurations again)."""
        _lib.call("gpk_batch_plan_force_config", self._handle, int(cfg))

    def selftest_stall(self, cycles: int):
        """Self-test of the tensor-core configuration's bounded waits: with
        ``cycles > 0`` the first MMA wait of every CTA also waits that many SM
        clocks on a barrier nothing arrives on, and its instances report
        ``info = -1`` (``0`` turns it off)."""
        _lib.call("gpk_batch_plan_selftest_stall", self._handle, int(cycles))

    def execute(self):
        """One launch over all instances; returns (mll, grads, info)."""
        _lib.call("gpk_batch_plan_execute", self._handle, self.workspace.data_ptr(),
                  self.workspace.numel(), _lib.stream_ptr(self.device))
        return self.mll, self.grads, self.info

    def close(self):
        if getattr(self, "_handle", None) is not None and self._handle.value:
            torch.cuda.synchronize(self.device)
            _lib.lib().gpk_batch_plan_destroy(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # interpreter shutdown
            pass


def conjugate_mll_batched(kinds, xs, ys, thetas, n_ls, jitter: float = 1e-6,
                          want_grad: bool = True):
    """conjugate_mll (gpjax/objectives.py:36-107) and its gradient for a batch of
    independent GPs of different sizes in one library call (float32 compute,
    instances spread over internal streams).

    kinds: kernel codes (``_lib.RBF`` / ``MATERN32`` / ``MATERN52``); xs: [n_i, d_i]
    float64 CUDA tensors; ys: [n_i]; thetas: the gpk theta layout
    ``[lengthscale (n_ls[i]), variance, obs_stddev, constant]``.  Returns
    (mll [B] float64, list of gradients in the theta layout, info [B] int32).
    The call is stream-ordered and capturable into a CUDA graph when the
    workspace is reused (pass the tensors of a previous call's inputs).
    """
    import ctypes

    B = len(xs)
    dev = _lib.require_cuda(*xs)
    xs = [x.detach().contiguous() for x in xs]
    ys = [y.detach().reshape(-1).contiguous() for y in ys]
    thetas = [t.detach().contiguous() for t in thetas]
    mll = torch.empty(B, dtype=torch.float64, device=dev)
    grads = [torch.zeros(int(nl) + 3, dtype=torch.float64, device=dev) for nl in n_ls]
    info = torch.zeros(B, dtype=torch.int32, device=dev)
    i32, i64, ptr = ctypes.c_int * B, ctypes.c_int64 * B, ctypes.c_void_p * B
    n = i64(*[x.shape[0] for x in xs])
    d = i32(*[x.shape[1] for x in xs])
    lib = _lib.lib()
    ws = _lib.workspace(lib.gpk_conjugate_mll_batched_workspace_bytes(B, n, d), dev)
    _lib.call("gpk_conjugate_mll_batched", B, i32(*[int(k) for k in kinds]), n, d,
              ptr(*[x.data_ptr() for x in xs]), i64(*[x.shape[1] for x in xs]),
              ptr(*[y.data_ptr() for y in ys]), ptr(*[t.data_ptr() for t in thetas]),
              i32(*[int(v) for v in n_ls]), float(jitter), int(want_grad),
              ptr(*[mll.data_ptr() + 8 * i for i in range(B)]),
              ptr(*[g.data_ptr() for g in grads]), info.data_ptr(), ws.data_ptr(), ws.numel(),
              _lib.stream_ptr(dev))
    return mll, grads, info
