"""Generates tests/golden/golden_small.npz: seeded small exact-GP cases with the
oracle's float64 MLL, gradient and predictive mean/variance.

GPJax pins no golden value for these functions and JAX is not importable
where this runs, so the values come from the float64 oracle (oracle/gp_oracle.py),
itself pinned by the reference's known-answer tests; the fixtures freeze them
so that drift in either the oracle or the GPU path shows up.
Run: python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import gp_oracle as O  # noqa: E402

CASES = [  # (kind, n, d, ard, seed)
    (O.RBF, 1, 1, False, 0), (O.RBF, 2, 2, True, 1), (O.MATERN32, 17, 3, True, 2),
    (O.MATERN52, 65, 4, True, 3), (O.MATERN52, 129, 8, True, 4), (O.RBF, 200, 4, False, 5),
]


def main():
    out = {"ncases": np.array(len(CASES))}
    for i, (kind, n, d, ard, seed) in enumerate(CASES):
        rng = np.random.default_rng(seed)
        x = rng.standard_normal((n, d))
        y = np.sin(x).sum(1, keepdims=True) + 0.1 * rng.standard_normal((n, 1))
        ls = np.exp(rng.uniform(np.log(0.3), np.log(3.0), d)) if ard else np.array(1.0)
        var, sd, c = 1.3, 0.2, 0.1
        t = rng.standard_normal((7, d))
        mll, g = O.conjugate_mll_torch(kind, x, y, ls, var, sd, c)
        mean, cov = O.predict(kind, x, y, t, ls, var, sd, c)
        for k, v in dict(kind=kind, x=x, y=y, ls=ls, var=var, sd=sd, c=c, t=t, mll=mll,
                         g_ls=g["lengthscale"], g_var=g["variance"], g_sd=g["obs_stddev"],
                         g_c=g["constant"], mean=mean, var_pred=np.diag(cov)).items():
            out[f"c{i}_{k}"] = np.asarray(v)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden_small.npz")
    np.savez_compressed(path, **out)
    print("wrote", path)


if __name__ == "__main__":
    main()
