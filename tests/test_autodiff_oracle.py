"""The torch restatement of the residual equals the NumPy oracle (CPU)."""
import numpy as np
import torch

import oracle
from oracle import autodiff
from scess_gb300.synthetic import make_workload


def test_torch_residual_matches_numpy_oracle():
    o, v = 3, 7
    w = make_workload(o, v, seed=2)
    eri = w.eri()
    rng = np.random.default_rng(0)
    t1 = 0.05 * rng.standard_normal((o, v))
    t2 = 0.05 * rng.standard_normal((o, o, v, v))
    ints = oracle.make_integral_blocks(eri, o)
    eia, eijab = oracle.rccsd.denominators(w.eps, o)
    u1, u2 = oracle.update_amplitudes(ints, eia, eijab, None, t1, t2)
    r1, r2 = autodiff.residual_numerators(torch.tensor(eri), o, torch.tensor(t1), torch.tensor(t2))
    assert np.allclose(r1.numpy() / eia, u1, atol=1e-13)
    assert np.allclose(r2.numpy() / eijab, u2, atol=1e-13)


def test_autograd_vjp_matches_finite_differences():
    o, v = 2, 5
    w = make_workload(o, v, seed=3)
    eri = w.eri()
    rng = np.random.default_rng(1)
    t1 = 0.05 * rng.standard_normal((o, v))
    t2 = 0.05 * rng.standard_normal((o, o, v, v))
    g1 = rng.standard_normal((o, v))
    g2 = rng.standard_normal((o, o, v, v))
    gt1, gt2, ge = autodiff.residual_vjp(eri, o, t1, t2, g1, g2)
    d1, d2, de = (rng.standard_normal(x.shape) for x in (t1, t2, eri))
    h = 1e-5

    def f(s):
        r1, r2 = autodiff.residual_numerators(torch.tensor(eri + s * de), o,
                                              torch.tensor(t1 + s * d1), torch.tensor(t2 + s * d2))
        return float((r1.numpy() * g1).sum() + (r2.numpy() * g2).sum())
    fd = (f(h) - f(-h)) / (2 * h)
    an = float((gt1 * d1).sum() + (gt2 * d2).sum() + (ge * de).sum())
    assert abs(fd - an) <= 1e-7 * max(1.0, abs(an))
