"""Contraction engine on the GPU: FP64 (DFMA) and tensor-core (tcgen05, split BF16) backends
against NumPy float64 einsum, including permuted operands, split-K and GEMV shapes."""
import numpy as np
import pytest

from tests.gpu_common import gctx, rel_err  # noqa: F401

pytestmark = pytest.mark.gpu

CASES = [
    ('mk,nk->mn', (128, 64), (256, 64)),
    ('mk,nk->mn', (300, 1000), (200, 1000)),
    ('mk,nk->mn', (1000, 50), (20, 50)),
    ('mk,nk->mn', (64, 7000), (500, 7000)),
    ('kcld,ilcd->ki', (5, 19, 5, 19), (5, 5, 19, 19)),
    ('kcld,klad->ac', (6, 33, 6, 33), (6, 6, 33, 33)),
    ('akic,kjcb->ijab', (21, 7, 7, 21), (7, 7, 21, 21)),
    ('abcd,ijcd->ijab', (30, 30, 30, 30), (9, 9, 30, 30)),
    ('kdac,ikcd->ia', (8, 40, 40, 40), (8, 8, 40, 40)),
    ('ka,kbij->ijab', (10, 90), (10, 90, 10, 10)),
    ('kcld,ld->kc', (10, 90, 10, 90), (10, 90)),
    ('kc,kica->ia', (10, 90), (10, 10, 90, 90)),
    ('ia,jb->ijab', (7, 11), (7, 11)),
    # operand packs whose tiles run along a row label that is not the first of
    # the row group (a of (i, a, b)), and gathers that cover their whole source
    ('abic,jc->ijab', (40, 40, 6, 40), (6, 40)),
    ('kibc,ka->abic', (6, 6, 40, 40), (6, 40)),
    ('cbai,jc->ijab', (36, 36, 36, 5), (5, 36)),
    ('ldkc,ilda->akic', (5, 33, 5, 33), (5, 5, 33, 33)),
]


def _operands(spec, sa, sb, seed=0):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal(sa)
    B = rng.standard_normal(sb)
    ref = np.einsum(spec, A, B)
    return A, B, ref


@pytest.mark.parametrize('spec,sa,sb', CASES)
def test_einsum_fp64(gctx, spec, sa, sb):
    A, B, ref = _operands(spec, sa, sb)
    C0 = np.random.default_rng(1).standard_normal(ref.shape)
    out = gctx.einsum(spec, A, B, C_init=C0, alpha=-0.5, beta=2.0, precision='fp64')
    assert rel_err(out, -0.5 * ref + 2.0 * C0) < 1e-13


@pytest.mark.parametrize('spec,sa,sb', CASES)
def test_einsum_tensor_cores(gctx, spec, sa, sb):
    # scaled FP16 hi+lo operands, FP32 accumulation: below 5e-6 of max|C| (measured ~2e-6)
    A, B, ref = _operands(spec, sa, sb)
    C0 = np.random.default_rng(2).standard_normal(ref.shape)
    out = gctx.einsum(spec, A, B, C_init=C0, alpha=1.5, beta=1.0, precision='mixed')
    assert rel_err(out, 1.5 * ref + C0) < 5e-6


def test_tensor_core_gemm_exact_on_bf16_values(gctx):
    # integers representable in BF16 with small sums: the tensor-core result is exact
    rng = np.random.default_rng(3)
    A = rng.integers(-8, 9, (384, 256)).astype(np.float64)
    B = rng.integers(-8, 9, (272, 256)).astype(np.float64)
    out = gctx.einsum('mk,nk->mn', A, B, out_shape=(384, 272), precision='mixed')
    assert np.array_equal(out, A @ B.T)


def test_fp64_einsum_deterministic(gctx):
    A, B, _ = _operands('kdac,ikcd->ia', (8, 40, 40, 40), (8, 8, 40, 40))
    o1 = gctx.einsum('kdac,ikcd->ia', A, B, out_shape=(8, 40))
    o2 = gctx.einsum('kdac,ikcd->ia', A, B, out_shape=(8, 40))
    assert np.array_equal(o1, o2)


SKINNY = [
    # (spec, A shape, B shape): K <= 32 and one free side of at most 256, the
    # other long: FP32 on the CUDA cores in the mixed form
    ('ki,kjab->ijab', (20, 20), (20, 20, 30, 30)),     # small side A, C unit stride on it
    ('lcki,la->akci', (20, 30, 20, 20), (20, 30)),     # small side B, C unit stride on it
    ('ka,kbij->ijab', (20, 30), (20, 30, 20, 20)),     # small side A, C unit stride on the long side
    ('kibj,ka->ijab', (12, 12, 40, 12), (12, 40)),
    ('mk,kn->mn', (250, 7), (7, 5000)),
]


@pytest.mark.parametrize('spec,sa,sb', SKINNY)
@pytest.mark.parametrize('alpha,beta', [(1.0, 1.0), (-2.0, 0.0), (0.5, 0.75)])
def test_skinny_contractions(gctx, spec, sa, sb, alpha, beta):
    # operands rounded to FP32, FP32 products and K sums: below 2e-6 of max|C|
    A, B, ref = _operands(spec, sa, sb, seed=5)
    C0 = np.random.default_rng(6).standard_normal(ref.shape)
    out = gctx.einsum(spec, A, B, C_init=C0, alpha=alpha, beta=beta, precision='mixed')
    assert rel_err(out, alpha * ref + beta * C0) < 2e-6
    # the FP64 form of the same contraction is unaffected
    out64 = gctx.einsum(spec, A, B, C_init=C0, alpha=alpha, beta=beta, precision='fp64')
    assert rel_err(out64, alpha * ref + beta * C0) < 1e-13
