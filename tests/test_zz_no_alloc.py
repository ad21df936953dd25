"""scess_einsum_static: the contraction entry point that allocates no device memory.

It serves programs that cannot call cudaMalloc: a framework whose caching
allocator already holds the GPU's memory, or an application that reserves a
fixed arena at start-up and forbids allocations afterwards.  They pass their
own device buffers; the library's only scratch is a fixed 16 MiB array shared
by all calls.

The GPU test compares it with scess_einsum (FP64) and with NumPy on the host,
within the 1e-13 relative tolerance of the other FP64 contraction tests, over
calls in a row that reuse the array (a split-K case, a different shape with
beta != 0, the first case again).  The file is named so that pytest collects it last: a run that stops
at the first failure has then already run every other test.
"""
import numpy as np
import pytest

from scess_gb300 import cc

# (spec, extents per label, alpha, beta): the first two split K (the partial
# sums live in the array), the third has no summed label and no split.
CASES = [
    ('kcld,ilcd->ki', dict(k=10, c=30, l=10, d=30, i=10), 1.0, 0.0),
    ('abcd,ijcd->ijab', dict(a=24, b=24, c=24, d=24, i=6, j=6), -0.5, 2.0),
    ('ia,jb->ijab', dict(i=12, a=60, j=12, b=60), 0.75, 1.0),
]


def _shapes(spec, ext):
    lhs, c = spec.split('->')
    a, b = lhs.split(',')
    return tuple(tuple(ext[x] for x in t) for t in (a, b, c))


def _rel_err(x, ref):
    return float(np.max(np.abs(x - ref)) / max(np.max(np.abs(ref)), 1e-300))


@pytest.fixture(scope='module')
def lib():
    from scess_gb300 import build
    build.build()
    return cc.load_library()


def test_rejects_before_touching_the_gpu(lib):
    """Too-large and malformed requests return at once (no CUDA call: runs on CPU too)."""
    fake = 1 << 20  # never dereferenced: the checks come first
    # 'i,j->ij' with M + N + K = 1,100,000 + 1 + 1 > 1,048,576
    assert cc.einsum_static('i,j->ij', fake, [1_100_000], fake, [1], fake, [1_100_000, 1]) \
        == cc.SCESS_ERR_TOO_LARGE
    assert lib.scess_status_string(cc.SCESS_ERR_TOO_LARGE) == b'too large for the fixed scratch'
    assert cc.einsum_static('ij,jk->ik', fake, [4, 5], fake, [6, 3], fake, [4, 3]) \
        == cc.SCESS_ERR_INVALID  # extent mismatch of j
    assert cc.einsum_static('ij,jk->ii', fake, [4, 5], fake, [5, 3], fake, [4, 4]) \
        == cc.SCESS_ERR_INVALID  # repeated label
    assert cc.einsum_static('ij,jk->ik', 0, [4, 5], fake, [5, 3], fake, [4, 3]) \
        == cc.SCESS_ERR_INVALID  # null pointer


@pytest.mark.gpu
def test_matches_scess_einsum_on_consecutive_calls(lib):
    torch = pytest.importorskip('torch')
    import scess_gb300 as s
    ctx = s.Context(0)
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(7)
    for spec, ext, alpha, beta in CASES + CASES[:1]:
        sa, sb, sc = _shapes(spec, ext)
        A = rng.standard_normal(sa)
        B = rng.standard_normal(sb)
        C0 = rng.standard_normal(sc)
        ref = ctx.einsum(spec, A, B, C_init=C0, alpha=alpha, beta=beta, precision='fp64')
        dev = [torch.from_numpy(np.asfortranarray(x).ravel(order='F').copy()).to('cuda:0')
               for x in (A, B, C0)]
        st = cc.einsum_static(spec, dev[0].data_ptr(), sa, dev[1].data_ptr(), sb,
                              dev[2].data_ptr(), sc, alpha=alpha, beta=beta, stream=stream)
        assert st == cc.SCESS_OK, (spec, st)
        torch.cuda.synchronize()
        out = dev[2].cpu().numpy().reshape(sc, order='F')
        assert _rel_err(out, ref) < 1e-13, spec
        # and against the host: the same kernels behind both entry points could
        # share a fault
        host = alpha * np.einsum(spec, A, B) + beta * C0
        assert _rel_err(out, host) < 1e-13, spec


@pytest.mark.gpu
def test_rejects_buffers_that_are_not_device_memory(lib):
    """A host buffer would fault in the kernels: the entry point refuses it
    before queueing work and leaves the device buffers untouched."""
    torch = pytest.importorskip('torch')
    a = np.ones((4, 5))
    Bd = torch.ones(5 * 3, dtype=torch.float64, device='cuda:0')
    Cd = torch.full((4 * 3,), 7.0, dtype=torch.float64, device='cuda:0')
    st = cc.einsum_static('ij,jk->ik', a.ctypes.data, [4, 5], Bd.data_ptr(), [5, 3],
                          Cd.data_ptr(), [4, 3])
    assert st == cc.SCESS_ERR_INVALID
    torch.cuda.synchronize()
    assert bool((Cd == 7.0).all())


@pytest.mark.gpu
def test_too_large_leaves_output_untouched(lib):
    torch = pytest.importorskip('torch')
    n = 1_100_000
    A = torch.ones(n, dtype=torch.float64, device='cuda:0')
    B = torch.ones(1, dtype=torch.float64, device='cuda:0')
    C = torch.full((n,), 3.0, dtype=torch.float64, device='cuda:0')
    st = cc.einsum_static('i,j->ij', A.data_ptr(), [n], B.data_ptr(), [1], C.data_ptr(), [n, 1])
    assert st == cc.SCESS_ERR_TOO_LARGE
    torch.cuda.synchronize()
    assert bool((C == 3.0).all())
