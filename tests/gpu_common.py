"""Shared helpers of the GPU tests."""
import numpy as np
import pytest


def ctx():
    import scess_gb300 as s
    if not hasattr(ctx, '_c'):
        ctx._c = s.Context(0)
    return ctx._c


def rel_err(x, ref):
    return float(np.max(np.abs(np.asarray(x) - ref)) / max(np.max(np.abs(ref)), 1e-300))


@pytest.fixture(scope='session')
def gctx():
    return ctx()
