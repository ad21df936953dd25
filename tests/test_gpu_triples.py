"""(T) on the GPU against the FP64 oracle and the reference's pins."""
import numpy as np
import pytest

import oracle
from scess_gb300.synthetic import make_workload
from tests.golden import PINS, load
from tests.gpu_common import gctx  # noqa: F401

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('tag', ['h2o_sto3g', 'h2o_ccpvdz'])
def test_triples_reference_pins(gctx, tag):
    d = load(tag)
    ref = oracle.solve_rccsd_diis(d['eri'], d['eps'], d['nocc'])
    et_ref = oracle.rccsd_triples_correction(d['eri'], d['eps'], d['nocc'], ref.t1, ref.t2)
    et = gctx.triples(d['eri'], d['eps'], d['nocc'], ref.t1, ref.t2)
    assert abs(et - et_ref) <= 1e-11
    val, tol = PINS[tag]['E_T']
    assert abs(et - val) <= tol
    em = gctx.triples(d['eri'], d['eps'], d['nocc'], ref.t1, ref.t2, precision='mixed')
    assert abs(em - et_ref) <= 1e-7


@pytest.mark.parametrize('o,v', [(3, 7), (5, 19), (4, 41), (10, 90)])
def test_triples_fixed_amplitudes(gctx, o, v):
    w = make_workload(o, v, seed=0, with_amplitudes=True)
    eri = w.eri()
    ref = oracle.rccsd_triples_correction(eri, w.eps, o, w.t1, w.t2)
    et = gctx.triples(eri, w.eps, o, w.t1, w.t2)
    assert abs(et - ref) <= 1e-9 * max(1.0, abs(ref))
    # mixed: FP32 tensor-core accumulation, relative error ~1e-6 of |E_T| (these fixed
    # amplitudes give unphysically large |E_T|, up to 1e4 Eh)
    em = gctx.triples(eri, w.eps, o, w.t1, w.t2, precision='mixed')
    assert abs(em - ref) <= 2e-6 * max(1.0, abs(ref))


def test_triples_df_equals_eri(gctx):
    w = make_workload(5, 19, seed=1, with_amplitudes=True)
    a = gctx.triples(w.eri(), w.eps, 5, w.t1, w.t2)
    b = gctx.triples(None, w.eps, 5, w.t1, w.t2, B=w.B)
    assert abs(a - b) <= 1e-12 * max(1.0, abs(a))


@pytest.mark.parametrize('precision,tol', [('fp64', 1e-12), ('mixed', 2e-6)])
def test_triples_df_native_multiblock(gctx, monkeypatch, precision, tol):
    """DF input, integrals contracted from B without the nmo^4 eri, several
    block triples with padded virtuals; against the eri route in FP64."""
    from scess_gb300.synthetic import convergent_sigma
    monkeypatch.setenv('SCESS_TUNE', 't_nb=7')
    o, v = 6, 40
    w = make_workload(o, v, seed=4, with_amplitudes=True, sigma=convergent_sigma(o, v))
    ref = gctx.triples(w.eri(), w.eps, o, w.t1, w.t2, precision='fp64')
    got = gctx.triples(None, w.eps, o, w.t1, w.t2, B=w.B, precision=precision)
    assert abs(got - ref) <= tol * max(1.0, abs(ref))



@pytest.mark.parametrize('o,v,nb', [(5, 18, 4), (7, 23, 5), (8, 30, 5), (12, 26, 9)])
def test_triples_mixed_block_layouts(gctx, monkeypatch, o, v, nb):
    """Several block triples with padded virtuals; odd o (scalar reads of the
    grouped W buffers, padded S rows) and o % 4 == 0 (4-row vector reads)."""
    from scess_gb300.synthetic import convergent_sigma
    monkeypatch.setenv('SCESS_TUNE', f't_nb={nb}')
    w = make_workload(o, v, seed=6, with_amplitudes=True, sigma=convergent_sigma(o, v))
    eri = w.eri()
    em = gctx.triples(eri, w.eps, o, w.t1, w.t2, precision='mixed')
    ref = gctx.triples(eri, w.eps, o, w.t1, w.t2, precision='fp64')
    assert abs(em - ref) <= 2e-6 * max(1.0, abs(ref))


def test_overlapped_launches_equal_serialised(gctx, monkeypatch):
    """The mixed (T) overlaps each block triple's grouped GEMM and energy
    launches with their neighbours (programmatic dependent launches: the
    energy kernel reads W, and the next GEMM adds into it, only after the
    earlier grid is complete).  Serialised launches (t_pdl = 0) must give the
    same energy up to the order in which the three groups' reductions land,
    over many block triples."""
    from scess_gb300.synthetic import convergent_sigma
    o, v = 8, 60
    w = make_workload(o, v, seed=6, with_amplitudes=True, sigma=convergent_sigma(o, v))
    eri = w.eri()
    ref = oracle.rccsd_triples_correction(eri, w.eps, o, w.t1, w.t2)
    monkeypatch.setenv('SCESS_TUNE', 't_nb=5,t_pdl=1')    # 12 blocks: 364 block triples
    over = [gctx.triples(eri, w.eps, o, w.t1, w.t2, precision='mixed') for _ in range(3)]
    monkeypatch.setenv('SCESS_TUNE', 't_nb=5,t_pdl=0')
    ser = gctx.triples(eri, w.eps, o, w.t1, w.t2, precision='mixed')
    for e in over:
        assert abs(e - ser) <= 1e-9 * abs(ser), (e, ser)
    assert abs(ser - ref) <= 2e-6 * max(1.0, abs(ref))
