"""The accuracy bar of the mixed form at o=20, v=180 (nmo = 200), the headline
workload: converged mixed-precision CCSD and (T) against the FP64 path on the
same seeded synthetic DF integrals (the convergent variant of the generator),
through the drop-in calls with the nmo^4 eri, as SolveRCCSD_DIIS and
RCCSD_TriplesCorrection take it (RCCSD.cpp:295-394, RCCSD_T.cpp:17-168).

Bar: |dE| <= 1 uEh for E_CCSD, for E_(T) on the same amplitudes and for the
whole correlation energy E_CCSD + E_(T) of the two chains."""
import numpy as np
import pytest

from scess_gb300.synthetic import convergent_sigma, make_workload
from tests.gpu_common import gctx  # noqa: F401

pytestmark = pytest.mark.gpu

O, V = 20, 180
MICRO_EH = 1e-6


@pytest.fixture(scope='module')
def solved(gctx):
    torch = pytest.importorskip('torch')
    import bench
    w = make_workload(O, V, seed=0, sigma=convergent_sigma(O, V))
    host, eri = bench.build_eri_pinned(w, torch)  # column-major, pinned: passed without a copy
    f = gctx.solve(eri, w.eps, O, precision='fp64')
    m = gctx.solve(eri, w.eps, O, precision='mixed')
    et = {}
    if f.converged and m.converged:
        et['fp64'] = gctx.triples(eri, w.eps, O, f.t1, f.t2, precision='fp64')
        et['mixed_same'] = gctx.triples(eri, w.eps, O, f.t1, f.t2, precision='mixed')
        et['mixed'] = gctx.triples(eri, w.eps, O, m.t1, m.t2, precision='mixed')
    yield w, f, m, et
    del eri, host


def test_converged_mixed_ccsd_within_a_microhartree(solved):
    w, f, m, et = solved
    assert f.converged and m.converged
    # the mixed solve ran mixed iterations, then FP64 refinement
    assert 0 < m.mixed_iterations < m.iterations
    assert abs(m.E_CCSD - f.E_CCSD) <= MICRO_EH, (m.E_CCSD, f.E_CCSD)
    assert np.max(np.abs(m.t2 - f.t2)) < 1e-6


def test_mixed_triples_within_a_microhartree(solved):
    w, f, m, et = solved
    assert abs(et['mixed_same'] - et['fp64']) <= MICRO_EH, (et['mixed_same'], et['fp64'])
    total_m = m.E_CCSD + et['mixed']
    total_f = f.E_CCSD + et['fp64']
    assert abs(total_m - total_f) <= MICRO_EH, (total_m, total_f)
