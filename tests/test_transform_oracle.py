"""Oracle of the AO->MO transform (TransformTEI) against the golden fixtures: the
stored MO integrals were produced from the stored AO integrals and RHF
coefficients, so the restated transform must reproduce them."""
import numpy as np
import pytest

from oracle.transforms import transform_tei
from tests.golden import load


@pytest.mark.parametrize('tag', ['h2_sto3g', 'h2o_sto3g', 'h2o_ccpvdz'])
def test_transform_reproduces_fixture(tag):
    d = load(tag)
    mo = transform_tei(d['ao_chem'], d['C'], chem_to_phys=True)
    assert np.max(np.abs(mo - d['eri'])) < 1e-12


def test_transform_index_order():
    rng = np.random.default_rng(0)
    n = 5
    tei = rng.standard_normal((n, n, n, n))
    A, B, C, D = (rng.standard_normal((n, k)) for k in (2, 3, 4, 5))
    ref = np.einsum('mp,nq,mnkl,kr,ls->pqrs', A, B, tei, C, D)
    assert np.allclose(transform_tei(tei, A, B, C, D), ref, atol=1e-12)
    assert np.allclose(transform_tei(tei, A, B, C, D, chem_to_phys=True),
                       ref.transpose(0, 2, 1, 3), atol=1e-12)
