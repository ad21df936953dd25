"""The C++ shim of INTEGRATION.md, compiled as a maintainer would add it to
SCESS: the first C++ block of INTEGRATION.md (SolveRCCSD_DIIS and
RCCSD_TriplesCorrection over the C ABI) is built with g++ against
include/scess_cc.h and stand-ins for the Eigen / SCESS types it touches
(tests/shim/stub), linked with libscess_cc.so and driven by tests/shim/drive.cpp.

CPU: the shim compiles and links.  GPU: the linked program reproduces the
reference's H2O/cc-pVDZ energies (src/SCESS/Tests.cpp:594-607)."""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(ROOT, 'tests', 'shim')


def _shim_source() -> str:
    text = open(os.path.join(ROOT, 'INTEGRATION.md')).read()
    blocks = re.findall(r'```cpp\n(.*?)```', text, flags=re.S)
    assert blocks, 'INTEGRATION.md has no C++ block'
    return blocks[0]


@pytest.fixture(scope='module')
def drive(tmp_path_factory):
    if shutil.which('g++') is None:
        pytest.skip('g++ not available')
    from scess_gb300 import build
    lib = build.build()
    d = tmp_path_factory.mktemp('shim')
    src = d / 'RCCSD_GB300.cpp'
    src.write_text(_shim_source())
    exe = d / 'drive'
    cmd = ['g++', '-std=c++20', '-O1', '-I', os.path.join(SHIM, 'stub'),
           '-I', os.path.join(ROOT, 'include'), str(src), os.path.join(SHIM, 'drive.cpp'),
           '-L', os.path.dirname(lib), '-lscess_cc', f'-Wl,-rpath,{os.path.dirname(lib)}',
           '-o', str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def test_shim_compiles_and_links(drive):
    assert os.access(drive, os.X_OK)
    r = subprocess.run([str(drive)], capture_output=True, text=True)
    assert r.returncode == 2  # usage error: no GPU work without arguments


@pytest.mark.gpu
def test_shim_reproduces_the_reference_h2o_energies(drive, tmp_path):
    from tests.golden import PINS, load
    d = load('h2o_ccpvdz')
    eri = np.asfortranarray(d['eri'], dtype=np.float64)
    n = eri.shape[0]
    (tmp_path / 'eri.bin').write_bytes(eri.ravel(order='F').tobytes())
    (tmp_path / 'eps.bin').write_bytes(np.asarray(d['eps'], dtype=np.float64).tobytes())
    r = subprocess.run([str(drive), str(tmp_path / 'eri.bin'), str(tmp_path / 'eps.bin'),
                        str(n), str(d['nocc'])], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-3000:]
    conv, e_ccsd, e_t = r.stdout.split()
    assert conv == '1'
    assert 'CCSD(' in r.stderr  # the per-iteration console lines reached the stringstream
    val, tol = PINS['h2o_ccpvdz']['E_CCSD']
    assert abs(float(e_ccsd) - val) <= tol
    val, tol = PINS['h2o_ccpvdz']['E_T']
    assert abs(float(e_t) - val) <= tol
