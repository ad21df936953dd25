"""The C-ABI library builds, loads and exports every symbol include/scess_cc.h declares (CPU only)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, 'include', 'scess_cc.h')).read()
    src = re.sub(r'/\*.*?\*/', '', src, flags=re.S)
    return sorted(set(re.findall(r'\b(scess_[a-z0-9_]+)\s*\(', src)) - {'scess_cancel_fn', 'scess_log_fn'})


@pytest.fixture(scope='module')
def lib():
    from scess_gb300 import build
    build.build()
    from scess_gb300 import load_library
    return load_library()


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 12
    for n in names:
        assert hasattr(lib, n), n


def test_python_binding_covers_header():
    from scess_gb300 import EXPORTS
    assert set(declared_functions()) == set(EXPORTS)


def test_status_strings(lib):
    assert lib.scess_status_string(0) == b'ok'
    assert lib.scess_status_string(4) == b'cancelled'


def test_default_options_match_reference_constants(lib):
    from scess_gb300.cc import Options
    import ctypes
    o = Options()
    lib.scess_rccsd_default_options(ctypes.byref(o))
    # RCCSD.cpp:302-307
    assert o.energy_convergence == 1e-10
    assert o.amplitude_convergence == 1e-8
    assert o.max_iterations == 100
    assert o.diis_start == 2
    assert o.max_diis_vectors == 8
    assert o.precision == 0


def test_options_struct_layout():
    """ctypes mirror of scess_rccsd_options has the C layout (checked with the C compiler)."""
    import ctypes
    import subprocess
    import tempfile
    from scess_gb300.cc import Options, Result
    code = ('#include <stdio.h>\n#include <stddef.h>\n#include "scess_cc.h"\n'
            'int main(){printf("%zu %zu %zu %zu\\n", sizeof(scess_rccsd_options),'
            ' offsetof(scess_rccsd_options, time_limit_s), sizeof(scess_rccsd_result),'
            ' offsetof(scess_rccsd_result, last_rms));return 0;}\n')
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, 'a.c')
        open(c, 'w').write(code)
        exe = os.path.join(d, 'a')
        subprocess.check_call(['gcc', '-I', os.path.join(ROOT, 'include'), c, '-o', exe])
        out = subprocess.check_output([exe]).decode().split()
    assert int(out[0]) == ctypes.sizeof(Options)
    assert int(out[1]) == Options.time_limit_s.offset
    assert int(out[2]) == ctypes.sizeof(Result)
    assert int(out[3]) == Result.last_rms.offset


def test_no_cpu_fallback_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip('GPU present')
    import scess_gb300 as s
    with pytest.raises(s.ScessError):
        s.Context(0)
