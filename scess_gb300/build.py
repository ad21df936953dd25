"""Builds libscess_cc.so (the C-ABI engine) in-tree for sm_103a with nvcc.

Every translation unit is compiled in parallel with
``-gencode arch=compute_103a,code=sm_103a`` and linked into
``scess_gb300/libscess_cc.so`` (static CUDA runtime, no torch dependency).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, 'csrc')
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(HERE, 'libscess_cc.so')
SOURCES = ['kernels.cu', 'engine.cu', 'gemm_tc.cu', 'rccsd.cu', 'triples.cu', 'adjoint.cu',
           'capi.cu', 'einsum_static.cu', 'ccsd_so.cu']
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']


def nvcc() -> str:
    p = shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'
    if not os.path.exists(p):
        raise RuntimeError('nvcc not found')
    return p


def _flags(extra=()):
    return ARCH + ['-O3', '-std=c++17', '-lineinfo', '-Xcompiler', '-fPIC,-O3',
                   '-I', os.path.join(ROOT, 'include'), '--expt-relaxed-constexpr',
                   '-DNDEBUG'] + list(extra)


def _newest(paths):
    return max(os.path.getmtime(p) for p in paths)


def build(verbose: bool = False, force: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(('.h', '.cuh'))]
    headers.append(os.path.join(ROOT, 'include', 'scess_cc.h'))
    hdr_time = _newest(headers)
    objs, jobs = [], []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace('.cu', '.o'))
        objs.append(o)
        if force or not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), hdr_time):
            extra = ['-Xptxas', '-v'] if ptxas_info else []
            jobs.append([nvcc()] + _flags(extra) + ['-c', s, '-o', o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
        for cmd, r in zip(jobs, results):
            if verbose or r.returncode != 0 or ptxas_info:
                sys.stderr.write(r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError('nvcc failed: ' + ' '.join(cmd))
    if jobs or not os.path.exists(LIB) or os.path.getmtime(LIB) < _newest(objs):
        tmp = LIB + '.tmp'
        cmd = [nvcc()] + ARCH + ['-shared', '-o', tmp] + objs + ['-cudart', 'static']
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError('link failed')
        os.replace(tmp, LIB)
    return LIB


if __name__ == '__main__':
    print(build(verbose=True, force='--force' in sys.argv, ptxas_info='--ptxas' in sys.argv))
