"""Python mirror of SCESS's closed-shell CC interface over the C ABI (libscess_cc.so).

``SolveRCCSD_DIIS`` and ``RCCSD_TriplesCorrection`` keep the names, argument
meaning and error behaviour of ``src/Quantum/CC/CC.h:136-158``:

* arrays are indexed like the reference's Eigen tensors (``eri[p,q,r,s] =
  <pq|rs>``, ``t1[i,a]``, ``t2[i,j,a,b]``); they are handed to the library as
  column-major (Fortran-order) buffers, exactly an Eigen tensor's memory;
* ``thread`` is any object with ``ShouldStop()``; when it asks to stop,
  ``SolveRCCSD_DIIS`` returns an empty ``RCCSD_Wfn`` and
  ``RCCSD_TriplesCorrection`` returns 0.0 (RCCSD.cpp:346-347, RCCSD_T.cpp:161-162);
* ``console`` is any object with ``write(str)``; it receives the reference's
  per-iteration lines;
* non-convergence gives ``converged = False`` with zero energies and no
  amplitudes (RCCSD.cpp:376-380).

Every other failure raises :class:`ScessError` carrying the C status.  The
library is GPU-only: there is no CPU fallback, and loading fails loudly when
``libscess_cc.so`` is missing.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, 'libscess_cc.so')

SCESS_OK = 0
SCESS_ERR_INVALID = 1
SCESS_ERR_OOM = 2
SCESS_ERR_CUDA = 3
SCESS_ERR_CANCELLED = 4
SCESS_ERR_TIMEOUT = 5
SCESS_ERR_UNSUPPORTED = 6
SCESS_ERR_TOO_LARGE = 7
PRECISION = {'fp64': 0, 'mixed': 1}


class ScessError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f'{message} (status {status})')
        self.status = status


class Options(C.Structure):
    """scess_rccsd_options (include/scess_cc.h)."""
    _fields_ = [('energy_convergence', C.c_double), ('amplitude_convergence', C.c_double),
                ('max_iterations', C.c_int32), ('diis_start', C.c_int32),
                ('max_diis_vectors', C.c_int32), ('precision', C.c_int32),
                ('refine_sweeps', C.c_int32),
                ('mixed_energy_switch', C.c_double), ('mixed_amplitude_switch', C.c_double),
                ('resume', C.c_int32),
                ('checkpoint_t1', C.POINTER(C.c_double)), ('checkpoint_t2', C.POINTER(C.c_double)),
                ('checkpoint_capacity', C.c_int32), ('history', C.POINTER(C.c_double)),
                ('time_limit_s', C.c_double)]


class Result(C.Structure):
    """scess_rccsd_result (include/scess_cc.h)."""
    _fields_ = [('E_CCSD', C.c_double), ('E_F12_Coupling', C.c_double), ('E_T', C.c_double),
                ('converged', C.c_int32), ('iterations', C.c_int32),
                ('mixed_iterations', C.c_int32), ('last_dE', C.c_double),
                ('last_rms', C.c_double), ('fp64_iterations', C.c_int32)]


CANCEL_FN = C.CFUNCTYPE(C.c_int, C.c_void_p)
LOG_FN = C.CFUNCTYPE(None, C.c_int, C.c_char_p, C.c_void_p)
_dp = C.POINTER(C.c_double)
_i64p = C.POINTER(C.c_int64)

EXPORTS = {
    'scess_status_string': (C.c_char_p, [C.c_int]),
    'scess_launch_count': (C.c_int64, []),
    'scess_ctx_create': (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    'scess_ctx_destroy': (None, [C.c_void_p]),
    'scess_ctx_last_error': (C.c_char_p, [C.c_void_p]),
    'scess_ctx_set_callbacks': (C.c_int, [C.c_void_p, CANCEL_FN, LOG_FN, C.c_void_p]),
    'scess_ctx_set_memory_limit': (C.c_int, [C.c_void_p, C.c_int64]),
    'scess_ctx_memory_held': (C.c_int64, [C.c_void_p]),
    'scess_ctx_arm_wait_expiry': (C.c_int, [C.c_void_p, C.c_int64]),
    'scess_rccsd_default_options': (None, [C.POINTER(Options)]),
    'scess_rccsd_solve': (C.c_int, [C.c_void_p, _dp, _dp, C.c_int64, C.c_int64, _dp, _dp,
                                    C.POINTER(Options), _dp, _dp, C.POINTER(Result)]),
    'scess_rccsd_solve_df': (C.c_int, [C.c_void_p, _dp, C.c_int64, _dp, C.c_int64, C.c_int64,
                                       _dp, _dp, C.POINTER(Options), _dp, _dp,
                                       C.POINTER(Result)]),
    'scess_rccsd_triples': (C.c_int, [C.c_void_p, _dp, _dp, C.c_int64, C.c_int64, _dp, _dp,
                                      C.c_int32, _dp]),
    'scess_rccsd_triples_df': (C.c_int, [C.c_void_p, _dp, C.c_int64, _dp, C.c_int64, C.c_int64,
                                         _dp, _dp, C.c_int32, _dp]),
    'scess_rccsd_state_create': (C.c_int, [C.c_void_p, _dp, _dp, C.c_int64, C.c_int64, _dp, _dp,
                                           C.POINTER(Options), C.POINTER(C.c_void_p)]),
    'scess_rccsd_state_create_df': (C.c_int, [C.c_void_p, _dp, C.c_int64, _dp, C.c_int64,
                                              C.c_int64, _dp, _dp, C.POINTER(Options),
                                              C.POINTER(C.c_void_p)]),
    'scess_rccsd_state_destroy': (None, [C.c_void_p]),
    'scess_rccsd_state_iterate': (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(Result),
                                            C.POINTER(C.c_double)]),
    'scess_rccsd_state_triples': (C.c_int, [C.c_void_p, C.c_int32, _dp, C.POINTER(C.c_double)]),
    'scess_rccsd_state_amplitudes': (C.c_int, [C.c_void_p, _dp, _dp]),
    'scess_rccsd_state_set_amplitudes': (C.c_int, [C.c_void_p, _dp, _dp]),
    'scess_ctx_profile': (C.c_int, [C.c_void_p, C.c_int32]),
    'scess_ctx_profile_report': (C.c_int, [C.c_void_p, C.c_char_p, C.c_int64]),
    'scess_rccsd_residual': (C.c_int, [C.c_void_p, _dp, C.c_int64, C.c_int64, _dp, _dp, _dp,
                                       C.c_int32, _dp, _dp]),
    'scess_rccsd_residual_df': (C.c_int, [C.c_void_p, _dp, C.c_int64, C.c_int64, C.c_int64, _dp,
                                          _dp, _dp, C.c_int32, _dp, _dp]),
    'scess_rccsd_residual_vjp': (C.c_int, [C.c_void_p, _dp, C.c_int64, C.c_int64, _dp, _dp, _dp,
                                           _dp, C.c_int32, _dp, _dp, _dp]),
    'scess_rccsd_residual_vjp_df': (C.c_int, [C.c_void_p, _dp, C.c_int64, C.c_int64, C.c_int64,
                                              _dp, _dp, _dp, _dp, C.c_int32, _dp, _dp, _dp]),
    'scess_rccsd_lambda': (C.c_int, [C.c_void_p, _dp, _dp, C.c_int64, C.c_int64, _dp, _dp,
                                     C.POINTER(Options), _dp, _dp, C.POINTER(Result)]),
    'scess_rccsd_rdm1': (C.c_int, [C.c_void_p, _dp, _dp, C.c_int64, C.c_int64, _dp, _dp, _dp, _dp,
                                   C.c_int32, _dp]),
    'scess_einsum': (C.c_int, [C.c_void_p, C.c_char_p, C.c_double, _dp, C.c_int32, _i64p, _dp,
                               C.c_int32, _i64p, C.c_double, _dp, C.c_int32, _i64p, C.c_int32]),
    'scess_rccsd_triples_vjp': (C.c_int, [C.c_void_p, _dp, _dp, C.c_int64, C.c_int64, _dp, _dp,
                                          C.c_int32, C.c_double, C.POINTER(C.c_double), _dp, _dp,
                                          _dp]),
    'scess_rccsd_triples_vjp_df': (C.c_int, [C.c_void_p, _dp, C.c_int64, _dp, C.c_int64,
                                             C.c_int64, _dp, _dp, C.c_int32, C.c_double,
                                             C.POINTER(C.c_double), _dp, _dp, _dp]),
    'scess_transform_tei': (C.c_int, [C.c_void_p, _dp, C.c_int64, _dp, C.c_int64, _dp, C.c_int64,
                                      _dp, C.c_int64, _dp, C.c_int64, C.c_int32, C.c_int32, _dp]),
    'scess_f12b_coupling': (C.c_int, [C.c_void_p, _dp, _dp, _dp, _dp, C.c_int64, C.c_int64,
                                      C.c_int32, _dp, _dp]),
    'scess_mp2_energy': (C.c_int, [C.c_void_p, _dp, _dp, C.c_int64, C.c_int64, _dp]),
    'scess_ccsd_so_solve': (C.c_int, [C.c_void_p, _dp, _dp, C.c_int64, C.c_int64, C.c_int32,
                                      C.c_int32, _dp, _dp, _dp, C.POINTER(Result)]),
    'scess_ccsd_so_triples': (C.c_int, [C.c_void_p, _dp, _dp, C.c_int64, C.c_int64, _dp, _dp,
                                        C.POINTER(C.c_double)]),
    'scess_mp2_energy_ao': (C.c_int, [C.c_void_p, _dp, _dp, _dp, C.c_int64, C.c_int64, C.c_int64,
                                      C.c_int32, _dp]),
    'scess_einsum_static': (C.c_int, [C.c_char_p, C.c_double, C.c_void_p, C.c_int32, _i64p,
                                      C.c_void_p, C.c_int32, _i64p, C.c_double, C.c_void_p,
                                      C.c_int32, _i64p, C.c_void_p]),
}

_lib = None


def load_library(path: str = LIB_PATH):
    """Loads libscess_cc.so and declares every exported C symbol."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ScessError(SCESS_ERR_UNSUPPORTED,
                         f'{path} is missing: build it with `python -m scess_gb300.build`')
    lib = C.CDLL(path)
    for name, (res, args) in EXPORTS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _f64(x, shape=None):
    a = np.asfortranarray(np.asarray(x, dtype=np.float64))
    if shape is not None and a.shape != tuple(shape):
        raise ScessError(SCESS_ERR_INVALID, f'expected shape {tuple(shape)}, got {a.shape}')
    return a


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_dp)


@dataclass
class RCCSD_Wfn:
    """RCCSD_Wfn, CC.h:105-115 (plus iteration bookkeeping)."""
    E_CCSD: float = 0.0
    E_F12_Coupling: float = 0.0
    E_T: float = 0.0
    converged: bool = False
    t1: np.ndarray | None = None
    t2: np.ndarray | None = None
    iterations: int = 0
    mixed_iterations: int = 0
    history: np.ndarray | None = field(default=None, repr=False)


@dataclass
class CCSD_Wfn:
    """CCSD_Wfn, CC.h:28-35: the spin-orbital solvers' result (spin orbital
    p = 2 x spatial + spin, occupied first)."""
    E_CCSD: float = 0.0
    E_T: float = 0.0
    t1: np.ndarray | None = None
    t2: np.ndarray | None = None
    mints: np.ndarray | None = field(default=None, repr=False)
    converged: bool = False
    iterations: int = 0


@dataclass
class RCCSD_F12Coupling:
    """RCCSD_F12Coupling, CC.h:121-124: both indexed (i, j, a, b)."""
    residual: np.ndarray
    energy: np.ndarray


class Context:
    """One GPU context (scess_ctx): device memory, stream and callbacks."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        h = C.c_void_p()
        st = self.lib.scess_ctx_create(device, C.byref(h))
        if st != SCESS_OK:
            raise ScessError(st, 'scess_ctx_create: ' + self.lib.scess_status_string(st).decode())
        self.h = h
        self._thread = None
        self._console = None
        self._cancel = CANCEL_FN(self._cancel_cb)
        self._log = LOG_FN(self._log_cb)
        self.lib.scess_ctx_set_callbacks(self.h, self._cancel, self._log, None)

    def close(self):
        if getattr(self, 'h', None):
            self.lib.scess_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _cancel_cb(self, user):
        t = self._thread
        try:
            return 1 if (t is not None and t.ShouldStop()) else 0
        except Exception:
            return 1

    def _log_cb(self, level, msg, user):
        if self._console is not None:
            self._console.write(msg.decode() + '\n')

    def _check(self, st, what):
        if st != SCESS_OK:
            msg = self.lib.scess_ctx_last_error(self.h).decode()
            raise ScessError(st, f'{what}: {msg}')

    # -- device memory and diagnostics -------------------------------------------------------
    def set_memory_limit(self, nbytes: int):
        """Caps the device memory this context's calls hold (0: no cap)."""
        self._check(self.lib.scess_ctx_set_memory_limit(self.h, int(nbytes)),
                    'scess_ctx_set_memory_limit')

    def memory_held(self) -> int:
        return int(self.lib.scess_ctx_memory_held(self.h))

    def arm_wait_expiry(self, wait_cycles: int = 1 << 20):
        """The next tensor-core launch runs out its bounded pipeline wait."""
        self._check(self.lib.scess_ctx_arm_wait_expiry(self.h, int(wait_cycles)),
                    'scess_ctx_arm_wait_expiry')

    # -- options ---------------------------------------------------------------------------
    def default_options(self) -> Options:
        o = Options()
        self.lib.scess_rccsd_default_options(C.byref(o))
        return o

    # -- SolveRCCSD_DIIS ----------------------------------------------------------------------
    def solve(self, eri=None, eps=None, nocc=None, f12: RCCSD_F12Coupling | None = None,
              precision: str = 'fp64', B=None, thread=None, console=None, t1_init=None,
              t2_init=None, checkpoint=0, **opts) -> RCCSD_Wfn:
        eps = _f64(eps)
        N = eps.shape[0]
        o, v = int(nocc), N - int(nocc)
        op = self.default_options()
        op.precision = PRECISION[precision]
        for k, val in opts.items():
            setattr(op, k, val)
        hist = np.zeros(3 * max(op.max_iterations, 1))
        op.history = _ptr(hist)
        t1 = np.zeros((o, v), order='F')
        t2 = np.zeros((o, o, v, v), order='F')
        if t1_init is not None:
            t1[...] = t1_init
            t2[...] = t2_init
            op.resume = 1
        ck1 = ck2 = None
        if checkpoint:
            ck1 = np.zeros((checkpoint, o * v))
            ck2 = np.zeros((checkpoint, o * o * v * v))
            op.checkpoint_t1, op.checkpoint_t2 = _ptr(ck1), _ptr(ck2)
            op.checkpoint_capacity = checkpoint
        fr = fe = None
        if f12 is not None:
            fr = _f64(f12.residual, (o, o, v, v))
            fe = _f64(f12.energy, (o, o, v, v))
        res = Result()
        self._thread, self._console = thread, console
        try:
            if B is not None:
                Bf = _f64(B)
                st = self.lib.scess_rccsd_solve_df(self.h, _ptr(Bf), Bf.shape[0], _ptr(eps), N, o,
                                                   _ptr(fr), _ptr(fe), C.byref(op), _ptr(t1),
                                                   _ptr(t2), C.byref(res))
            else:
                ef = _f64(eri, (N, N, N, N))
                st = self.lib.scess_rccsd_solve(self.h, _ptr(ef), _ptr(eps), N, o, _ptr(fr),
                                                _ptr(fe), C.byref(op), _ptr(t1), _ptr(t2),
                                                C.byref(res))
        finally:
            self._thread, self._console = None, None
        if st == SCESS_ERR_CANCELLED:
            return RCCSD_Wfn()
        self._check(st, 'scess_rccsd_solve')
        w = RCCSD_Wfn(iterations=res.iterations, mixed_iterations=res.mixed_iterations,
                      history=hist[:3 * res.iterations].reshape(-1, 3))
        if checkpoint:
            w.checkpoints = (ck1, ck2)
        if not res.converged:
            return w
        w.converged = True
        w.E_CCSD = res.E_CCSD
        w.E_F12_Coupling = res.E_F12_Coupling
        w.t1, w.t2 = t1, t2
        return w

    # -- RCCSD_TriplesCorrection --------------------------------------------------------------
    def triples(self, eri=None, eps=None, nocc=None, t1=None, t2=None, precision: str = 'fp64',
                B=None, thread=None) -> float:
        eps = _f64(eps)
        N = eps.shape[0]
        o, v = int(nocc), N - int(nocc)
        t1f = _f64(t1, (o, v))
        t2f = _f64(t2, (o, o, v, v))
        et = C.c_double(0.0)
        self._thread = thread
        try:
            if B is not None:
                Bf = _f64(B)
                st = self.lib.scess_rccsd_triples_df(self.h, _ptr(Bf), Bf.shape[0], _ptr(eps), N,
                                                     o, _ptr(t1f), _ptr(t2f),
                                                     PRECISION[precision], C.byref(et))
            else:
                ef = _f64(eri, (N, N, N, N))
                st = self.lib.scess_rccsd_triples(self.h, _ptr(ef), _ptr(eps), N, o, _ptr(t1f),
                                                  _ptr(t2f), PRECISION[precision], C.byref(et))
        finally:
            self._thread = None
        if st == SCESS_ERR_CANCELLED:
            return 0.0
        self._check(st, 'scess_rccsd_triples')
        return et.value

    # -- device-resident session -------------------------------------------------------------
    def state(self, eri=None, eps=None, nocc=None, B=None, precision: str = 'fp64',
              f12: RCCSD_F12Coupling | None = None, **opts) -> 'State':
        return State(self, eri, eps, nocc, B=B, precision=precision, f12=f12, **opts)

    # -- kernel timing ------------------------------------------------------------------------
    def profile(self, enable: bool = True):
        self._check(self.lib.scess_ctx_profile(self.h, 1 if enable else 0), 'scess_ctx_profile')

    def profile_report(self) -> dict:
        import json
        buf = C.create_string_buffer(1 << 16)
        self._check(self.lib.scess_ctx_profile_report(self.h, buf, len(buf)),
                    'scess_ctx_profile_report')
        return json.loads(buf.value.decode())

    # -- one residual -------------------------------------------------------------------------
    def residual(self, eri, nocc, t1, t2, t2_driver=None, precision: str = 'fp64', B=None):
        """(t1new, t2new) numerators of UpdateAmplitudes (before the division), from
        the eri or, with B, from DF factors (scess_rccsd_residual_df)."""
        if B is not None:
            Bf = _f64(B)
            N = Bf.shape[1]
        else:
            ef = _f64(eri)
            N = ef.shape[0]
        o, v = int(nocc), N - int(nocc)
        t1f, t2f = _f64(t1, (o, v)), _f64(t2, (o, o, v, v))
        drv = None if t2_driver is None else _f64(t2_driver, (o, o, v, v))
        r1 = np.zeros((o, v), order='F')
        r2 = np.zeros((o, o, v, v), order='F')
        if B is not None:
            st = self.lib.scess_rccsd_residual_df(self.h, _ptr(Bf), Bf.shape[0], N, o, _ptr(t1f),
                                                  _ptr(t2f), _ptr(drv), PRECISION[precision],
                                                  _ptr(r1), _ptr(r2))
        else:
            st = self.lib.scess_rccsd_residual(self.h, _ptr(ef), N, o, _ptr(t1f), _ptr(t2f),
                                               _ptr(drv), PRECISION[precision], _ptr(r1), _ptr(r2))
        self._check(st, 'scess_rccsd_residual')
        return r1, r2

    # -- residual VJP -------------------------------------------------------------------------
    def residual_vjp(self, eri, nocc, t1, t2, g_r1, g_r2, precision='fp64', B=None,
                     want_integrals=False):
        """(g_t1, g_t2, g_eri or g_B) = VJP of the residual numerators."""
        o = int(nocc)
        if B is not None:
            Bf = _f64(B)
            N = Bf.shape[1]
        else:
            ef = _f64(eri)
            N = ef.shape[0]
        v = N - o
        args = [_f64(t1, (o, v)), _f64(t2, (o, o, v, v)), _f64(g_r1, (o, v)), _f64(g_r2, (o, o, v, v))]
        gt1 = np.zeros((o, v), order='F')
        gt2 = np.zeros((o, o, v, v), order='F')
        if B is not None:
            gI = np.zeros(Bf.shape, order='F') if want_integrals else None
            st = self.lib.scess_rccsd_residual_vjp_df(self.h, _ptr(Bf), Bf.shape[0], N, o,
                                                      *[_ptr(a) for a in args],
                                                      PRECISION[precision], _ptr(gt1), _ptr(gt2),
                                                      _ptr(gI))
        else:
            gI = np.zeros((N, N, N, N), order='F') if want_integrals else None
            st = self.lib.scess_rccsd_residual_vjp(self.h, _ptr(ef), N, o, *[_ptr(a) for a in args],
                                                   PRECISION[precision], _ptr(gt1), _ptr(gt2),
                                                   _ptr(gI))
        self._check(st, 'scess_rccsd_residual_vjp')
        return gt1, gt2, gI

    def triples_vjp(self, eri=None, eps=None, nocc=None, t1=None, t2=None, g_e=1.0, B=None,
                    want_integrals=False, precision='fp64'):
        """(E_T, g_t1, g_t2, g_eri or g_B): g_e times the gradient of E_(T)
        (FP64, or MIXED: its GEMMs on the tensor cores)."""
        eps = _f64(eps)
        N = eps.shape[0]
        o, v = int(nocc), N - int(nocc)
        t1f, t2f = _f64(t1, (o, v)), _f64(t2, (o, o, v, v))
        gt1 = np.zeros((o, v), order='F')
        gt2 = np.zeros((o, o, v, v), order='F')
        et = C.c_double(0.0)
        if B is not None:
            Bf = _f64(B)
            gI = np.zeros(Bf.shape, order='F') if want_integrals else None
            st = self.lib.scess_rccsd_triples_vjp_df(self.h, _ptr(Bf), Bf.shape[0], _ptr(eps), N, o,
                                                     _ptr(t1f), _ptr(t2f), PRECISION[precision],
                                                     float(g_e), C.byref(et), _ptr(gt1),
                                                     _ptr(gt2), _ptr(gI))
        else:
            ef = _f64(eri, (N, N, N, N))
            gI = np.zeros((N, N, N, N), order='F') if want_integrals else None
            st = self.lib.scess_rccsd_triples_vjp(self.h, _ptr(ef), _ptr(eps), N, o, _ptr(t1f),
                                                  _ptr(t2f), PRECISION[precision], float(g_e),
                                                  C.byref(et), _ptr(gt1), _ptr(gt2), _ptr(gI))
        self._check(st, 'scess_rccsd_triples_vjp')
        return et.value, gt1, gt2, gI

    def transform_tei(self, tei, A, B=None, C_=None, D=None, chem_to_phys=False,
                      precision='fp64'):
        """TransformTEI (IntegralTransforms.cpp:32-59) on the GPU; B, C_, D default to A."""
        t = _f64(tei)
        n = t.shape[0]
        mats = [_f64(m) for m in (A, A if B is None else B, A if C_ is None else C_,
                                  A if D is None else D)]
        na, nb, nc, nd = (m.shape[1] for m in mats)
        shape = (na, nc, nb, nd) if chem_to_phys else (na, nb, nc, nd)
        out = np.zeros(shape, order='F')
        st = self.lib.scess_transform_tei(self.h, _ptr(t), n, _ptr(mats[0]), na, _ptr(mats[1]), nb,
                                          _ptr(mats[2]), nc, _ptr(mats[3]), nd,
                                          1 if chem_to_phys else 0, PRECISION[precision],
                                          _ptr(out))
        self._check(st, 'scess_transform_tei')
        return out

    def mp2_energy(self, mo_chem, eps, nocc):
        """MP2_RHF_ClosedShell (RHF.cpp:306-345) from chemists' MO integrals (pq|rs)."""
        g = _f64(mo_chem)
        N = g.shape[0]
        e = _f64(eps, (N,))
        out = C.c_double()
        st = self.lib.scess_mp2_energy(self.h, _ptr(g), _ptr(e), N, int(nocc), C.byref(out))
        self._check(st, 'scess_mp2_energy')
        return out.value

    def mp2_energy_ao(self, ao_chem, C_mo, eps, nocc, precision='fp64'):
        """MP2_RHF_ClosedShellAO (RHF.cpp:267-304) from AO integrals (mu nu|kap lam) and
        MO coefficients C (nao x nmo, occupied first)."""
        g = _f64(ao_chem)
        n = g.shape[0]
        cm = _f64(C_mo)
        nmo = cm.shape[1]
        e = _f64(eps, (nmo,))
        out = C.c_double()
        st = self.lib.scess_mp2_energy_ao(self.h, _ptr(g), _ptr(cm), _ptr(e), n, nmo, int(nocc),
                                          PRECISION[precision], C.byref(out))
        self._check(st, 'scess_mp2_energy_ao')
        return out.value

    def ccsd_so(self, mo_chem, eps, nocc, diis=True, triples=False, keep_ints=False) -> CCSD_Wfn:
        """Spin-orbital CCSD (CCSD.cpp:21-106), CCSD_DIIS (CCSD-DIIS.cpp:17-198) or, with
        triples, CCSD_T (CCSD_T.cpp:18-66) from chemists' MO integrals (pq|rs)."""
        g = _f64(mo_chem)
        N = g.shape[0]
        e = _f64(eps, (N,))
        o, v = 2 * int(nocc), 2 * (N - int(nocc))
        t1 = np.zeros((o, v), order='F')
        t2 = np.zeros((o, o, v, v), order='F')
        gs = np.zeros((2 * N,) * 4, order='F') if keep_ints else None
        res = Result()
        st = self.lib.scess_ccsd_so_solve(self.h, _ptr(g), _ptr(e), N, int(nocc), int(bool(diis)),
                                          int(bool(triples)), _ptr(t1), _ptr(t2), _ptr(gs),
                                          C.byref(res))
        self._check(st, 'scess_ccsd_so_solve')
        return CCSD_Wfn(E_CCSD=res.E_CCSD, E_T=res.E_T, t1=t1, t2=t2, mints=gs,
                        converged=bool(res.converged), iterations=res.iterations)

    def ccsd_so_triples(self, g, eps, nocc, t1, t2) -> float:
        """CalculateTriplesCorrection (CCSD_T.cpp:89-229) from <pq||rs> ((2 nmo)^4)."""
        e = _f64(eps)
        N = e.shape[0]
        o, v = 2 * int(nocc), 2 * (N - int(nocc))
        gf = _f64(g, (2 * N,) * 4)
        out = C.c_double()
        st = self.lib.scess_ccsd_so_triples(self.h, _ptr(gf), _ptr(e), N, int(nocc),
                                            _ptr(_f64(t1, (o, v))), _ptr(_f64(t2, (o, o, v, v))),
                                            C.byref(out))
        self._check(st, 'scess_ccsd_so_triples')
        return out.value

    def f12b_coupling(self, eri, f12, f12_repulsion, C, nocc, precision='fp64'):
        """The CCSD-F12b coupling of CCSD_F12b.cpp:83-94: V_klab = <kl|r12^-1 f12|ab>
        - sum_rs <ab|rs><kl|f12|rs>, then RCCSD_F12Coupling(residual = F(C + V),
        energy = F(C)) with F(X) = 3/8 X + 1/8 X^(i<->j).  eri, f12 and f12_repulsion
        are nmo^4 (physicists' notation), C is (o, o, v, v)."""
        e = _f64(eri)
        N = e.shape[0]
        o, v = int(nocc), N - int(nocc)
        f = _f64(f12, (N, N, N, N))
        r = _f64(f12_repulsion, (N, N, N, N))
        c = _f64(C, (o, o, v, v))
        res = np.zeros((o, o, v, v), order='F')
        en = np.zeros((o, o, v, v), order='F')
        st = self.lib.scess_f12b_coupling(self.h, _ptr(e), _ptr(f), _ptr(r), _ptr(c), N, o,
                                          PRECISION[precision], _ptr(res), _ptr(en))
        self._check(st, 'scess_f12b_coupling')
        return RCCSD_F12Coupling(residual=res, energy=en)

    # -- Lambda equations and the one-particle density ---------------------------------------
    def lambda_solve(self, eri, eps, nocc, t1, t2, precision='fp64', **opts):
        eps = _f64(eps)
        N = eps.shape[0]
        o, v = int(nocc), N - int(nocc)
        op = self.default_options()
        op.precision = PRECISION[precision]
        for k, val in opts.items():
            setattr(op, k, val)
        l1 = np.zeros((o, v), order='F')
        l2 = np.zeros((o, o, v, v), order='F')
        res = Result()
        st = self.lib.scess_rccsd_lambda(self.h, _ptr(_f64(eri, (N, N, N, N))), _ptr(eps), N, o,
                                         _ptr(_f64(t1, (o, v))), _ptr(_f64(t2, (o, o, v, v))),
                                         C.byref(op), _ptr(l1), _ptr(l2), C.byref(res))
        self._check(st, 'scess_rccsd_lambda')
        return l1, l2, res

    def rdm1(self, eri, eps, nocc, t1, t2, l1, l2, precision='fp64'):
        eps = _f64(eps)
        N = eps.shape[0]
        o, v = int(nocc), N - int(nocc)
        dm = np.zeros((N, N), order='F')
        st = self.lib.scess_rccsd_rdm1(self.h, _ptr(_f64(eri, (N, N, N, N))), _ptr(eps), N, o,
                                       _ptr(_f64(t1, (o, v))), _ptr(_f64(t2, (o, o, v, v))),
                                       _ptr(_f64(l1, (o, v))), _ptr(_f64(l2, (o, o, v, v))),
                                       PRECISION[precision], _ptr(dm))
        self._check(st, 'scess_rccsd_rdm1')
        return dm

    # -- generic contraction ------------------------------------------------------------------
    def einsum(self, spec: str, A, B, C_init=None, alpha=1.0, beta=0.0, precision='fp64',
               out_shape=None):
        Af, Bf = _f64(A), _f64(B)
        if C_init is None:
            Cf = np.zeros(out_shape, order='F')
        else:
            Cf = _f64(C_init).copy(order='F')
        ext = lambda a: (C.c_int64 * a.ndim)(*a.shape)  # noqa: E731
        st = self.lib.scess_einsum(self.h, spec.encode(), alpha, _ptr(Af), Af.ndim, ext(Af),
                                   _ptr(Bf), Bf.ndim, ext(Bf), beta, _ptr(Cf), Cf.ndim, ext(Cf),
                                   PRECISION[precision])
        self._check(st, 'scess_einsum')
        return Cf


def einsum_static(spec: str, A_ptr: int, a_ext, B_ptr: int, b_ext, C_ptr: int, c_ext,
                  alpha: float = 1.0, beta: float = 0.0, stream: int = 0) -> int:
    """scess_einsum_static on device buffers given by address (column-major
    extents as for Context.einsum), queued on `stream` (a cudaStream_t as int).
    For callers that cannot allocate device memory: the library allocates
    nothing here; its scratch is a fixed 16 MiB array.  Returns the status."""
    lib = load_library()
    ext = lambda e: (C.c_int64 * len(e))(*[int(x) for x in e])  # noqa: E731
    return lib.scess_einsum_static(spec.encode(), float(alpha), C.c_void_p(A_ptr), len(a_ext),
                                   ext(a_ext), C.c_void_p(B_ptr), len(b_ext), ext(b_ext),
                                   float(beta), C.c_void_p(C_ptr), len(c_ext), ext(c_ext),
                                   C.c_void_p(stream))


class State:
    """scess_rccsd_state: integrals, amplitudes and DIIS resident in GPU memory."""

    def __init__(self, ctx: Context, eri, eps, nocc, B=None, precision='fp64', f12=None, **opts):
        self.ctx = ctx
        self.lib = ctx.lib
        self.eps = _f64(eps)
        N = self.eps.shape[0]
        self.o, self.v = int(nocc), N - int(nocc)
        o, v = self.o, self.v
        self.op = ctx.default_options()
        self.op.precision = PRECISION[precision]
        for k, val in opts.items():
            setattr(self.op, k, val)
        self.hist = np.zeros(3 * max(self.op.max_iterations, 1))
        self.op.history = _ptr(self.hist)
        fr = fe = None
        if f12 is not None:
            fr = _f64(f12.residual, (o, o, v, v))
            fe = _f64(f12.energy, (o, o, v, v))
        h = C.c_void_p()
        if B is not None:
            Bf = B if (isinstance(B, np.ndarray) and B.flags.f_contiguous) else _f64(B)
            st = self.lib.scess_rccsd_state_create_df(ctx.h, _ptr(Bf), Bf.shape[0], _ptr(self.eps),
                                                      N, o, _ptr(fr), _ptr(fe), C.byref(self.op),
                                                      C.byref(h))
        else:
            ef = eri if (isinstance(eri, np.ndarray) and eri.flags.f_contiguous
                         and eri.dtype == np.float64) else _f64(eri, (N, N, N, N))
            st = self.lib.scess_rccsd_state_create(ctx.h, _ptr(ef), _ptr(self.eps), N, o, _ptr(fr),
                                                   _ptr(fe), C.byref(self.op), C.byref(h))
        ctx._check(st, 'scess_rccsd_state_create')
        self.h = h

    def iterate(self, n: int = 1):
        res = Result()
        ms = C.c_double(0.0)
        self.ctx._check(self.lib.scess_rccsd_state_iterate(self.h, n, C.byref(res), C.byref(ms)),
                        'scess_rccsd_state_iterate')
        return res, ms.value

    def triples(self, precision='fp64'):
        et = C.c_double(0.0)
        ms = C.c_double(0.0)
        self.ctx._check(self.lib.scess_rccsd_state_triples(self.h, PRECISION[precision],
                                                           C.byref(et), C.byref(ms)),
                        'scess_rccsd_state_triples')
        return et.value, ms.value

    def amplitudes(self):
        t1 = np.zeros((self.o, self.v), order='F')
        t2 = np.zeros((self.o, self.o, self.v, self.v), order='F')
        self.ctx._check(self.lib.scess_rccsd_state_amplitudes(self.h, _ptr(t1), _ptr(t2)),
                        'scess_rccsd_state_amplitudes')
        return t1, t2

    def set_amplitudes(self, t1, t2):
        t1f = _f64(t1, (self.o, self.v))
        t2f = _f64(t2, (self.o, self.o, self.v, self.v))
        self.ctx._check(self.lib.scess_rccsd_state_set_amplitudes(self.h, _ptr(t1f), _ptr(t2f)),
                        'scess_rccsd_state_set_amplitudes')

    def close(self):
        if getattr(self, 'h', None):
            self.lib.scess_rccsd_state_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


def SolveRCCSD_DIIS(eri, orbitalEnergies, nOcc, f12: RCCSD_F12Coupling | None = None,
                    thread=None, console=None, precision: str = 'fp64') -> RCCSD_Wfn:
    """CC::SolveRCCSD_DIIS (CC.h:136-141) on the GPU."""
    return default_context().solve(eri, orbitalEnergies, nOcc, f12=f12, thread=thread,
                                   console=console, precision=precision)


def RCCSD_TriplesCorrection(eri, orbitalEnergies, nOcc, t1, t2, thread=None,
                            precision: str = 'fp64') -> float:
    """CC::RCCSD_TriplesCorrection (CC.h:154-158) on the GPU."""
    return default_context().triples(eri, orbitalEnergies, nOcc, t1, t2, precision=precision,
                                     thread=thread)


def CCSD(mo_chem, orbitalEnergies, nOcc) -> CCSD_Wfn:
    """CC::CCSD (CC.h:53-62) on the GPU, from the MO integrals TransformTEI gives."""
    return default_context().ccsd_so(mo_chem, orbitalEnergies, nOcc, diis=False)


def CCSD_DIIS(mo_chem, orbitalEnergies, nOcc) -> CCSD_Wfn:
    """CC::CCSD_DIIS (CC.h:64-72) on the GPU; ``mints`` holds <pq||rs>."""
    return default_context().ccsd_so(mo_chem, orbitalEnergies, nOcc, diis=True, keep_ints=True)


def CCSD_T(mo_chem, orbitalEnergies, nOcc) -> CCSD_Wfn:
    """CC::CCSD_T (CC.h:74-76) on the GPU."""
    return default_context().ccsd_so(mo_chem, orbitalEnergies, nOcc, diis=True, triples=True,
                                     keep_ints=True)


def CalculateTriplesCorrection(ccsd: CCSD_Wfn, F, eri, nOcc, nVirt) -> float:
    """CC::CalculateTriplesCorrection (CC.h:78-81): F the spin-orbital Fock matrix
    (diagonal), eri = <pq||rs>, nOcc / nVirt spin-orbital counts."""
    eps = np.diag(np.asarray(F))[::2]
    return default_context().ccsd_so_triples(eri, eps, int(nOcc) // 2, ccsd.t1, ccsd.t2)
