"""Benchmark: one closed-shell CCSD iteration + (T), mixed precision vs FP64, on one GB300.

Metric (lower is better): seconds for one CCSD iteration (residual, Jacobi
update, DIIS, energy) plus the full (T) correction, mixed-precision form, at
o=20, v=180 on seeded synthetic DF integrals (the convergent variant of the
generator; see scess_gb300/synthetic.py), inputs resident in HBM.  The timed
state never leaves the mixed phase (its switch to FP64 refinement is
disabled), so every timed step is the same work: one mixed iteration and one
mixed (T); the loop checks that the mixed iteration count advanced by one.

Beside it:

* ``fp64``: the FP64 GPU path on the same workload (the drop-in form), one
  iteration and one (T), and the energy differences mixed - FP64;
* ``converged``: the drop-in calls themselves, SolveRCCSD_DIIS to convergence
  (scess_rccsd_solve) followed by RCCSD_TriplesCorrection
  (scess_rccsd_triples), once in the mixed form (tensor-core iterations and
  the refinement that ends in FP64 iterations) and once in FP64, host buffers
  in and out: seconds, iteration counts and the differences of E_CCSD, E_(T)
  and their sum;
* ``triples_o24_v240``: (T) alone at o=24, v=240 from DF factors on fixed
  seeded amplitudes, mixed (median of 3 calls) and FP64 once, with the
  difference of the two E_(T) in Eh and relative;
* ``e2e``: the timed step through the public C ABI from pinned host buffers
  (state create = nmo^4 eri upload + block build + MP2 guess, one iteration,
  (T), amplitudes back), median over the e2e steps;
* ``roofline`` of the dominant kernel (the grouped (T) tcgen05 GEMM) from the
  library's per-launch CUDA-event timers over the timed steps;
* ``cpu_baseline``: the FP64 oracle on this host (one full NumPy CCSD
  iteration + (T) of the C restatement, extrapolated from its costliest
  leading-virtual slices).

``--impl reference`` times only that CPU oracle on the same workload (each
step the same bounded sample) and prints the same JSON line with
``"impl": "reference"``.  Run ``python bench.py`` for the defaults (N=1).
Under torchrun every rank runs an independent replica (one solve does not
shard across GPUs: replicas only) and rank 0 prints.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = 'CCSD iter + (T) seconds, mixed vs FP64 GPU at <=1uEh; % tensor-pipe peak'
UNIT = 's'
CPU_TSLICES = 2  # costliest leading virtuals of the (T) sample (both CPU legs)
CPU_SAMPLE = ('one full FP64 CCSD iteration of the NumPy oracle (MP2 guess, BLAS einsums) + '
              '(T) of the C+OpenMP restatement of RCCSD_TriplesCorrection: its repack timed '
              f'once plus the {CPU_TSLICES} costliest leading virtuals scaled by the triple count '
              '(a full (T) at o=10, v=90 lands within 16% of this estimate); the eri is '
              'column-major, as the C restatement reads it, so no step copies it')


# DRAM bytes (read + write) of one grouped (T) GEMM launch at o=20, nb=12,
# measured with ncu: the three W buffers (166 MB) are written once, 112 MB of
# them reach DRAM, operands are read mostly from L2.
TRIPLES_LAUNCH_TRAFFIC = 36.6e6
TRIPLES_TRAFFIC_SOURCE = ('ncu dram__bytes_read.sum + dram__bytes_write.sum (30.7 MB + 5.9 MB) of one '
                          'grouped (T) launch of `bench.py --triples-only --o 20 --v 180`, the same '
                          'launches as this workload (nb=12, 864 work units of 256 x 256 on cluster '
                          'pairs), application replay with --cache-control none: the L2 as the '
                          'program leaves it, W (55 MB) resident between the GEMM and the energy '
                          'kernel')


def peaks():
    p = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get('hbm_gbs', 6800.0), d.get('bf16_tflops', 1900.0), 'measured'
    return 6800.0, 1900.0, 'fallback'


class Clocks:
    """nvidia-smi sampler running during the timed region."""
    Q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
         'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
         'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, dev):
        self.dev = dev
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(['nvidia-smi', '-i', str(self.dev), f'--query-gpu={self.Q}',
                                          '--format=csv,noheader,nounits', '-lms', '200'],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['nvidia-smi unavailable']}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for ln in self.lines:
            f = [x.strip() for x in ln.split(',')]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, val in zip(names, f[5:9]):
                if val.lower() == 'active':
                    reasons.add(n)
        return {'sm_mhz': float(np.median(sm)) if sm else None, 'sm_max_mhz': mx,
                'reasons': sorted(reasons), 'samples': len(sm)}


def build_eri_pinned(w, torch):
    """eri(p,q,r,s) = (pr|qs), column-major, in pinned host memory (built on the GPU)."""
    N = w.nmo
    B = torch.from_numpy(w.B).cuda()
    # T[s,r,q,p] (row-major) == eri(p,q,r,s) at p + N q + N^2 r + N^3 s
    T = torch.einsum('Qpr,Qqs->srqp', B, B).contiguous()
    host = torch.empty(N ** 4, dtype=torch.float64, pin_memory=True)
    host.copy_(T.reshape(-1))
    del T, B
    torch.cuda.empty_cache()
    return host, host.numpy().reshape((N, N, N, N), order='F')


def fp64_peak_tflops(torch):
    n = 8192
    a = torch.randn(n, n, dtype=torch.float64, device='cuda')
    b = torch.randn(n, n, dtype=torch.float64, device='cuda')
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e9
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    del a, b
    return 2.0 * n ** 3 / best / 1e12


def build_eri_host_colmajor(w):
    """eri(p,q,r,s) = (pr|qs) as a column-major N^4 array built on the host.

    Formed one s slice at a time (an N^2 x naux by naux x N product each), so
    that neither a full chemists' copy nor a layout conversion is needed: the
    slice s of the column-major array is X[r,q,p] = (rp|sq) = chem[(r,p),(s,q)].
    """
    N = w.nmo
    Bm = np.ascontiguousarray(w.B.reshape(w.naux, N * N))
    flat = np.empty(N ** 4)
    X = flat.reshape(N, N, N, N)  # C-order [s, r, q, p] == column-major (p, q, r, s)
    for s in range(N):
        blk = Bm.T @ Bm[:, s * N:(s + 1) * N]         # [(r, p), q]
        X[s] = blk.reshape(N, N, N).transpose(0, 2, 1)
    return flat.reshape((N, N, N, N), order='F')


def cpu_oracle_step(eri, eps, o, ints=None, tslices=CPU_TSLICES):
    """One FP64 CPU CCSD iteration + (T) on a bounded sample, in seconds.

    CCSD: one full UpdateAmplitudes + energy of the NumPy oracle (BLAS-backed
    einsums) from the MP2 guess.  (T): the C + OpenMP restatement of
    RCCSD_TriplesCorrection (oracle/rccsd_t_ref.c) over the `tslices`
    costliest leading virtuals a = v-1, v-2, ...; every triple costs the same,
    so the full (T) time is the sample time x (all triples / sampled triples).
    """
    import oracle
    from oracle import build_ref
    v = eri.shape[0] - o
    if ints is None:
        ints = oracle.make_integral_blocks(eri, o)
    eia, eijab = oracle.rccsd.denominators(eps, o)
    t1 = np.zeros((o, v))
    t2 = ints.oovv_phys / eijab
    t0 = time.perf_counter()
    n1, n2 = oracle.update_amplitudes(ints, eia, eijab, None, t1, t2)
    E = oracle.correlation_energy(ints, n1, n2)
    t_ccsd = time.perf_counter() - t0
    a0 = max(0, v - tslices)
    t0 = time.perf_counter()
    build_ref.triples(eri, eps, o, n1, n2, a_begin=v, a_end=v)     # repack only
    t_repack = time.perf_counter() - t0
    t0 = time.perf_counter()
    build_ref.triples(eri, eps, o, n1, n2, a_begin=a0, a_end=v)
    t_slice = time.perf_counter() - t0
    ntrip = lambda a: (a + 1) * (a + 2) // 2  # noqa: E731
    sampled = sum(ntrip(a) for a in range(a0, v))
    total = v * (v + 1) * (v + 2) // 6
    t_T = t_repack + max(t_slice - t_repack, 0.0) * total / sampled
    return t_ccsd + t_T, {'ccsd_iter_s': t_ccsd, 'triples_s_extrapolated': t_T,
                          'triples_repack_s': t_repack, 'triples_sample_s': t_slice,
                          'triples_sampled': sampled, 'triples_total': total, 'E_iter': E}


def transform_only(args, wl, config, ctx_factory, lib, torch):
    """AO->MO transform (scess_transform_tei) of chemists' integrals
    (pq|rs) = sum_Q B(Q,p,q) B(Q,r,s) from the seeded DF factors (nao = nmo =
    o + v) with a seeded orthogonal C, to physicists' order; host buffers in and
    out.  Mixed timed over --steps calls after --warmup, FP64 once."""
    N = wl.nmo
    B = torch.from_numpy(wl.B).cuda()
    host = torch.empty(N ** 4, dtype=torch.float64, pin_memory=True)
    host.copy_(torch.einsum('Qpq,Qrs->srqp', B, B).contiguous().reshape(-1))  # column-major (pq|rs)
    del B
    torch.cuda.empty_cache()
    tei = host.numpy().reshape((N, N, N, N), order='F')
    g = torch.Generator().manual_seed(args.seed)
    Cm = np.asfortranarray(torch.linalg.qr(torch.randn(N, N, dtype=torch.float64, generator=g))[0].numpy())
    ctx = ctx_factory()
    flops = 8.0 * N ** 5
    for _ in range(args.warmup):
        ctx.transform_tei(tei, Cm, chem_to_phys=True, precision='mixed')
    ctx.profile(True)
    n0 = lib.scess_launch_count()
    walls = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        out_m = ctx.transform_tei(tei, Cm, chem_to_phys=True, precision='mixed')
        walls.append(time.perf_counter() - t0)
    launches = int(lib.scess_launch_count() - n0)
    prof = ctx.profile_report()
    ctx.profile(False)
    kern_ms = sum(v['ms'] for k, v in prof.items() if not k.startswith('host:')) / args.steps
    fp64 = None
    if not args.no_fp64:
        t0 = time.perf_counter()
        out_f = ctx.transform_tei(tei, Cm, chem_to_phys=True, precision='fp64')
        tf = time.perf_counter() - t0
        fp64 = {'seconds': tf, 'tflops': flops / tf / 1e12,
                'max_rel_diff_mixed': float(np.max(np.abs(out_m - out_f)) / np.max(np.abs(out_f)))}
    t = float(np.mean(walls))
    print(json.dumps({
        'metric': 'AO->MO transform seconds (TransformTEI), mixed vs FP64 GPU', 'value': t,
        'unit': 's', 'n_gpus': 1, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': t * 1e3, 'higher_is_better': False, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'f16x2-split (FP32 acc) + f64', 'data': 'synthetic',
        'config': dict(config, workload=f'AO->MO transform, nao = nmo = {N}, chemists AO integrals '
                                        'from the seeded DF factors, seeded orthogonal C'),
        'algorithmic_tflop': flops / 1e12, 'kernel_ms_per_call': kern_ms,
        'kernel_tflops': flops / (kern_ms / 1e3) / 1e12 if kern_ms > 0 else None,
        'e2e': {'value': t, 'unit': 's', 'h2d_bytes_per_step': int(8 * (N ** 4 + 4 * N * N)),
                'd2h_bytes_per_step': int(8 * N ** 4)},
        'fp64': fp64, 'kernel_timers': prof, 'gpu_launches': launches}))


def measure_triples_df(ctx, lib, torch, o, v, seed, sigma, steps, warmup, with_fp64,
                       bf16_peak, peak_kind):
    """(T) alone through scess_rccsd_triples_df on the seeded denominator-scaled
    amplitudes of the (T) workload at (o, v): each call uploads B, t1 and t2 from
    pinned host buffers, contracts the integral slices (T) reads from B (the
    nmo^4 eri is never formed), packs and runs (T).  Mixed is timed over `steps`
    calls after `warmup` (host clock around the call, plus the library's kernel
    timers), FP64 once on the same inputs."""
    from scess_gb300.synthetic import make_workload
    import oracle
    wl = make_workload(o, v, seed=seed, with_amplitudes=True, sigma=sigma)
    # the ABI's column-major layout in pinned host memory, prepared once (a C
    # caller passes such buffers directly; the binding then copies nothing)
    keep = []

    def pinned_f(a):
        h = torch.empty(a.size, dtype=torch.float64, pin_memory=True)
        keep.append(h)
        hn = h.numpy()
        hn[:] = np.asarray(a, dtype=np.float64).ravel(order='F')
        return hn.reshape(a.shape, order='F')

    Bh, t1h, t2h = pinned_f(wl.B), pinned_f(wl.t1), pinned_f(wl.t2)
    for _ in range(warmup):
        ctx.triples(eps=wl.eps, nocc=o, t1=t1h, t2=t2h, B=Bh, precision='mixed')
    clk = Clocks(torch.cuda.current_device())
    clk.start()
    n0 = lib.scess_launch_count()
    walls, ets = [], []
    for _ in range(steps):  # (no per-kernel timers: their events would serialise the launches)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ets.append(ctx.triples(eps=wl.eps, nocc=o, t1=t1h, t2=t2h, B=Bh, precision='mixed'))
        walls.append(time.perf_counter() - t0)
    launches = int(lib.scess_launch_count() - n0)
    clocks = clk.stop()
    # the same calls again with the per-kernel CUDA-event timers (roofline, shares)
    ctx.profile(True)
    for _ in range(steps):
        ctx.triples(eps=wl.eps, nocc=o, t1=t1h, t2=t2h, B=Bh, precision='mixed')
    prof = ctx.profile_report()
    ctx.profile(False)
    t_mixed = float(np.median(walls))
    tc = prof.get('tc_gemm[triples]', {'launches': 0, 'ms': 0.0, 'flops': 0.0})
    per_launch_alg = oracle.triples_flops(o, v) * steps / max(tc['launches'], 1)
    avg_ms = tc['ms'] / max(tc['launches'], 1)
    achieved = per_launch_alg / (avg_ms / 1e3) / 1e12 if avg_ms > 0 else 0.0
    fp64 = None
    if with_fp64:
        t0 = time.perf_counter()
        etf = ctx.triples(eps=wl.eps, nocc=o, t1=t1h, t2=t2h, B=Bh, precision='fp64')
        tf = time.perf_counter() - t0
        fp64 = {'triples_s': tf, 'E_T_fp64': etf, 'dE_T_mixed_vs_fp64_Eh': abs(ets[-1] - etf),
                'rel_dE_T': abs(ets[-1] - etf) / max(abs(etf), 1e-300),
                'speedup_mixed_vs_fp64': tf / t_mixed,
                'fp64_tflops': oracle.triples_flops(o, v) / tf / 1e12}
    peak_alg = bf16_peak / 3.0
    N = o + v
    return {
        'workload': f'(T) alone, o={o} v={v}, seeded DF integrals (sigma_B={sigma:.5f}) and '
                    'seeded denominator-scaled t1/t2 (not converged amplitudes: E_T is large), '
                    'through scess_rccsd_triples_df',
        'seconds_mixed': t_mixed, 'statistic': f'median of {steps} calls',
        'E_T_mixed': ets[-1], 'fp64': fp64,
        'h2d_bytes_per_call': int(8 * (wl.naux * N * N + N + o * v + o * o * v * v)),
        'roofline': {'kernel': 'tc_gemm_kernel, grouped (T) launch', 'bound': 'tensor',
                     'achieved': achieved, 'peak': peak_alg, 'unit': 'TFLOP/s',
                     'frac': achieved / peak_alg, 'avg_launch_ms': avg_ms,
                     'launches': tc['launches'], 'traffic': None,
                     'peak_basis': f'bf16 dense {bf16_peak} TFLOP/s ({peak_kind}) / 3'},
        'kernel_timers': prof, 'gpu_launches': launches, 'clocks': clocks}


def triples_only(args, wl, config, ctx_factory, lib, bf16_peak, peak_kind, torch):
    """(T) alone at (--o, --v): measure_triples_df as its own JSON line."""
    o, v = args.o, args.v
    r = measure_triples_df(ctx_factory(), lib, torch, o, v, args.seed, wl.sigma, args.steps,
                           args.warmup, not args.no_fp64, bf16_peak, peak_kind)
    N = o + v
    t = r['seconds_mixed']
    print(json.dumps({
        'metric': '(T) seconds, mixed vs FP64 GPU (fixed amplitudes)', 'value': t,
        'unit': 's', 'n_gpus': 1, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': t * 1e3, 'higher_is_better': False, 'scaling': 'weak',
        'vs_baseline': None, 'dtype': 'f16x2-split (FP32 acc) + f64', 'data': 'synthetic',
        'config': dict(config, workload=r['workload'],
                       l2='inputs larger than L2 (packed (ia|bf) and W buffers)'),
        'E_T_mixed': r['E_T_mixed'], 'fp64': r['fp64'],
        'e2e': {'value': t, 'unit': 's', 'h2d_bytes_per_step': r['h2d_bytes_per_call'],
                'd2h_bytes_per_step': 8},
        'roofline': r['roofline'], 'kernel_timers': r['kernel_timers'],
        'gpu_launches': r['gpu_launches'], 'clocks': r['clocks']}))


def max_over_ranks(value, world, device='cuda'):
    """The largest of the ranks' values (every rank gets it); world == 1: value."""
    if world <= 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def rank_info():
    return (int(os.environ.get('RANK', 0)), int(os.environ.get('WORLD_SIZE', 1)),
            int(os.environ.get('LOCAL_RANK', 0)))


def reference_arm(args, wl, config):
    """The reference's CPU implementation of the path (the FP64 oracle: NumPy
    CCSD iteration + C/OpenMP (T) restatement) on this host's cores, each step
    the same bounded sample as the cpu_baseline leg."""
    o = args.o
    eri = build_eri_host_colmajor(wl)
    import oracle
    ints = oracle.make_integral_blocks(eri, o)
    warm = min(args.warmup, 1)
    for _ in range(warm):
        cpu_oracle_step(eri, wl.eps, o, ints=ints)
    times = []
    det = None
    for _ in range(args.steps):
        t, det = cpu_oracle_step(eri, wl.eps, o, ints=ints)
        times.append(t)
    val = float(np.median(times))
    print(json.dumps({
        'impl': 'reference', 'metric': METRIC, 'value': val, 'unit': UNIT, 'n_gpus': args.gpus,
        'steps': args.steps, 'warmup': warm, 'ms_per_step': val * 1e3,
        'higher_is_better': False, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
        'data': 'synthetic', 'config': config,
        'cpu_baseline': {'value': val, 'unit': UNIT, 'cores': os.cpu_count(), 'kind': 'port',
                         'sample': CPU_SAMPLE, 'details': det,
                         'step_times_s': times, 'statistic': 'median over the steps'},
        'e2e': {'value': val, 'unit': UNIT, 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0},
    }))


def converged_solves(ctx, eri_h, wl, o, torch):
    """The drop-in calls to convergence, mixed then FP64: scess_rccsd_solve
    (SolveRCCSD_DIIS) followed by scess_rccsd_triples (RCCSD_TriplesCorrection),
    host eri in, amplitudes and energies out, timed on the host."""
    out = {}
    amps = {}
    for prec in ('mixed', 'fp64'):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        w = ctx.solve(eri_h, wl.eps, o, precision=prec)
        t1 = time.perf_counter()
        et = ctx.triples(eri_h, wl.eps, o, w.t1, w.t2, precision=prec) if w.converged else None
        t2 = time.perf_counter()
        amps[prec] = (w.t1, w.t2)
        out[prec] = {'seconds': t2 - t0, 'solve_s': t1 - t0, 'triples_s': t2 - t1,
                     'converged': bool(w.converged), 'iterations': int(w.iterations),
                     'mixed_iterations': int(w.mixed_iterations),
                     'fp64_iterations': int(w.iterations - w.mixed_iterations),
                     'E_CCSD': w.E_CCSD, 'E_T': et}
    m, f = out['mixed'], out['fp64']
    ok = m['converged'] and f['converged']
    res = {'call': 'scess_rccsd_solve (eri from pinned host, MP2 guess, DIIS(8), dE < 1e-10 and '
                   'rms < 1e-8) + scess_rccsd_triples (eri, t1, t2 from host), per precision',
           'mixed': m, 'fp64': f,
           'speedup_mixed_vs_fp64': f['seconds'] / m['seconds'] if ok else None}
    if ok:
        res['dE_CCSD'] = abs(m['E_CCSD'] - f['E_CCSD'])
        res['dE_T'] = abs(m['E_T'] - f['E_T'])
        res['dE_corr'] = abs(m['E_CCSD'] + m['E_T'] - f['E_CCSD'] - f['E_T'])
        res['max_abs_dt2'] = float(np.max(np.abs(amps['mixed'][1] - amps['fp64'][1])))
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=3)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--o', type=int, default=20)
    ap.add_argument('--v', type=int, default=180)
    ap.add_argument('--seed', type=int, default=0)
    ap.add_argument('--fp64-steps', type=int, default=1)
    ap.add_argument('--e2e-steps', type=int, default=5)
    ap.add_argument('--no-cpu', action='store_true')
    ap.add_argument('--no-fp64', action='store_true')
    ap.add_argument('--no-converged', action='store_true',
                    help='skip the converged mixed and FP64 solves + (T)')
    ap.add_argument('--no-large-triples', action='store_true',
                    help='skip the (T) workload at o=24, v=240 (mixed, and FP64 once)')
    ap.add_argument('--transform', action='store_true',
                    help='AO->MO transform of nmo^4 integrals (TransformTEI), mixed vs FP64')
    ap.add_argument('--triples-only', action='store_true',
                    help='(T) alone on fixed seeded amplitudes (e.g. --o 24 --v 240), mixed vs FP64')
    args = ap.parse_args()
    rank, world, local = rank_info()
    o, v = args.o, args.v

    from scess_gb300.synthetic import convergent_sigma, make_workload
    import oracle
    sigma = convergent_sigma(o, v)
    wl = make_workload(o, v, seed=args.seed, sigma=sigma)
    config = {'workload': f'closed-shell CCSD iteration + (T), o={o} v={v} (nmo={o + v}, '
                          f'naux={wl.naux}), seeded synthetic DF integrals (sigma_B={sigma:.5f})',
              'o': o, 'v': v, 'naux': wl.naux, 'seed': args.seed,
              'ccsd_flops_per_iter': oracle.ccsd_flops(o, v),
              'triples_flops': oracle.triples_flops(o, v),
              'l2': 'inputs larger than L2 (nmo^4 eri 12.8 GB, packed vvvv 4.2 GB)',
              'parallelism': 'replicas' if world > 1 else 'single GPU'}

    if args.impl == 'reference':
        if rank == 0:
            reference_arm(args, wl, config)
        return

    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('nccl')
    from scess_gb300 import build as sbuild
    sbuild.build()
    import scess_gb300 as s
    lib = s.load_library()
    hbm, bf16_peak, peak_kind = peaks()

    if args.transform:
        return transform_only(args, wl, config, ctx_factory=lambda: s.Context(local), lib=lib,
                              torch=torch)
    if args.triples_only:
        return triples_only(args, wl, config, ctx_factory=lambda: s.Context(local), lib=lib,
                            bf16_peak=bf16_peak, peak_kind=peak_kind, torch=torch)

    host_t, eri_h = build_eri_pinned(wl, torch)
    N = wl.nmo
    ctx = s.Context(local)

    # ---- mixed form, inputs resident ----------------------------------------------------
    # mixed_energy_switch = 0: the state never moves to its FP64 refinement phase,
    # so every step below is one mixed iteration and one mixed (T)
    st = ctx.state(eri_h, wl.eps, o, precision='mixed', max_iterations=1000,
                   mixed_energy_switch=0.0)
    for _ in range(args.warmup):
        st.iterate(1)
        st.triples('mixed')
    torch.cuda.synchronize()
    clk = Clocks(local)
    clk.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    n0 = lib.scess_launch_count()
    it_ms, t_ms, ets = [], [], []
    mixed_before = args.warmup

    def mixed_step():
        nonlocal mixed_before
        r, ms1 = st.iterate(1)
        et, ms2 = st.triples('mixed')
        if r.mixed_iterations != mixed_before + 1 or r.iterations != r.mixed_iterations:
            raise RuntimeError(f'timed step was not one mixed iteration: {r.mixed_iterations} '
                               f'mixed, {r.iterations} total after {mixed_before}')
        mixed_before = r.mixed_iterations
        return ms1, ms2, et

    # the timed steps run without the per-kernel timers (their events between
    # launches would serialise the (T) launches that overlap their neighbours)
    wall0 = time.perf_counter()
    for _ in range(args.steps):
        ms1, ms2, et = mixed_step()
        it_ms.append(ms1)
        t_ms.append(ms2)
        ets.append(et)
    torch.cuda.synchronize()
    wall = (time.perf_counter() - wall0) / args.steps
    launches = int(lib.scess_launch_count() - n0)
    clocks = clk.stop()
    # the same steps again with the per-kernel CUDA-event timers: the roofline,
    # the kernel shares and the breakdown come from these
    ctx.profile(True)
    for _ in range(args.steps):
        mixed_step()
    torch.cuda.synchronize()
    prof = ctx.profile_report()
    ctx.profile(False)
    step_s = (float(np.mean(it_ms)) + float(np.mean(t_ms))) / 1e3
    step_s = max_over_ranks(step_s, world)
    hist_mixed = st.hist.reshape(-1, 3)
    n_iter_mixed = args.warmup + args.steps

    # ---- roofline of the dominant kernel ----------------------------------------------------
    # The grouped (T) GEMM (one launch per block triple).  Algorithmic FLOPs are the
    # reference's (T) count (unique triples a >= b >= c, 12 o^3 (v + o) each) spread
    # over the launches of one (T); the launches also compute the repeated triples of
    # the diagonal block triples, which the timer's own count includes.
    tc = prof.get('tc_gemm[triples]', {'launches': 0, 'ms': 0.0, 'flops': 0.0})
    top = max(((k, v) for k, v in prof.items() if not k.startswith('phase:')),
              key=lambda kv: kv[1]['ms'], default=(None, None))[0]
    n_t = max(args.steps, 1)
    per_launch_alg = oracle.triples_flops(o, v) * n_t / max(tc['launches'], 1)
    avg_ms = tc['ms'] / max(tc['launches'], 1)
    achieved = per_launch_alg / (avg_ms / 1e3) / 1e12 if avg_ms > 0 else 0.0
    issued = tc['flops'] / (tc['ms'] / 1e3) / 1e12 if tc['ms'] > 0 else 0.0
    peak_alg = bf16_peak / 3.0
    roofline = {'kernel': 'tc_gemm_kernel, grouped (T) launch (tcgen05 split hi/lo, FP32 accumulate)',
                'bound': 'tensor',
                'achieved': achieved, 'peak': peak_alg, 'unit': 'TFLOP/s', 'frac': achieved / peak_alg,
                'peak_basis': f'bf16 dense {bf16_peak} TFLOP/s ({peak_kind}) / 3 products per '
                              'algorithmic FLOP; achieved = algorithmic (T) FLOPs per launch / '
                              'CUDA-event launch time',
                'issued_tflops': issued,
                'tensor_pipe_frac': 3.0 * issued / bf16_peak,
                'launches': tc['launches'], 'avg_launch_ms': avg_ms,
                'algorithmic_flops_per_launch': per_launch_alg,
                'traffic': TRIPLES_LAUNCH_TRAFFIC if (o, v) == (20, 180) else None,
                'traffic_source': TRIPLES_TRAFFIC_SOURCE,
                'top_kernel_by_time': top}
    # "phase:" timers enclose kernel timers: shown, but not part of the shares
    kern = {k: v for k, v in prof.items() if not k.startswith('phase:')}
    share = {k: round(v['ms'] / max(sum(x['ms'] for x in kern.values()), 1e-9), 4) for k, v in kern.items()}

    # ---- FP64 form on the same workload -------------------------------------------------------
    fp64 = None
    if not args.no_fp64:
        sf = ctx.state(eri_h, wl.eps, o, precision='fp64', max_iterations=1000)
        for _ in range(args.fp64_steps):
            sf.iterate(1)
        rf, fms1 = sf.iterate(1)
        etf, fms2 = sf.triples('fp64')
        etm_same, _ = sf.triples('mixed')
        hist_f = sf.hist.reshape(-1, 3)
        nf = args.fp64_steps + 1
        dE_iter = float(np.max(np.abs(hist_mixed[:nf, 0] - hist_f[:nf, 0])))
        fp64 = {'ccsd_iter_s': fms1 / 1e3, 'triples_s': fms2 / 1e3,
                'step_s': (fms1 + fms2) / 1e3,
                'speedup_mixed_vs_fp64': (fms1 + fms2) / 1e3 / step_s,
                'dE_ccsd_iter_mixed_vs_fp64_max': dE_iter,
                'dE_T_mixed_vs_fp64_same_amplitudes': abs(etm_same - etf),
                'E_T_fp64': etf, 'fp64_peak_tflops_cublas_dgemm': fp64_peak_tflops(torch),
                'fp64_ccsd_tflops': oracle.ccsd_flops(o, v) / (fms1 / 1e3) / 1e12,
                'fp64_triples_tflops': oracle.triples_flops(o, v) / (fms2 / 1e3) / 1e12}
        sf.close()
        del sf
    st.close()
    del st

    # ---- the drop-in calls to convergence, mixed vs FP64 --------------------------------------
    converged = None if args.no_converged else converged_solves(ctx, eri_h, wl, o, torch)

    # ---- (T) alone on the largest workload, o=24 v=240 (DF integrals, fixed amplitudes) ---------
    large_t = None
    if not args.no_large_triples and world == 1:
        from scess_gb300.synthetic import convergent_sigma as csig
        large_t = measure_triples_df(ctx, lib, torch, 24, 240, args.seed, csig(24, 240), 3, 1,
                                     not args.no_fp64, bf16_peak, peak_kind)
        large_t.pop('kernel_timers')

    # ---- e2e through the public API from pinned host buffers ----------------------------------
    # host->device bandwidth of the pinned input right before the e2e steps (torch copy)
    h2d_probe = None
    if args.e2e_steps > 0:
        tmp = torch.empty(host_t.numel(), dtype=torch.float64, device='cuda')
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        tmp.copy_(host_t, non_blocking=True)
        torch.cuda.synchronize()
        h2d_probe = host_t.numel() * 8 / (time.perf_counter() - t0) / 1e9
        del tmp
        torch.cuda.empty_cache()
    e2e_times, e2e_phases = [], []
    for _ in range(args.e2e_steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        se = ctx.state(eri_h, wl.eps, o, precision='mixed', max_iterations=1000)
        t1 = time.perf_counter()
        se.iterate(1)
        t2 = time.perf_counter()
        se.triples('mixed')
        t3 = time.perf_counter()
        se.amplitudes()
        se.close()
        torch.cuda.synchronize()
        t4 = time.perf_counter()
        e2e_times.append(t4 - t0)
        e2e_phases.append({'state_create_s': t1 - t0, 'iterate_s': t2 - t1, 'triples_s': t3 - t2,
                           'amplitudes_destroy_s': t4 - t3})
    e2e_profile = None
    if args.e2e_steps > 0:  # one more, untimed, with the library's phase timers on
        ctx.profile(True)
        se = ctx.state(eri_h, wl.eps, o, precision='mixed', max_iterations=1000)
        se.iterate(1)
        se.triples('mixed')
        se.amplitudes()
        se.close()
        rep = ctx.profile_report()
        ctx.profile(False)
        e2e_profile = {k: round(v['ms'], 3) for k, v in rep.items()
                       if k.startswith('host:') or v['ms'] > 1.0}
    med = int(np.argsort(e2e_times)[len(e2e_times) // 2]) if e2e_times else None
    e2e = {'value': float(np.median(e2e_times)) if e2e_times else None, 'unit': UNIT,
           'statistic': f'median of {len(e2e_times)} steps',
           'h2d_bytes_per_step': int(8 * (N ** 4 + N)),
           'd2h_bytes_per_step': int(8 * (o * v + o * o * v * v) + 64),
           'path': 'scess_rccsd_state_create (eri from pinned host) + state_iterate(1) + '
                   'state_triples(MIXED) + state_amplitudes + destroy',
           'phases_of_median': e2e_phases[med] if e2e_times else None,
           'all_times': e2e_times, 'profiled_ms': e2e_profile,
           'pinned_h2d_gbps_torch_probe': h2d_probe}

    # ---- CPU baseline (rank 0 only) -------------------------------------------------------------
    cpu = None
    if rank == 0 and not args.no_cpu:
        t, det = cpu_oracle_step(np.asarray(eri_h), wl.eps, o)
        cpu = {'value': t, 'unit': UNIT, 'cores': os.cpu_count(), 'kind': 'port',
               'sample': CPU_SAMPLE, 'details': det}

    if rank == 0:
        line = {'metric': METRIC, 'value': step_s, 'unit': UNIT, 'n_gpus': world, 'steps': args.steps,
                'warmup': args.warmup, 'ms_per_step': step_s * 1e3, 'higher_is_better': False,
                'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f16x2-split (FP32 acc) + f64',
                'data': 'synthetic', 'config': config,
                'step': 'one mixed CCSD iteration + one mixed (T) on a state held in its mixed phase',
                'breakdown_ms': {'ccsd_iter': float(np.mean(it_ms)), 'triples': float(np.mean(t_ms)),
                                 'wall_per_step': wall * 1e3},
                'E_T_mixed': ets[-1], 'E_ccsd_iter_mixed': float(hist_mixed[n_iter_mixed - 1, 0]),
                'fp64': fp64, 'converged': converged, 'triples_o24_v240': large_t,
                'roofline': roofline, 'kernel_share': share,
                'kernel_timers': prof, 'cpu_baseline': cpu, 'e2e': e2e,
                'gpu_launches': launches // max(args.steps, 1),
                'gpu_launches_total': launches, 'clocks': clocks}
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == '__main__':
    main()
