"""Benchmark of the GB300 crm(): CRM column-steps/s on the 2D nx64 nz58 workload.

One step = one crm() call: 1024 GCM columns, each an embedded 64 x 58 CRM
(dx 1 km, dt 10 s) integrated over one GCM step of 1200 s (120 CRM steps),
sam1mom microphysics, SGS TKE, MPDATA.  Throughput = ncrms * nstop /
seconds.  Reported:
  value   FP32-mixed form, arguments resident in HBM (crm_run_device),
          device time from CUDA events around the K timed calls
  e2e     the same through the host C ABI (crm_run) from pinned host
          buffers, host<->device copies inside the timed region
  fp64    the FP64 plain form (bit-identical to the CPU oracle), same way
  cpu_baseline  the CPU FP64 restatement on the host cores (bounded sample)

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

For N > 1 (torchrun) every rank integrates its own 1024 columns: CRM columns
are independent, so the work shards with no collective ("weak" scaling).
--impl reference times the CPU restatement of the reference's crm() on the
host cores instead (the reference itself is Fortran/OpenACC and cannot be
built here).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, 'acme-ecp_gb300'))

METRIC = 'CRM column-steps/s, nx64 nz58, FP32-mixed vs FP64 on 1 GB300; p99 chunk latency'
UNIT = 'column-steps/s'
NCRMS = 1024
WORDS_PER_CELL = 27          # algorithmic HBM words per cell per CRM step


def measured_peaks():
    try:
        with open(os.path.join(REPO, 'MEASURED_PEAKS.json')) as f:
            d = json.load(f)
        return float(d['hbm_gbs']), 'measured'
    except Exception:
        return 6800.0, 'fallback'


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled while the timed region runs."""
    Q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
         'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
         'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, gpu):
        self.gpu = gpu
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', '-i', str(self.gpu), '--query-gpu=' + self.Q,
                 '--format=csv,noheader,nounits', '-lms', '200'],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(',')])

    def stop(self):
        if self.proc is None:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['unavailable']}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                smax = float(r[2])
                for n, v in zip(names, r[5:9]):
                    if v.strip().lower() in ('active', '1'):
                        reasons.add(n)
            except (ValueError, IndexError):
                pass
        return {'sm_mhz': float(np.median(sm)) if sm else None, 'sm_max_mhz': smax,
                'reasons': sorted(reasons), 'samples': len(sm)}


def dist_info():
    ws = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    return ws, rank, local


def cpu_baseline(ncols, nthreads=0):
    """The oracle (CPU FP64 restatement) on a bounded sample of the workload."""
    sys.path.insert(0, os.path.join(REPO, 'oracle'))
    import oracle
    from crm_gb300 import synthetic as S
    oracle.build()
    cfg, cin, st, rad, desc = S.workload_64x58(ncrms=ncols)
    cores = nthreads or os.cpu_count()
    t0 = time.perf_counter()
    rc, _, _ = oracle.run(cfg, desc, cin, st, rad, nthreads=cores)
    dt = time.perf_counter() - t0
    return {'value': ncols * 120 / dt, 'unit': UNIT, 'cores': cores, 'kind': 'port',
            'sample': 'per-column rate measured on %d of the %d columns (columns are independent, so the '
                      'rate of the full batch is this rate); full GCM step (120 CRM steps), FP64, '
                      'OpenMP over columns' % (ncols, NCRMS), 'seconds': dt, 'rc': rc}


def workload_config(nstop=120):
    """The bench workload, as both arms report it in `config`."""
    return {'workload': '2D CRM batch: %d columns x (64 x 1 x 58), dx 1 km, dt 10 s, '
                        'dt_gl 1200 s (%d CRM steps), sam1mom, SGS TKE, MPDATA' % (NCRMS, nstop),
            'ncrms': NCRMS, 'crm_nx': 64, 'crm_nz': 58, 'plev': 72, 'nstop': nstop,
            'batch_mode': 'per-column'}


def run_reference(args):
    ws, rank, _ = dist_info()
    if rank != 0:
        return
    ncols = int(os.environ.get('CRM_BENCH_CPU_COLS', '128'))
    for _ in range(args.warmup):
        cpu_baseline(ncols)
    vals = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        vals.append(cpu_baseline(ncols))
    total = time.perf_counter() - t0
    v = ncols * 120 * args.steps / total
    cb = dict(vals[-1])
    cb['value'] = v
    line = {'metric': METRIC, 'value': v, 'unit': UNIT, 'n_gpus': ws, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': 1000 * total / args.steps,
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
            'dtype': 'f64', 'data': 'synthetic', 'impl': 'reference',
            'config': dict(workload_config(), form='fp64, CPU restatement of crm() on the host cores',
                           sample='per-column rate measured on %d of the %d columns per step (columns are '
                                  'independent: the rate of the whole batch is this rate)' % (ncols, NCRMS)),
            'cpu_baseline': {k: cb[k] for k in ('value', 'unit', 'cores', 'kind', 'sample')},
            'e2e': {'value': v, 'unit': UNIT, 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=5)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--fp64-steps', type=int, default=2)
    ap.add_argument('--cpu-cols', type=int, default=512)
    ap.add_argument('--autotune', type=int, default=1, help='choose the launch shape by timing (1) or use the default table (0)')
    ap.add_argument('--serve-seconds', type=float, default=15.0,
                    help='duration of each serving window: the closed-loop peak and the 25/50/80/100%% '
                         'loads (0: skip serving)')
    ap.add_argument('--serve-steps', type=int, default=48, help='GCM steps per served chunk')
    ap.add_argument('--steps-3d', type=int, default=2,
                    help='timed steps of the 3D batch (256 columns of 32 x 32 x 58; 0: skip it)')
    ap.add_argument('--moist-steps', type=int, default=3,
                    help='timed steps of the moist 1024-column batch (0: skip it)')
    args = ap.parse_args()
    if args.impl == 'reference':
        return run_reference(args)

    import torch
    from crm_gb300 import build as B
    from crm_gb300 import synthetic as S
    from crm_gb300 import crm_types as T
    from crm_gb300.device import DeviceCrmArrays
    from crm_gb300.lib import CrmContext
    from crm_gb300.shard import column_shard
    from crm_gb300.autotune import autotune

    ws, rank, local = dist_info()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group('nccl')
    else:
        torch.cuda.set_device(0)
    if rank == 0:
        B.build()
    if ws > 1:
        dist.barrier()
    B.build()

    def barrier():
        if ws > 1:
            dist.barrier()
        torch.cuda.synchronize()

    # ---- synthetic workload (each rank its own columns)
    # weak scaling: NCRMS columns per rank, rank r owning global columns
    # [r * NCRMS, (r + 1) * NCRMS) (contiguous blocks, no data exchange)
    first, count = column_shard(ws * NCRMS, rank, ws)
    cfg32, cin, st, rad, desc = S.workload_64x58(ncrms=count, seed=first, gcol0=first + 1,
                                            precision=T.CRM_FP32_MIXED)
    cfg32.max_ncrms = NCRMS
    nstop = int(desc.dt_gl / cfg32.crm_dt)
    colsteps = NCRMS * nstop
    cells = cfg32.crm_nx * cfg32.crm_ny * cfg32.crm_nz

    tuned = {}
    medians = {}        # median per-step time of each form on this rank [ms]

    def device_rate(cfg, steps, warmup, work=None, tag=None, tune=True):
        w_cin, w_st, w_rad, w_desc = work or (cin, st, rad, desc)
        tag = tag or ('fp64' if cfg.precision == T.CRM_FP64 else 'fp32')
        ctx = CrmContext(cfg)
        dev = DeviceCrmArrays(cfg, w_cin, w_st, w_rad, w_desc, w_desc._keep)
        stream = torch.cuda.current_stream().cuda_stream
        # launch shape chosen by the autotuner on this batch (untimed)
        if args.autotune and tune:
            best, times = autotune(ctx, dev, w_st, reps=1, stream=stream)
            tuned[tag] = {'shape': best, 'ms_per_shape': {str(k): round(v, 2) for k, v in times.items()}}
        # warm-up: at least `warmup` calls and at least 2 s of device work
        # (a GPU coming out of idle runs its first seconds slower)
        t_w = time.perf_counter()
        nw = 0
        while nw < warmup or time.perf_counter() - t_w < 2.0:
            dev.reset_state(w_st)
            ctx.run_device(dev, stream)
            torch.cuda.synchronize()
            nw += 1
        barrier()
        # each step restarts from the same initial state (igstep 1): the
        # state (213 MB) is re-read from HBM every step, larger than L2
        kms = []
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        tot = 0.0
        step_ms = []
        for _ in range(steps):
            dev.reset_state(w_st)
            e0.record()
            ctx.run_device(dev, stream)
            e1.record()
            e1.synchronize()
            dt = e0.elapsed_time(e1)
            tot += dt
            step_ms.append(dt)
            kms.append(ctx.last_kernel_ms)
        medians[tag] = float(np.median(step_ms))
        if tag not in tuned:
            tuned[tag] = {'shape': ctx.launch_shape, 'ms_per_step_median': round(medians[tag], 2)}
        barrier()
        t = torch.tensor([tot], device='cuda')
        if ws > 1:
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item()) / steps
        return ctx, dev, ms, kms

    clocks = ClockSampler(local)
    clocks.start()
    ctx32, dev32, ms32, kms32 = device_rate(cfg32, args.steps, args.warmup)
    clk = clocks.stop()
    value = ws * colsteps / (ms32 / 1000.0)

    # ---- end to end through the host C ABI, pinned host buffers
    def pinned_copy(bundle):
        out = bundle.copy()
        for n, a in bundle.arrays().items():
            t = torch.empty(a.shape[::-1], dtype=torch.float64, pin_memory=True)
            v = t.numpy().T
            v[...] = a
            setattr(out, n, v)
            out._keep = getattr(out, '_keep', []) + [t]
        return out

    cin_p, st_p, rad_p = pinned_copy(cin), pinned_copy(st), pinned_copy(rad)
    out_t = {}
    out_p = T.CrmOutput(desc.ld, cfg32.crm_nx, cfg32.crm_ny, cfg32.crm_nz, cfg32.plev)
    for n, a in out_p.arrays().items():
        t = torch.empty(a.shape[::-1], dtype=torch.float64, pin_memory=True)
        out_t[n] = t
        setattr(out_p, n, t.numpy().T)
    ctx32.run(desc, cin_p, st_p, rad_p, out_p)
    barrier()
    e2e_t = 0.0
    for _ in range(args.steps):
        for n, a in st.arrays().items():
            getattr(st_p, n)[...] = a
        t0 = time.perf_counter()
        ctx32.run(desc, cin_p, st_p, rad_p, out_p)
        e2e_t += time.perf_counter() - t0
    barrier()
    tt = torch.tensor([e2e_t], device='cuda')
    if ws > 1:
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    e2e_ms = float(tt.item()) * 1000.0 / args.steps
    ld = desc.ld
    h2d = (sum(a.nbytes for a in cin.arrays().values() if a.ndim == 2) + 3 * ld * 8 + 4 * ld +
           sum(a.nbytes for a in st.arrays().values()) + rad.qrad.nbytes)
    d2h = (sum(a.nbytes for a in st.arrays().values()) + 5 * rad.qrad.nbytes +
           sum(a.nbytes for a in out_p.arrays().values()) + 4 * NCRMS)

    # ---- FP64 plain form
    cfg64 = S.config_64x58(precision=T.CRM_FP64)
    cfg64.max_ncrms = NCRMS
    ctx64, dev64, ms64, _ = device_rate(cfg64, args.fp64_steps, 1)
    value64 = ws * colsteps / (ms64 / 1000.0)
    # the FP64 form with multiply-add contraction (within 1e-10 of the plain
    # form, not bit-identical)
    cfgf = S.config_64x58(precision=T.CRM_FP64_FMA)
    cfgf.max_ncrms = NCRMS
    ctxf, devf, msf, _ = device_rate(cfgf, args.fp64_steps, 1, tag='fp64_fma', tune=False)
    valuef = ws * colsteps / (msf / 1000.0)

    # ---- accuracy of the FP32-mixed form against the FP64 form (same inputs)
    # (the FP64 form equals the oracle bit for bit, so this is the error
    # against the oracle): every state field and every crm() output
    def rel(a, b):
        den = np.linalg.norm(b)
        return float(np.linalg.norm(a - b) / den) if den > 0 else float(np.linalg.norm(a - b))

    def form_errors(d32, d64, n=NCRMS):
        es = {k: rel(d32.state_numpy(k)[:n], d64.state_numpy(k)[:n]) for k in d32.state}
        eo = {k: rel(d32.out_numpy(k)[:n], d64.out_numpy(k)[:n]) for k in d32.out}
        return es, eo

    errs, errs_out = form_errors(dev32, dev64)
    esf, eof = form_errors(devf, dev64)
    del ctxf, devf
    del ctx64, dev64

    # ---- the same batch from moist soundings: clouds and rain form, so the
    # exact sedimentation / qp-transport skips apply to no precipitating
    # column (the dry headline takes both skips in every column)
    moist = None
    if args.moist_steps > 0:
        mw = S.workload_64x58(ncrms=count, seed=first, gcol0=first + 1, precision=T.CRM_FP32_MIXED, moist=True)
        mcfg32, mwork = mw[0], mw[1:]
        mcfg32.max_ncrms = NCRMS
        mctx32, mdev32, mms32, _ = device_rate(mcfg32, args.moist_steps, 1, mwork, 'fp32_moist')
        mcfg64 = S.config_64x58(precision=T.CRM_FP64)
        mcfg64.max_ncrms = NCRMS
        mctx64, mdev64, mms64, _ = device_rate(mcfg64, 1, 1, mwork, 'fp64_moist')
        mes, meo = form_errors(mdev32, mdev64)
        prec_cols = int((mdev64.out_numpy('precc')[:NCRMS] + mdev64.out_numpy('precl')[:NCRMS] > 0).sum())
        moist = {'workload': 'as the headline, moist soundings (supersaturated layers; clouds and rain form)',
                 'value': ws * colsteps / (mms32 / 1000.0), 'unit': UNIT, 'ms_per_step': mms32,
                 'steps': args.moist_steps, 'fp64_value': ws * colsteps / (mms64 / 1000.0),
                 'fp64_ms_per_step': mms64, 'precipitating_columns': prec_cols,
                 'fp32_rel_l2_vs_fp64_tendencies': {n: meo[n] for n in ('sltend', 'qltend', 'qcltend', 'qiltend')},
                 'fp32_rel_l2_vs_fp64_state': mes, 'fp32_rel_l2_vs_fp64_outputs': meo}
        del mctx32, mdev32, mctx64, mdev64

    # ---- the 3D CRM: 256 columns of 32 x 32 x 58 (dx = dy = 2 km), dt_gl
    # 1200 s, the headline's soundings with a sheared v
    three_d = None
    if args.steps_3d > 0:
        n3 = 256
        f3, c3 = column_shard(ws * n3, rank, ws)
        w3 = S.workload_3d(ncrms=c3, seed=f3, gcol0=f3 + 1, precision=T.CRM_FP32_MIXED)
        cfg3, work3 = w3[0], w3[1:]
        cfg3.max_ncrms = n3
        cs3 = n3 * int(work3[3].dt_gl / cfg3.crm_dt)
        ctx3, dev3, ms3, kms3 = device_rate(cfg3, args.steps_3d, 1, work3, 'fp32_3d')
        # the same with the pressure solve's transforms on the tensor cores
        # (their own kernel instance, one CTA per SM)
        os.environ['CRM_GB300_TRANSFORM'] = 'tc'
        try:
            ctx3t, dev3t, ms3t, _ = device_rate(cfg3, 1, 1, work3, 'fp32_3d_tc', tune=False)
        finally:
            os.environ.pop('CRM_GB300_TRANSFORM', None)
        es3t, eo3t = form_errors(dev3t, dev3, n3)
        del ctx3t, dev3t
        cfg3d = S.config_3d(precision=T.CRM_FP64)
        cfg3d.max_ncrms = n3
        ctx3d, dev3d, ms3d, _ = device_rate(cfg3d, 1, 1, work3, 'fp64_3d', tune=False)
        es3, eo3 = form_errors(dev3, dev3d, n3)
        cells3 = cfg3.crm_nx * cfg3.crm_ny * cfg3.crm_nz
        three_d = {'workload': '%d columns of %d x %d x %d, dx = dy = %.0f m, dt %.0f s, dt_gl %.0f s' %
                               (n3, cfg3.crm_nx, cfg3.crm_ny, cfg3.crm_nz, cfg3.crm_dx, cfg3.crm_dt, work3[3].dt_gl),
                   'value': ws * cs3 / (ms3 / 1000.0), 'unit': UNIT, 'ms_per_step': ms3,
                   'kernel_ms': float(np.median(kms3)), 'steps': args.steps_3d,
                   'cell_steps_per_s': ws * cs3 * cells3 / (ms3 / 1000.0),
                   'fp64_value': ws * cs3 / (ms3d / 1000.0), 'fp64_ms_per_step': ms3d, 'fp64_steps': 1,
                   'fp32_rel_l2_vs_fp64_state': es3,
                   'fp32_rel_l2_vs_fp64_tendencies': {n: eo3[n] for n in ('sltend', 'qltend', 'qcltend', 'qiltend')},
                   'fp32_tensor_core_transforms': {
                       'value': ws * cs3 / (ms3t / 1000.0), 'ms_per_step': ms3t, 'steps': 1,
                       'note': 'x/y transforms of the pressure solve as split-TF32 tcgen05 GEMMs; the kernel '
                               'instance with tcgen05 code runs one CTA per SM',
                       'rel_l2_vs_fft_form_tendencies': {n: eo3t[n] for n in ('sltend', 'qltend')}}}
        del ctx3, dev3, ctx3d, dev3d

    # ---- serving: Poisson chunks of mixed (nx, nz) at 80 % of the closed-loop peak
    serving = None
    if rank == 0 and args.serve_seconds > 0:
        from crm_gb300 import serve_bench as SB
        from crm_gb300.serving import CrmServer, config_key
        scfg = SB.chunk_configs(T.CRM_FP32_MIXED)
        server = CrmServer(scfg, capacity=1024, hbm_budget=120 * 2 ** 30)
        for c in scfg:
            server.pool(config_key(c))
        steps_per_chunk = args.serve_steps
        pk = SB.measure_peak(server, scfg, steps_per_chunk, args.serve_seconds)
        if pk['column_steps_per_s'] > 0:
            sweep = []
            for f in (0.25, 0.5, 0.8, 1.0):
                r = SB.run_load(server, scfg, steps_per_chunk, f * pk['column_steps_per_s'], args.serve_seconds)
                sweep.append({'load': f, 'offered_column_steps_per_s': r['offered_column_steps_per_s'],
                              'column_steps_per_s': r['column_steps_per_s'], 'p50_ms': r['p50_ms'],
                              'p99_ms': r['p99_ms'], 'chunk_steps': r['steps'], 'chunks': r['chunks']})
            at80 = sweep[2]
            serving = {'workload': 'chunks of U{1..64} columns, crm_nx in {32,64,128}, crm_nz in {28,58}, '
                                   '72 levels, dt_gl 1200 s, %d GCM steps per chunk, Poisson arrivals, '
                                   'FP32-mixed, 120 GB HBM budget' % steps_per_chunk,
                       'peak_column_steps_per_s': pk['column_steps_per_s'], 'peak_p50_ms': pk['p50_ms'],
                       'peak_p99_ms': pk['p99_ms'],
                       'load': 0.8, 'offered_column_steps_per_s': at80['offered_column_steps_per_s'],
                       'column_steps_per_s': at80['column_steps_per_s'],
                       'p50_ms': at80['p50_ms'], 'p99_ms': at80['p99_ms'], 'chunk_steps': at80['chunk_steps'],
                       'sweep': sweep, 'window_s': args.serve_seconds,
                       'note': 'achieved counts the chunk-steps completed inside the window after a 25 % warm-up; '
                               'chunks still running at its end are not counted',
                       'launches': server.launches}
        else:
            # a window too short for any chunk-step to finish
            serving = {'skipped': 'no chunk-step completed in the %.1f s peak window' % args.serve_seconds}
        server.close()

    if rank != 0:
        if ws > 1:
            dist.destroy_process_group()
        return
    peak, peak_kind = measured_peaks()
    kernel_ms = float(np.median(kms32))
    bytes_per_launch = NCRMS * nstop * cells * WORDS_PER_CELL * 4
    achieved = bytes_per_launch / (kernel_ms / 1000.0) / 1e9
    traffic = None
    try:
        with open(os.path.join(REPO, 'profiles', 'crm_columns_fp32_traffic.json')) as f:
            tr = json.load(f)
        traffic = tr.get('bytes_per_launch')
    except Exception:
        pass
    # the FP64 form is bound by the FP64 pipe (2 lanes per SM per clock on
    # GB300): its FP64 warp-instructions per column-step (ncu) against the
    # pipe's peak at the sampled SM clock
    fp64_pipe = None
    try:
        with open(os.path.join(REPO, 'profiles', 'crm_columns_fp64_pipe.json')) as f:
            fp = json.load(f)
        nsm = torch.cuda.get_device_properties(local).multi_processor_count
        mhz = (clk or {}).get('sm_mhz') or 2070.0
        peak_inst = nsm * fp['peak_fp64_warp_inst_per_sm_cycle'] * mhz * 1e6
        fp64_pipe = {'frac': value64 / ws * fp['fp64_warp_inst_per_column_step'] / peak_inst,
                     'fp64_warp_inst_per_column_step': fp['fp64_warp_inst_per_column_step'],
                     'peak_warp_inst_per_s': peak_inst, 'sm_mhz': mhz}
    except Exception:
        pass
    cb = None
    if ws == 1:
        try:
            c = cpu_baseline(args.cpu_cols)
            cb = {k: c[k] for k in ('value', 'unit', 'cores', 'kind', 'sample')}
        except Exception as e:  # the oracle needs g++; report why it is absent
            cb = {'value': None, 'unit': UNIT, 'cores': os.cpu_count(), 'kind': 'port',
                  'sample': 'failed: %s' % e}
    line = {
        'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': ws, 'steps': args.steps,
        'warmup': args.warmup, 'ms_per_step': ms32, 'ms_per_step_median': medians.get('fp32'),
        'higher_is_better': True,
        'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'f32 (f64 tridiagonal solve, domain sums, saturation Newton)',
        'data': 'synthetic (idealised soundings, seeded)',
        'config': dict(workload_config(nstop), form='fp32-mixed',
                       l2='inputs larger than L2: every step re-reads the %d MB state' %
                          (dev32.nbytes_state() // 2 ** 20)),
        'roofline': {'bound': 'hbm', 'achieved': achieved, 'peak': peak, 'unit': 'GB/s',
                     'frac': achieved / peak, 'traffic': traffic,
                     'peak_kind': peak_kind, 'kernel_ms': kernel_ms,
                     'algorithmic_bytes_per_launch': bytes_per_launch},
        'cpu_baseline': cb,
        'e2e': {'value': ws * colsteps / (e2e_ms / 1000.0), 'unit': UNIT,
                'h2d_bytes_per_step': int(h2d), 'd2h_bytes_per_step': int(d2h),
                'ms_per_step': e2e_ms},
        'clocks': clk,
        'gpu_launches': 2 * args.steps,   # crm_prep_kernel + crm_columns_kernel per timed step
        'fp64_plain': {'value': value64, 'unit': UNIT, 'ms_per_step': ms64,
                       'ms_per_step_median': medians.get('fp64'), 'steps': args.fp64_steps,
                       'fp64_pipe': fp64_pipe},
        'fp64_fma': {'value': valuef, 'unit': UNIT, 'ms_per_step': msf, 'steps': args.fp64_steps,
                     'max_rel_l2_vs_fp64_plain': max(list(esf.values()) + list(eof.values()))},
        'fp32_over_fp64': value / value64,
        'fp32_rel_l2_vs_fp64_state': errs,
        'fp32_rel_l2_vs_fp64_outputs': errs_out,
        'serving': serving,
        'moist': moist,
        'crm_3d': three_d,
        'launch_shapes': tuned,
    }
    print(json.dumps(line))
    if ws > 1:
        dist.destroy_process_group()


if __name__ == '__main__':
    main()
