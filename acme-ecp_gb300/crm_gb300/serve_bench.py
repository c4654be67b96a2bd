"""Serving workload: Poisson-arriving GCM chunks against a CrmServer.

    python acme-ecp_gb300/crm_gb300/serve_bench.py [--loads 0.25,0.5,0.8,1.0]
        [--duration 60] [--steps 48] [--precision fp32|fp64]

Chunks of U{1..64} columns with crm_nx in {32, 64, 128} and crm_nz in
{28, 58} (72-level GCM, dx 1 km, dt 10 s, dt_gl 1200 s) arrive as a Poisson
process.  Each chunk is admitted (slots + HBM budget), keeps its CRM state
resident and runs `steps` GCM steps; after every step its driver applies the
returned tendencies to its GCM columns (state += ptend * dt_gl) and submits
the next step at once.  Peak throughput is measured first with a closed
loop that keeps the GPU full; each load level then offers that fraction of
the peak in column-steps/s.  Reported per level: achieved column-steps/s and
p50 / p99 latency of a chunk's GCM step (submit -> results on the host).
"""
import argparse
import json
import os
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if __name__ == '__main__':
    sys.path.insert(0, os.path.dirname(HERE))

from crm_gb300 import crm_types as T            # noqa: E402
from crm_gb300 import synthetic as S            # noqa: E402
from crm_gb300.serving import CrmServer, apply_tendencies, config_key  # noqa: E402

NX_CHOICES = (32, 64, 128)
NZ_CHOICES = (28, 58)
DT_GL = 1200.0


def chunk_configs(precision):
    return [T.CrmConfig(crm_nx=nx, crm_ny=1, crm_nz=nz, plev=72, crm_dx=1000.0, crm_dt=10.0,
                        precision=precision) for nx in NX_CHOICES for nz in NZ_CHOICES]


def make_chunk(cfg, ncol, gcol0, seed):
    """Inputs of one chunk from the 72-level workload soundings."""
    rng = np.random.Generator(np.random.PCG64(10_000 + seed))
    lat = rng.uniform(-60.0, 60.0, size=ncol)
    cl = np.cos(np.deg2rad(lat))
    cin, st, rad, desc = S.make_inputs(cfg, ncol, 271.0 + 29.0 * cl, 10.0 * cl, 100.0 * cl,
                                       seed=seed, gcol0=gcol0)
    return cin, st, rad, list(np.asarray(desc._keep))


class Driver:
    """Runs chunks to completion and records step latencies and work."""

    def __init__(self, server, configs, steps, seed=0):
        self.server = server
        self.configs = configs
        self.steps = steps
        self.rng = np.random.Generator(np.random.PCG64(seed))
        self.lock = threading.Lock()
        self.lat = []              # (t_done, latency, column-steps)
        self.threads = []
        self.next_gcol = 1
        self.errors = []

    def spawn(self, t_stop):
        cfg = self.configs[int(self.rng.integers(len(self.configs)))]
        ncol = int(self.rng.integers(1, 65))
        seed = int(self.rng.integers(1 << 30))
        with self.lock:
            g0 = self.next_gcol
            self.next_gcol += ncol
        th = threading.Thread(target=self._run, args=(cfg, ncol, g0, seed, t_stop), daemon=True)
        th.start()
        self.threads.append(th)

    def _run(self, cfg, ncol, g0, seed, t_stop):
        try:
            cin, st, rad, gcol = make_chunk(cfg, ncol, g0, seed)
            ch = self.server.open_chunk(cfg, cin, st, rad, gcol)
            nstop = int(DT_GL / cfg.crm_dt)
            try:
                for _ in range(self.steps):
                    if time.perf_counter() > t_stop:
                        break
                    t0 = time.perf_counter()
                    vals, status = self.server.step(ch, cin, DT_GL).result(timeout=300)
                    t1 = time.perf_counter()
                    if status.any():
                        raise RuntimeError('column status %s' % status)
                    with self.lock:
                        self.lat.append((t1, t1 - t0, ncol * nstop))
                    apply_tendencies(cin, vals, DT_GL)
            finally:
                self.server.close_chunk(ch)
        except Exception as e:        # recorded and re-raised by the caller
            self.errors.append(e)

    def window(self, t0, t1):
        rows = [r for r in self.lat if t0 <= r[0] <= t1]
        if not rows:
            return {'column_steps_per_s': 0.0, 'p50_ms': None, 'p99_ms': None, 'steps': 0}
        lat = np.array([r[1] for r in rows]) * 1000.0
        work = sum(r[2] for r in rows)
        return {'column_steps_per_s': work / (t1 - t0), 'p50_ms': float(np.percentile(lat, 50)),
                'p99_ms': float(np.percentile(lat, 99)), 'steps': len(rows)}


def measure_peak(server, configs, steps, duration, concurrency=64, seed=1):
    """Closed loop: keep `concurrency` chunks in flight; column-steps/s."""
    d = Driver(server, configs, steps, seed)
    t_start = time.perf_counter()
    t_stop = t_start + duration
    while time.perf_counter() < t_stop:
        alive = sum(t.is_alive() for t in d.threads)
        for _ in range(concurrency - alive):
            d.spawn(t_stop)
        time.sleep(0.01)
    for t in d.threads:
        t.join()
    if d.errors:
        raise d.errors[0]
    warm = t_start + 0.25 * duration
    return d.window(warm, t_stop)


def run_load(server, configs, steps, rate_colsteps, duration, seed=2):
    """Open loop: Poisson chunk arrivals offering `rate_colsteps` (> 0)."""
    if not rate_colsteps > 0:
        raise ValueError('run_load needs a positive offered rate, got %r' % (rate_colsteps,))
    mean_work = 32.5 * (DT_GL / 10.0) * steps        # E[ncol] * nstop * steps per chunk
    lam = rate_colsteps / mean_work                  # chunks per second
    d = Driver(server, configs, steps, seed)
    rng = np.random.Generator(np.random.PCG64(seed + 1))
    t_start = time.perf_counter()
    t_stop = t_start + duration
    t_next = t_start
    while t_next < t_stop:
        now = time.perf_counter()
        if now < t_next:
            time.sleep(min(t_next - now, 0.01))
            continue
        d.spawn(t_stop)
        t_next += rng.exponential(1.0 / lam)
    for t in d.threads:
        t.join()
    if d.errors:
        raise d.errors[0]
    res = d.window(t_start + 0.25 * duration, t_stop)
    res['offered_column_steps_per_s'] = rate_colsteps
    res['chunks'] = len(d.threads)
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--loads', default='0.25,0.5,0.8,1.0')
    ap.add_argument('--duration', type=float, default=60.0)
    ap.add_argument('--peak-duration', type=float, default=40.0)
    ap.add_argument('--steps', type=int, default=48)
    ap.add_argument('--precision', default='fp32', choices=['fp32', 'fp64'])
    ap.add_argument('--budget-gb', type=float, default=120.0)
    args = ap.parse_args()
    import torch
    from crm_gb300 import build as B
    from crm_gb300 import lib as L
    L.load(path=B.build())
    torch.cuda.set_device(0)
    prec = T.CRM_FP32_MIXED if args.precision == 'fp32' else T.CRM_FP64
    configs = chunk_configs(prec)
    server = CrmServer(configs, capacity=2048, hbm_budget=args.budget_gb * 2 ** 30)
    for c in configs:                  # device pools and handles up front
        server.pool(config_key(c))
    peak = measure_peak(server, configs, args.steps, args.peak_duration)
    out = {'precision': args.precision, 'peak': peak, 'loads': []}
    for f in [float(x) for x in args.loads.split(',')]:
        r = run_load(server, configs, args.steps, f * peak['column_steps_per_s'], args.duration)
        r['load'] = f
        out['loads'].append(r)
        print(json.dumps(r), flush=True)
    server.close()
    print(json.dumps(out))


if __name__ == '__main__':
    main()
