"""A small, self-contained crm() run for profilers (ncu) and quick timing.

    python profile_case.py --ncrms 152 --dt-gl 100 \
        --precision fp32 --reps 2

runs the 64 x 58 workload (--workload 64x58, the default; 32x28: 16-column
sized one at dx 4 km, dt 20 s; 3d: the 3D CRM, --nx x --ny x 58 at dx = dy
= 2 km, dt 10 s) on
device-resident arrays (crm_run_device) `reps` times and prints the kernel
time of each call.  Sized so that a profiler capture of one launch ends in
seconds.
"""
import argparse
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, 'acme-ecp_gb300'))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--ncrms', type=int, default=152)
    ap.add_argument('--dt-gl', type=float, default=100.0)
    ap.add_argument('--precision', default='fp32', choices=['fp32', 'fp64'])
    ap.add_argument('--reps', type=int, default=2)
    ap.add_argument('--nx', type=int, default=64)
    ap.add_argument('--ny', type=int, default=32, help='3D workload: crm_ny')
    ap.add_argument('--workload', default='64x58', choices=['32x28', '64x58', '3d'])
    ap.add_argument('--shape', type=int, default=None,
                    help='column-kernel launch shape index (crm_kernel.h kShapes)')
    ap.add_argument('--phase-timers', action='store_true',
                    help='use the profiling build and print cycles per phase')
    args = ap.parse_args()
    if args.shape is not None:
        os.environ['CRM_GB300_SHAPE'] = str(args.shape)
    import torch
    from crm_gb300 import build as B
    from crm_gb300 import synthetic as S
    from crm_gb300 import crm_types as T
    from crm_gb300.device import DeviceCrmArrays
    from crm_gb300 import lib as L
    from crm_gb300.lib import CrmContext
    L.load(path=B.build(phase_timers=args.phase_timers))
    prec = T.CRM_FP32_MIXED if args.precision == 'fp32' else T.CRM_FP64
    if args.workload == '32x28':
        cfg, cin, st, rad, desc = S.workload_32x28(ncrms=args.ncrms, precision=prec)
    elif args.workload == '3d':
        cfg, cin, st, rad, desc = S.workload_3d(ncrms=args.ncrms, nx=args.nx, ny=args.ny, precision=prec)
    else:
        cfg, cin, st, rad, desc = S.workload_64x58(ncrms=args.ncrms, nx=args.nx, precision=prec)
    desc.dt_gl = args.dt_gl
    cfg.max_ncrms = args.ncrms
    ctx = CrmContext(cfg)
    dev = DeviceCrmArrays(cfg, cin, st, rad, desc, desc._keep)
    stream = torch.cuda.current_stream().cuda_stream
    for r in range(args.reps):
        dev.reset_state(st)
        ctx.run_device(dev, stream)
        ms = ctx.last_kernel_ms
        nstop = int(args.dt_gl / cfg.crm_dt)
        print('rep %d: %.3f ms  (%.0f column-steps/s)' % (r, ms, args.ncrms * nstop / (ms / 1000.0)))
    torch.cuda.synchronize()
    assert int(dev.status.sum().item()) == 0
    import hashlib
    h = hashlib.sha256()
    for n in sorted(dev.state):
        h.update(dev.state[n].cpu().numpy().tobytes())
    print('state sha256 %s' % h.hexdigest()[:16])
    if args.phase_timers:
        from crm_gb300.crm_types import PHASE_NAMES
        cyc = ctx.phase_cycles()
        tot = float(sum(cyc)) or 1.0
        print('phase cycles (all CTAs, %d reps):' % args.reps)
        for name, c in sorted(zip(PHASE_NAMES, cyc), key=lambda x: -x[1]):
            print('  %-12s %6.2f %%  %.3e' % (name, 100.0 * c / tot, c))


if __name__ == '__main__':
    main()
