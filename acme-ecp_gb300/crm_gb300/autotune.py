"""Launch-shape autotuner for the column kernel.

The kernel can run with several launch shapes (threads per CTA, CTAs per SM
the register budget is sized for, scratch planes in shared memory;
crm_launch_shape_info).  Which is fastest depends on the CRM size, the
precision and the batch; results are identical for every shape.  `autotune`
times each launchable shape on the caller's own device-resident batch
(restoring the state before every trial, so the batch is left as it was)
and leaves the handle on the fastest.
"""
import ctypes as C

from . import lib as L


def shapes():
    """[(index, threads, ctas_per_sm, smem_planes)] of the library's table."""
    lib = L.load()
    out = []
    for s in range(lib.crm_num_launch_shapes()):
        t, c, m = C.c_int(), C.c_int(), C.c_int()
        lib.crm_launch_shape_info(s, C.byref(t), C.byref(c), C.byref(m))
        out.append((s, t.value, c.value, m.value))
    return out


def autotune(ctx, dev, state, reps=2, stream=None):
    """Time every launchable shape of handle `ctx` on DeviceCrmArrays `dev`
    (initial state `state`, restored before each run) and select the
    fastest.  Returns (best shape, {shape: median ms})."""
    import torch
    stream = stream or torch.cuda.current_stream().cuda_stream
    times = {}
    for s, _, _, _ in shapes():
        if ctx.set_launch_shape(s) != 0:
            continue
        ms = []
        for _ in range(reps + 1):
            dev.reset_state(state)
            ctx.run_device(dev, stream)
            ms.append(ctx.last_kernel_ms)
        times[s] = sorted(ms[1:])[len(ms[1:]) // 2]      # first run warms up
    best = min(times, key=times.get)
    ctx.set_launch_shape(best)
    dev.reset_state(state)
    return best, times
