"""Continuous-batching CRM service: resident column state, HBM admission,
per-chunk latency.

The reference integrates the CRMs of each GCM chunk synchronously inside
crm_physics_tend (cam/crm_physics.F90:1145-1156) and keeps every column's CRM
state in the physics buffer between GCM steps (pbuf 'global' fields,
crm_physics.F90:126-191).  Here the same two facts are organised for a GPU
that serves many chunks at once:

  * each configuration gets a device-resident pool of column slots; the
    pool's device memory (its slot arrays and the handles' column slabs) is
    charged to the HBM budget when the pool is created, before anything is
    allocated, and a pool is made smaller, or idle pools of other
    configurations are released, when the budget cannot hold a full one;
    a new configuration that does not fit at all is refused (BudgetError,
    CRM_ERR_BUDGET);
  * each chunk (1..64 GCM columns of one CRM configuration) is *admitted*:
    it receives slots in its configuration's pool if the pool has room;
    otherwise it waits;
  * its CRM state stays in those slots across GCM steps; a step request
    carries only the new GCM input profiles;
  * the engine thread gathers every step request that is waiting, groups
    them by configuration and launches ONE column kernel per group over the
    union of their slots (crm_run_device with a col_map), so requests that
    arrive while others are on the GPU join the next launch; a chunk has at
    most one step in flight (its next request waits until the current one
    completes, since both would integrate the same slots); groups of
    different configurations and successive launches of one configuration
    run on their own streams and overlap on the device;
  * results (the crm_output fields a GCM step consumes) are copied back per
    request and its future completes; latency = submit -> results on host.

Per-column mode makes every column's result independent of what it is
batched with, so a chunk gets the same bits alone and in any mix.
"""
import ctypes as C
import queue
import threading
import time
from concurrent.futures import Future
from dataclasses import dataclass, field

import numpy as np

from . import crm_types as T

# crm_output fields returned to the GCM per step (what crm_physics_tend reads
# back for ptend and the surface fluxes, crm_physics.F90:1163-1300)
STEP_OUTPUTS = ('sltend', 'qltend', 'qcltend', 'qiltend', 'precc', 'precl', 'precsc',
                'precsl', 'cltot', 'prectend', 'precstend', 'taux', 'tauy', 'z0m')


class SlotPool:
    """Free-list of column slots 0..capacity-1 (host logic only)."""

    def __init__(self, capacity):
        self.capacity = int(capacity)
        self._free = list(range(self.capacity - 1, -1, -1))
        self._lock = threading.Lock()

    def alloc(self, n):
        with self._lock:
            if n > len(self._free):
                return None
            return [self._free.pop() for _ in range(n)]

    def free(self, slots):
        with self._lock:
            for s in sorted(slots, reverse=True):
                if s in self._free:
                    raise ValueError('slot %d freed twice' % s)
                self._free.append(s)

    @property
    def available(self):
        return len(self._free)


class BudgetError(RuntimeError):
    """A configuration's pool does not fit the HBM budget (CRM_ERR_BUDGET)."""
    status = T.CRM_ERR_BUDGET


class HbmBudget:
    """Bytes of device memory the service may hold (pools and handles)."""

    def __init__(self, total_bytes):
        self.total = int(total_bytes)
        self.used = 0
        self._lock = threading.Lock()

    def reserve(self, nbytes):
        with self._lock:
            if self.used + nbytes > self.total:
                return False
            self.used += nbytes
            return True

    def release(self, nbytes):
        with self._lock:
            self.used -= nbytes
            if self.used < 0:
                raise ValueError('budget released below zero')


def slot_bytes(cfg):
    """Device bytes one resident column of this configuration holds."""
    nx, nz, plev, nxr = cfg.crm_nx, cfg.crm_nz, cfg.plev, cfg.crm_nx_rad
    state = 7 * nx * nz
    rad = 6 * nxr * nz
    inp = 11 * (plev + 1) + 10
    out = 6 * nx * nz + nx + 16 + 39 * plev
    return 8 * (state + rad + inp + out) + 8


def pool_bytes(cfg, capacity, handles, handle_bytes):
    """Device bytes a DevicePool of `capacity` slots holds: the resident
    arrays of every slot, the per-launch slot maps of each handle, and the
    handles themselves (handle_bytes(cfg with max_ncrms = capacity))."""
    return capacity * slot_bytes(cfg) + handles * 12 * capacity + handles * handle_bytes(capacity)


def config_key(cfg):
    """Everything that selects a handle except the column capacity."""
    return tuple(sorted((k, v) for k, v in cfg.__dict__.items() if k != 'max_ncrms'))


class DevicePool:
    """Device arrays of one configuration with ld = capacity (torch tensors
    in Fortran layout: the column slot is the fastest index), plus the C ABI
    handles that integrate any subset of the slots."""

    def __init__(self, cfg, capacity, handles=2):
        import torch
        from .lib import CrmContext
        self.torch = torch
        self.cfg = T.CrmConfig(**{**cfg.__dict__, 'max_ncrms': capacity})
        self.capacity = capacity
        self.slots = SlotPool(capacity)
        dev = 'cuda'
        ld, nx, nz, plev = capacity, cfg.crm_nx, cfg.crm_nz, cfg.plev
        z = T.CrmInput.zeros(1, plev)
        self.inp = {n: torch.zeros(a.shape[1:][::-1] + (ld,), dtype=torch.float64, device=dev)
                    for n, a in z.arrays().items()}
        self.state = {n: torch.zeros((nz, 1, nx, ld), dtype=torch.float64, device=dev)
                      for n in T.STATE_FIELDS}
        self.rad = {n: torch.zeros((nz, 1, cfg.crm_nx_rad, ld), dtype=torch.float64, device=dev)
                    for n in T.RAD_FIELDS}
        o = T.CrmOutput(1, nx, 1, nz, plev)
        self.out = {n: torch.zeros(a.shape[1:][::-1] + (ld,), dtype=torch.float64, device=dev)
                    for n, a in o.arrays().items()}
        dp = lambda t: C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_double))
        self.c_in = T.CCrmInput(*[dp(self.inp[n]) for n in T.INPUT_FIELDS])
        self.c_state = T.CCrmState(*[dp(self.state[n]) for n in T.STATE_FIELDS])
        self.c_rad = T.CCrmRad(*[dp(self.rad[n]) for n in T.RAD_FIELDS])
        self.c_out = T.CCrmOutput()
        for i, (n, _) in enumerate(T.OUTPUT_FIELDS):
            self.c_out.field[i] = dp(self.out[n])
        self.ctx = [CrmContext(self.cfg) for _ in range(handles)]
        self.streams = [torch.cuda.Stream() for _ in range(handles)]
        self.busy = [False] * handles
        # per-launch device scratch: col_map, gcol, status (one set per handle)
        self.d_map = [torch.zeros(capacity, dtype=torch.int32, device=dev) for _ in range(handles)]
        self.d_gcol = [torch.zeros(capacity, dtype=torch.int32, device=dev) for _ in range(handles)]
        self.d_status = [torch.zeros(capacity, dtype=torch.int32, device=dev) for _ in range(handles)]

    def close(self):
        """Free the handles (the torch arrays go with the pool object)."""
        for c in self.ctx:
            c.close()
        self.ctx = []

    # -- host <-> slots (on a given stream)
    def _scatter(self, dst, slots_t, host):
        """dst[..., slots] = host, host an (n, ...) Fortran-order bundle array
        (its transpose has the device layout: the column index last)."""
        torch = self.torch
        src = torch.from_numpy(np.ascontiguousarray(host.T)).pin_memory()
        dst.index_copy_(dst.dim() - 1, slots_t, src.to(dst.device, non_blocking=True))

    def load(self, slots, cin, st, rad, stream):
        torch = self.torch
        with torch.cuda.stream(stream):
            s = torch.tensor(slots, dtype=torch.int64).to('cuda', non_blocking=True)
            for n, a in st.arrays().items():
                self._scatter(self.state[n], s, a[:len(slots)])
            for n, a in rad.arrays().items():
                self._scatter(self.rad[n], s, a[:len(slots)])
            self.set_inputs(slots, cin, stream, s)

    def set_inputs(self, slots, cin, stream, s=None):
        torch = self.torch
        with torch.cuda.stream(stream):
            if s is None:
                s = torch.tensor(slots, dtype=torch.int64).to('cuda', non_blocking=True)
            for n, a in cin.arrays().items():
                self._scatter(self.inp[n], s, a[:len(slots)])

    def gather(self, slots, names, stream):
        """{name: pinned host tensor (..., n)} for the given slots, copied
        asynchronously on `stream` (valid once the stream reaches it)."""
        torch = self.torch
        res = {}
        with torch.cuda.stream(stream):
            s = torch.tensor(slots, dtype=torch.int64).to('cuda', non_blocking=True)
            for n in names:
                t = self.out[n].index_select(self.out[n].dim() - 1, s)
                h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
                h.copy_(t, non_blocking=True)
                res[n] = h
        return res

    def idle_handle(self):
        """A handle with no launch in flight, or None."""
        for h in range(len(self.ctx)):
            if not self.busy[h]:
                return h
        return None

    def launch(self, h, slots, gcol, igstep, dt_gl):
        """One column kernel over `slots` on handle h (and its stream)."""
        from .lib import CrmError
        torch = self.torch
        stream = self.streams[h]
        n = len(slots)
        with torch.cuda.stream(stream):
            self.d_map[h][:n].copy_(torch.tensor(slots, dtype=torch.int32), non_blocking=True)
            self.d_gcol[h][:n].copy_(torch.tensor(gcol, dtype=torch.int32), non_blocking=True)
        desc = T.CCrmCallDesc(0, n, self.capacity, float(dt_gl), int(igstep),
                              C.cast(C.c_void_p(self.d_gcol[h].data_ptr()), C.POINTER(C.c_int)),
                              C.cast(C.c_void_p(self.d_map[h].data_ptr()), C.POINTER(C.c_int)))
        lib = self.ctx[h]._lib
        rc = lib.crm_run_device(self.ctx[h]._h, C.byref(desc), C.byref(self.c_in), C.byref(self.c_state),
                                C.byref(self.c_rad), C.byref(self.c_out),
                                C.c_void_p(self.d_status[h].data_ptr()), C.c_void_p(stream.cuda_stream))
        if rc != T.CRM_OK:
            raise CrmError(rc, 'crm_run_device')
        self.busy[h] = True


@dataclass
class Chunk:
    """An admitted GCM chunk: its configuration, slots and global columns."""
    key: tuple
    slots: list
    gcol: list
    nbytes: int
    steps: int = 0


@dataclass
class StepRequest:
    chunk: Chunk
    cin: object
    dt_gl: float
    future: Future = field(default_factory=Future)
    t_submit: float = 0.0


class CrmServer:
    """The service: open_chunk / step / close_chunk; see the module docstring."""

    def __init__(self, configs, capacity=1024, hbm_budget=120 * 2 ** 30, handles=3):
        self.configs = {config_key(c): c for c in configs}
        self.pool_charge = {}
        self.capacity = capacity
        self.budget = HbmBudget(hbm_budget)
        self.handles = handles
        self.pools = {}
        self._q = queue.Queue()
        self._stop = threading.Event()
        self._pending = []
        self.launches = 0
        self.latencies = []
        self._lock = threading.Lock()
        self._thread = threading.Thread(target=self._engine, daemon=True)
        self._thread.start()

    def _handle_bytes(self, cfg):
        from .lib import plan_device_bytes
        return lambda cap: plan_device_bytes(T.CrmConfig(**{**cfg.__dict__, 'max_ncrms': cap}))

    def _release_idle_pools(self, keep):
        """Free the pools (other than `keep`) that hold no chunk."""
        for k in list(self.pools):
            p = self.pools[k]
            if k != keep and p.slots.available == p.capacity and not any(p.busy):
                del self.pools[k]
                self.budget.release(self.pool_charge.pop(k))
                p.close()

    def pool(self, key, need=1):
        """The pool of a configuration, created on first use: charged to the
        budget before it allocates; capacity halves while it does not fit
        (down to `need` slots), else BudgetError."""
        with self._lock:
            p = self.pools.get(key)
            if p is not None:
                return p
            cfg = self.configs[key]
            hb = self._handle_bytes(cfg)
            cap = self.capacity
            for attempt in range(2):
                while cap >= need:
                    nbytes = pool_bytes(cfg, cap, self.handles, hb)
                    if self.budget.reserve(nbytes):
                        p = DevicePool(cfg, cap, self.handles)
                        self.pools[key] = p
                        self.pool_charge[key] = nbytes
                        return p
                    if cap == need:
                        break
                    cap = max(need, cap // 2)
                if attempt == 0:
                    self._release_idle_pools(key)
                    cap = self.capacity
            raise BudgetError('HBM budget: %d of %d bytes in use; a pool of %d slots of this '
                              'configuration does not fit' % (self.budget.used, self.budget.total, need))

    # -- admission
    def open_chunk(self, cfg, cin, st, rad, gcol, timeout=60.0):
        """Admit a chunk: slots + budget, then its state is copied in.
        Waits (up to timeout s) while the pool or the budget is full."""
        key = config_key(cfg)
        n = len(gcol)
        pool = self.pool(key, need=n)
        if n > pool.capacity:
            raise BudgetError('chunk of %d columns exceeds its pool (%d slots)' % (n, pool.capacity))
        nbytes = n * slot_bytes(cfg)
        t0 = time.perf_counter()
        while True:
            slots = pool.slots.alloc(n)
            if slots is not None:
                break
            if time.perf_counter() - t0 > timeout:
                raise TimeoutError('admission timed out')
            time.sleep(0.001)
        stream = pool.streams[0]
        pool.load(slots, cin, st, rad, stream)
        stream.synchronize()
        return Chunk(key, slots, list(gcol), nbytes)

    def chunk_state(self, chunk):
        """A chunk's resident CRM state: (config, CrmState, qrad).  Call
        between steps of that chunk."""
        torch = __import__('torch')
        pool = self.pools[chunk.key]
        stream = pool.streams[0]
        with torch.cuda.stream(stream):
            s = torch.tensor(chunk.slots, dtype=torch.int64).to('cuda')
            host = {n: pool.state[n].index_select(3, s).cpu().numpy().T for n in T.STATE_FIELDS}
            qrad = pool.rad['qrad'].index_select(3, s).cpu().numpy().T
        stream.synchronize()
        st = T.CrmState(**{n: np.asfortranarray(a) for n, a in host.items()})
        cfg = T.CrmConfig(**{**pool.cfg.__dict__, 'max_ncrms': 0})
        return cfg, st, np.asfortranarray(qrad)

    def checkpoint_chunk(self, chunk, path):
        """Write a chunk's resident CRM state (the pbuf restart fields, see
        checkpoint.py) to `path`.  Call between steps of that chunk."""
        from . import checkpoint as CK
        cfg, st, qrad = self.chunk_state(chunk)
        CK.save(path, cfg, st, qrad, chunk.gcol)

    def write_gcm_restart(self, chunk, path, ncol):
        """Write a chunk's resident CRM state as the GCM's restart file holds
        it (CRM_* variables of dimensions (pbuf_NNNNN, ncol), netCDF classic,
        pbuf_restart.write_crm_state); ncol: the physics grid's columns."""
        from . import pbuf_restart as PR
        cfg, st, qrad = self.chunk_state(chunk)
        PR.write_crm_state(path, cfg, ncol, chunk.gcol, st, qrad)

    def restore_chunk(self, path, cin):
        """Admit a chunk from a restart file (its GCM inputs given anew)."""
        from . import checkpoint as CK
        cfg, st, qrad, gcol = CK.load(path)
        rad = T.CrmRad.zeros(len(gcol), cfg.crm_nx_rad, cfg.crm_ny_rad, cfg.crm_nz)
        rad.qrad[...] = qrad
        ch = self.open_chunk(cfg, cin, st, rad, gcol)
        ch.steps = 1          # a restarted chunk is past its first step
        return ch

    def restore_chunk_from_gcm_restart(self, path, cfg, gcol, cin):
        """Admit a chunk of GCM columns gcol (global ids, 1-based) with the
        CRM state the GCM's own restart file holds for them (the CRM_*
        physics-buffer fields, pbuf_restart.read_crm_state); its GCM inputs
        given anew."""
        from . import pbuf_restart as PR
        st, qrad = PR.read_crm_state(path, cfg, gcol)
        rad = T.CrmRad.zeros(len(gcol), cfg.crm_nx_rad or cfg.crm_nx, cfg.crm_ny_rad or cfg.crm_ny, cfg.crm_nz)
        rad.qrad[...] = qrad
        ch = self.open_chunk(cfg, cin, st, rad, gcol)
        ch.steps = 1          # past its first step: no setperturb
        return ch

    def close_chunk(self, chunk):
        self.pools[chunk.key].slots.free(chunk.slots)

    # -- steps
    def step(self, chunk, cin, dt_gl):
        """Submit one GCM step of a chunk (new input profiles); returns a
        Future of ({output name: (n, ...) array}, status array)."""
        r = StepRequest(chunk, cin, dt_gl)
        r.t_submit = time.perf_counter()
        self._q.put(r)
        return r.future

    def close(self):
        self._stop.set()
        self._q.put(None)
        self._thread.join(timeout=30)

    def _engine(self):
        """Continuous batching: requests accumulate per pool while its handles
        are busy; whenever a handle is idle, every request waiting for that
        pool (same dt_gl and first-step flag) goes into one launch on it."""
        import torch
        torch.cuda.set_device(0)
        pending = {}         # pool key -> waiting requests, in arrival order
        inflight = []        # (pool, handle, requests, outputs, status, event)
        busy = set()         # chunks with a step in flight
        while not self._stop.is_set():
            try:
                r = self._q.get(timeout=0.0005 if (inflight or pending) else 0.05)
                while True:
                    if r is not None:
                        pending.setdefault(r.chunk.key, []).append(r)
                    r = self._q.get_nowait()
            except queue.Empty:
                pass
            for key in list(pending):
                pool = self.pools[key]
                while pending.get(key):
                    h = pool.idle_handle()
                    if h is None:
                        break
                    rs, rest = select_launch(pending[key], busy)
                    if not rs:
                        break
                    pending[key] = rest
                    item = self._launch(pool, h, rs, (rs[0].dt_gl, rs[0].chunk.steps == 0))
                    if item is not None:
                        busy.update(id(r.chunk) for r in rs)
                        inflight.append(item)
                if not pending.get(key):
                    pending.pop(key, None)
            still = []
            for item in inflight:
                if item[5].query():
                    self._complete(item)
                    busy.difference_update(id(r.chunk) for r in item[2])
                else:
                    still.append(item)
            inflight = still

    def _launch(self, pool, h, rs, tag):
        import torch
        dt_gl, first = tag
        slots, gcol = [], []
        for r in rs:
            slots += r.chunk.slots
            gcol += r.chunk.gcol
        stream = pool.streams[h]
        # one host->device copy per input field for the whole group
        cat = {n: np.concatenate([getattr(r.cin, n)[:len(r.chunk.slots)] for r in rs], axis=0)
               for n in T.INPUT_FIELDS}
        pool.set_inputs(slots, T.CrmInput(**cat), stream)
        try:
            pool.launch(h, slots, gcol, 1 if first else 2, dt_gl)
        except Exception as e:    # argument errors: fail these requests
            for r in rs:
                r.future.set_exception(e)
            return None
        outs = pool.gather(slots, STEP_OUTPUTS, stream)
        st = torch.empty(len(slots), dtype=torch.int32, pin_memory=True)
        with torch.cuda.stream(stream):
            st.copy_(pool.d_status[h][:len(slots)], non_blocking=True)
        ev = torch.cuda.Event()
        ev.record(stream)
        self.launches += 1
        return (pool, h, rs, outs, st, ev)

    def _complete(self, item):
        pool, h, rs, res, st, ev = item
        pool.busy[h] = False
        status = st.numpy()
        allv = {k: v.numpy().T for k, v in res.items()}    # (N, ...) per field
        o = 0
        t_done = time.perf_counter()
        for r in rs:
            n = len(r.chunk.slots)
            r.chunk.steps += 1
            vals = {k: v[o:o + n].copy() for k, v in allv.items()}
            with self._lock:
                self.latencies.append(t_done - r.t_submit)
            r.future.set_result((vals, status[o:o + n].copy()))
            o += n


def select_launch(waiting, busy):
    """Split the waiting requests of one pool into (this launch, the rest).

    The launch takes the oldest request whose chunk has no step in flight
    and every later one with the same (dt_gl, first-step) tag, at most one
    request per chunk: a chunk's later steps wait for its earlier ones,
    whose results they depend on, and two requests of one chunk in one
    launch would integrate the same slots twice."""
    head = next((r for r in waiting if id(r.chunk) not in busy), None)
    if head is None:
        return [], list(waiting)
    tag = (head.dt_gl, head.chunk.steps == 0)
    take, rest, seen = [], [], set()
    for r in waiting:
        c = id(r.chunk)
        if c not in busy and c not in seen and (r.dt_gl, r.chunk.steps == 0) == tag:
            take.append(r)
            seen.add(c)
        else:
            rest.append(r)
    return take, rest


def apply_tendencies(cin, vals, dt_gl):
    """Advance the GCM columns by the CRM tendencies of a step's results, as
    physics_update does with ptend (gcm_coupling.apply_ptend)."""
    from .gcm_coupling import apply_ptend
    pt = {'s': vals['sltend'], 'q': vals['qltend'], 'qc': vals['qcltend'], 'qi': vals['qiltend']}
    return apply_ptend(cin, pt, dt_gl)
