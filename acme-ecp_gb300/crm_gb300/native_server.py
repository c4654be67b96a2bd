"""ctypes wrapper of the C-ABI serving entry points (crm_server_create,
crm_chunk_open / read_state / close, crm_submit, crm_poll in
include/crm_gb300.h): the same continuous-batching service a C or Fortran
GCM host calls, driven from Python with the numpy bundles of crm_types.

The engine, the resident slot pools and the batching live in the library
(csrc/crm_serve.cu); this module only marshals arrays.  Arrays handed to
submit() are kept alive by the returned Ticket until poll() reports it.
"""
import ctypes as C

import numpy as np

from . import crm_types as T
from .lib import CrmError, load


class Ticket:
    """A submitted step: poll() it; its result arrays live here."""

    def __init__(self, server, tid, out, rad, status, keep):
        self.server, self.id, self.out, self.rad, self.status = server, tid, out, rad, status
        self._keep = keep
        self.rc = None

    def poll(self, wait=True):
        """None while pending, else the step's worst column status."""
        if self.rc is None:
            rc = self.server._lib.crm_poll(self.server._h, self.id, 1 if wait else 0)
            if rc == T.CRM_PENDING:
                return None
            self.rc = rc
            self._keep = None
        return self.rc


class NativeCrmServer:
    """One configuration's resident-slot pool and engine (crm_server)."""

    def __init__(self, cfg, capacity=256, handles=3, hbm_budget=120 * 2 ** 30):
        self._lib = load()
        self.cfg = cfg
        st = C.c_int(0)
        self._c_cfg = cfg.to_c()
        h = self._lib.crm_server_create(C.byref(self._c_cfg), int(capacity), int(handles),
                                        C.c_ulonglong(int(hbm_budget)), C.byref(st))
        if not h:
            raise CrmError(st.value, 'crm_server_create')
        self._h = h

    def close(self):
        if getattr(self, '_h', None):
            self._lib.crm_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def device_bytes(self):
        return int(self._lib.crm_server_device_bytes(self._h))

    @property
    def launches(self):
        return int(self._lib.crm_server_launches(self._h))

    def open_chunk(self, st, rad, gcol):
        """Admit the columns of a CrmState/CrmRad bundle; returns the chunk id."""
        n = len(gcol)
        g = np.ascontiguousarray(gcol, dtype=np.int32)
        cid = C.c_int(-1)
        c_st, c_rad = st.to_c(), rad.to_c()
        rc = self._lib.crm_chunk_open(self._h, n, g.ctypes.data_as(C.POINTER(C.c_int)), st.u_wind.shape[0],
                                      C.byref(c_st), C.byref(c_rad), C.byref(cid))
        if rc != T.CRM_OK:
            raise CrmError(rc, 'crm_chunk_open')
        return cid.value

    def read_state(self, chunk, n):
        """The chunk's resident CRM state and heating (a CrmState, qrad)."""
        cfg = self.cfg
        st = T.CrmState.zeros(n, cfg.crm_nx, cfg.crm_ny, cfg.crm_nz)
        nxr = cfg.crm_nx_rad or cfg.crm_nx
        qrad = np.zeros((n, nxr, cfg.crm_ny_rad or 1, cfg.crm_nz), order='F')
        c_st = st.to_c()
        rc = self._lib.crm_chunk_read_state(self._h, chunk, n, C.byref(c_st),
                                            qrad.ctypes.data_as(C.POINTER(C.c_double)))
        if rc != T.CRM_OK:
            raise CrmError(rc, 'crm_chunk_read_state')
        return st, qrad

    def close_chunk(self, chunk):
        rc = self._lib.crm_chunk_close(self._h, chunk)
        if rc != T.CRM_OK:
            raise CrmError(rc, 'crm_chunk_close')

    def submit(self, chunk, cin, n, dt_gl, fields=None, qrad=None, rad_means=False):
        """Submit one GCM step of a chunk of n columns (cin: CrmInput with
        at least n columns).  fields: crm_output names to return (None: all);
        rad_means: also return the crm_rad means.  Returns a Ticket."""
        cfg = self.cfg
        out = T.CrmOutput(n, cfg.crm_nx, cfg.crm_ny, cfg.crm_nz, cfg.plev)
        c_out = out.to_c()
        if fields is not None:
            for i, (name, _) in enumerate(T.OUTPUT_FIELDS):
                if name not in fields:
                    c_out.field[i] = C.cast(None, C.POINTER(C.c_double))
        rad = None
        c_rad = None
        if rad_means:
            rad = T.CrmRad.zeros(n, cfg.crm_nx_rad or cfg.crm_nx, cfg.crm_ny_rad or 1, cfg.crm_nz)
            c_rad = rad.to_c()
        status = np.zeros(n, dtype=np.int32)
        ld = cin.tl.shape[0]
        c_in = cin.to_c()
        q = None
        if qrad is not None:
            q = np.asfortranarray(qrad, dtype=np.float64)
        tid = C.c_longlong(0)
        rc = self._lib.crm_submit(self._h, chunk, C.byref(c_in),
                                  None if q is None else q.ctypes.data_as(C.POINTER(C.c_double)),
                                  ld, float(dt_gl), C.byref(c_out), None if c_rad is None else C.byref(c_rad),
                                  status.ctypes.data_as(C.POINTER(C.c_int)), C.byref(tid))
        if rc != T.CRM_OK:
            raise CrmError(rc, 'crm_submit')
        return Ticket(self, tid.value, out, rad, status, (c_out, c_rad, c_in, cin, q, status))
