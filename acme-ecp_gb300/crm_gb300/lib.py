"""ctypes binding of libcrm_gb300.so (include/crm_gb300.h).

This is the binding a Python host would add; a Fortran host binds the same
symbols through iso_c_binding.  There is no CPU fallback: if the library or
a CUDA device is missing, CrmContext raises.
"""
import ctypes as C
import os

import numpy as np

from . import crm_types as T

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, 'libcrm_gb300.so')

EXPORTS = ('crm_create', 'crm_destroy', 'crm_run', 'crm_run_device', 'crm_last_launch_count',
           'crm_last_kernel_ms', 'crm_set_stream', 'crm_status_string', 'crm_version',
           'crm_debug_phase_cycles', 'crm_run_device_noalloc', 'crm_num_launch_shapes',
           'crm_launch_shape_info', 'crm_set_launch_shape', 'crm_get_launch_shape',
           'crm_device_bytes', 'crm_plan_device_bytes', 'crm_debug_barrier_test',
           'crm_server_create', 'crm_server_destroy', 'crm_server_device_bytes', 'crm_server_launches',
           'crm_chunk_open', 'crm_chunk_read_state', 'crm_chunk_close', 'crm_submit', 'crm_poll',
           'crm_debug_tc_transform')

_lib = None


class CrmError(RuntimeError):
    def __init__(self, status, what=''):
        self.status = status
        super().__init__('%s: %s (status %d)' % (what or 'crm', status_string(status), status))


def load(path=None, build_if_missing=False):
    """Load the library (optionally building it first)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        if not build_if_missing:
            raise OSError('libcrm_gb300.so not built: run crm_gb300.build.build()')
        from . import build as B
        path = B.build()
    lib = C.CDLL(path)
    lib.crm_create.restype = C.c_void_p
    lib.crm_create.argtypes = [C.POINTER(T.CCrmConfig), C.POINTER(C.c_int)]
    lib.crm_destroy.restype = None
    lib.crm_destroy.argtypes = [C.c_void_p]
    lib.crm_run.restype = C.c_int
    lib.crm_run.argtypes = [C.c_void_p, C.POINTER(T.CCrmCallDesc), C.POINTER(T.CCrmInput),
                            C.POINTER(T.CCrmState), C.POINTER(T.CCrmRad), C.POINTER(T.CCrmOutput),
                            C.POINTER(C.c_int)]
    lib.crm_run_device.restype = C.c_int
    lib.crm_run_device.argtypes = [C.c_void_p, C.POINTER(T.CCrmCallDesc), C.POINTER(T.CCrmInput),
                                   C.POINTER(T.CCrmState), C.POINTER(T.CCrmRad),
                                   C.POINTER(T.CCrmOutput), C.c_void_p, C.c_void_p]
    lib.crm_run_device_noalloc.restype = C.c_int
    lib.crm_run_device_noalloc.argtypes = [C.POINTER(T.CCrmConfig), C.POINTER(T.CCrmCallDesc),
                                           C.POINTER(T.CCrmInput), C.POINTER(T.CCrmState),
                                           C.POINTER(T.CCrmRad), C.POINTER(T.CCrmOutput),
                                           C.c_void_p, C.c_void_p]
    lib.crm_last_launch_count.restype = C.c_int
    lib.crm_last_launch_count.argtypes = [C.c_void_p]
    lib.crm_last_kernel_ms.restype = C.c_double
    lib.crm_last_kernel_ms.argtypes = [C.c_void_p]
    lib.crm_set_stream.restype = C.c_int
    lib.crm_set_stream.argtypes = [C.c_void_p, C.c_void_p]
    lib.crm_status_string.restype = C.c_char_p
    lib.crm_status_string.argtypes = [C.c_int]
    lib.crm_version.restype = C.c_char_p
    lib.crm_version.argtypes = []
    lib.crm_num_launch_shapes.restype = C.c_int
    lib.crm_num_launch_shapes.argtypes = []
    lib.crm_launch_shape_info.restype = C.c_int
    lib.crm_launch_shape_info.argtypes = [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
    lib.crm_set_launch_shape.restype = C.c_int
    lib.crm_set_launch_shape.argtypes = [C.c_void_p, C.c_int]
    lib.crm_get_launch_shape.restype = C.c_int
    lib.crm_get_launch_shape.argtypes = [C.c_void_p]
    lib.crm_server_create.restype = C.c_void_p
    lib.crm_server_create.argtypes = [C.POINTER(T.CCrmConfig), C.c_int, C.c_int, C.c_ulonglong,
                                      C.POINTER(C.c_int)]
    lib.crm_server_destroy.restype = None
    lib.crm_server_destroy.argtypes = [C.c_void_p]
    lib.crm_server_device_bytes.restype = C.c_ulonglong
    lib.crm_server_device_bytes.argtypes = [C.c_void_p]
    lib.crm_server_launches.restype = C.c_longlong
    lib.crm_server_launches.argtypes = [C.c_void_p]
    lib.crm_chunk_open.restype = C.c_int
    lib.crm_chunk_open.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.c_int,
                                   C.POINTER(T.CCrmState), C.POINTER(T.CCrmRad), C.POINTER(C.c_int)]
    lib.crm_chunk_read_state.restype = C.c_int
    lib.crm_chunk_read_state.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(T.CCrmState),
                                         C.POINTER(C.c_double)]
    lib.crm_chunk_close.restype = C.c_int
    lib.crm_chunk_close.argtypes = [C.c_void_p, C.c_int]
    lib.crm_submit.restype = C.c_int
    lib.crm_submit.argtypes = [C.c_void_p, C.c_int, C.POINTER(T.CCrmInput), C.POINTER(C.c_double),
                               C.c_int, C.c_double, C.POINTER(T.CCrmOutput), C.POINTER(T.CCrmRad),
                               C.POINTER(C.c_int), C.POINTER(C.c_longlong)]
    lib.crm_poll.restype = C.c_int
    lib.crm_poll.argtypes = [C.c_void_p, C.c_longlong, C.c_int]
    lib.crm_debug_barrier_test.restype = C.c_int
    lib.crm_debug_barrier_test.argtypes = [C.c_void_p, C.c_longlong, C.c_int]
    lib.crm_device_bytes.restype = C.c_ulonglong
    lib.crm_device_bytes.argtypes = [C.c_void_p]
    lib.crm_plan_device_bytes.restype = C.c_int
    lib.crm_plan_device_bytes.argtypes = [C.POINTER(T.CCrmConfig), C.POINTER(C.c_ulonglong)]
    lib.crm_debug_tc_transform.restype = C.c_int
    lib.crm_debug_tc_transform.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float)]
    lib.crm_debug_phase_cycles.restype = C.c_int
    lib.crm_debug_phase_cycles.argtypes = [C.c_void_p, C.POINTER(C.c_ulonglong), C.c_int]
    _lib = lib
    return lib


def status_string(s):
    try:
        return load().crm_status_string(int(s)).decode()
    except OSError:
        return 'status %d' % s


def plan_device_bytes(cfg):
    """Device bytes crm_create would allocate for cfg (nothing allocated)."""
    lib = load()
    n = C.c_ulonglong(0)
    c_cfg = cfg.to_c()
    rc = lib.crm_plan_device_bytes(C.byref(c_cfg), C.byref(n))
    if rc != T.CRM_OK:
        raise CrmError(rc, 'crm_plan_device_bytes')
    return int(n.value)


def run_device_noalloc(cfg, dev, stream=0):
    """crm_run_device_noalloc on a DeviceCrmArrays bundle: no handle and no
    device allocation (the library's fixed 32 MiB scratch is used instead).
    Asynchronous; returns the crm_status of the call (argument and size
    checks; CRM_ERR_TOO_LARGE when the call does not fit the scratch)."""
    lib = load()
    c_cfg = cfg.to_c()
    return lib.crm_run_device_noalloc(C.byref(c_cfg), C.byref(dev.c_desc), C.byref(dev.c_in),
                                      C.byref(dev.c_state), C.byref(dev.c_rad), C.byref(dev.c_out),
                                      C.c_void_p(dev.status_ptr), C.c_void_p(stream))


class CrmContext:
    """One configured handle (crm_create / crm_run / crm_destroy)."""

    def __init__(self, cfg: T.CrmConfig):
        lib = load()
        self.cfg = cfg
        st = C.c_int(0)
        self._c_cfg = cfg.to_c()
        h = lib.crm_create(C.byref(self._c_cfg), C.byref(st))
        if not h:
            raise CrmError(st.value, 'crm_create')
        self._h = h
        self._lib = lib

    def close(self):
        if getattr(self, '_h', None):
            self._lib.crm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_ptr):
        return self._lib.crm_set_stream(self._h, C.c_void_p(stream_ptr))

    def run(self, desc, cin, state, rad, out, raise_on_error=False):
        """crm_run on host arrays; returns the per-column status array."""
        status = np.zeros(desc.ncrms, dtype=np.int32)
        c_in, c_st, c_rad, c_out = cin.to_c(), state.to_c(), rad.to_c(), out.to_c()
        rc = self._lib.crm_run(self._h, C.byref(desc), C.byref(c_in), C.byref(c_st),
                               C.byref(c_rad), C.byref(c_out),
                               status.ctypes.data_as(C.POINTER(C.c_int)))
        self.last_rc = rc
        if raise_on_error and rc != T.CRM_OK:
            raise CrmError(rc, 'crm_run')
        return status

    def run_device(self, dev, stream=0):
        """crm_run_device on a DeviceCrmArrays bundle (asynchronous)."""
        rc = self._lib.crm_run_device(self._h, C.byref(dev.c_desc), C.byref(dev.c_in),
                                      C.byref(dev.c_state), C.byref(dev.c_rad),
                                      C.byref(dev.c_out), C.c_void_p(dev.status_ptr),
                                      C.c_void_p(stream))
        if rc != T.CRM_OK:
            raise CrmError(rc, 'crm_run_device')

    @property
    def launch_shape(self):
        return self._lib.crm_get_launch_shape(self._h)

    def set_launch_shape(self, shape):
        """Select a launch shape (-1: default); returns the crm_status."""
        return self._lib.crm_set_launch_shape(self._h, int(shape))

    def phase_cycles(self, n=64):
        """Per-phase cycle counters of a profiling build (None otherwise)."""
        buf = (C.c_ulonglong * n)()
        m = self._lib.crm_debug_phase_cycles(self._h, buf, n)
        return None if m < 0 else [int(buf[i]) for i in range(m)]

    @property
    def device_bytes(self):
        """Device memory this handle holds [bytes]."""
        return int(self._lib.crm_device_bytes(self._h))

    @property
    def last_kernel_ms(self):
        return self._lib.crm_last_kernel_ms(self._h)

    @property
    def last_launch_count(self):
        return self._lib.crm_last_launch_count(self._h)
