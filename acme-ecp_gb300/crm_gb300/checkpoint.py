"""Restart files for resident CRM state.

The reference carries a CRM's state across GCM steps, and across model
restarts, in the physics buffer: the 'global' pbuf fields written to the
restart file (components/cam/src/physics/cam/crm_physics.F90:126-170):

    CRM_U, CRM_V, CRM_W, CRM_T          (pcols, crm_nx, crm_ny, crm_nz)
    CRM_QT, CRM_QP, CRM_QN              (pcols, crm_nx, crm_ny, crm_nz)  sam1mom
    CRM_QRAD                            (pcols, crm_nx_rad, crm_ny_rad, crm_nz)

This module writes exactly those fields, under those names, for any batch of
columns, plus the global column ids and the configuration, so a serving loop
can resume resident columns from a GCM restart and a GCM can read a
checkpoint the serving loop wrote.

File layout (little-endian):
    b'CRMCKPT1\\n'
    one line of JSON: {"config": {...}, "ncols": n, "fields": [{"name", "shape",
                       "dtype", "offset", "nbytes"}, ...]}
    zero padding to a 64-byte boundary, then each field's raw bytes in
    Fortran order (column index fastest), each starting on a 64-byte
    boundary at its recorded offset from the start of the file.
"""
import json
import os

import numpy as np

from . import crm_types as T

MAGIC = b'CRMCKPT1\n'
STATE_NAMES = {'u_wind': 'CRM_U', 'v_wind': 'CRM_V', 'w_wind': 'CRM_W', 'temperature': 'CRM_T',
               'qt': 'CRM_QT', 'qp': 'CRM_QP', 'qn': 'CRM_QN'}
ALIGN = 64


def _pad(n):
    return (n + ALIGN - 1) // ALIGN * ALIGN


def save(path, cfg, state, qrad, gcol):
    """Write the restart fields of len(gcol) columns (state: CrmState with
    ld >= ncols; qrad: (ld, nx_rad, 1, nz))."""
    n = len(gcol)
    arrays = [(pb, np.asfortranarray(getattr(state, f)[:n])) for f, pb in STATE_NAMES.items()]
    arrays.append(('CRM_QRAD', np.asfortranarray(np.asarray(qrad)[:n])))
    arrays.append(('GCOL', np.asfortranarray(np.asarray(gcol, dtype=np.int32))))
    fields = []
    # offsets are fixed after the header size is known: two passes
    for attempt in range(2):
        head = json.dumps({'config': cfg.__dict__, 'ncols': n, 'fields': fields}).encode() + b'\n'
        off = _pad(len(MAGIC) + len(head))
        new = []
        for name, a in arrays:
            new.append({'name': name, 'shape': list(a.shape), 'dtype': a.dtype.str,
                        'offset': off, 'nbytes': int(a.nbytes)})
            off = _pad(off + a.nbytes)
        if new == fields:
            break
        fields = new
    head = json.dumps({'config': cfg.__dict__, 'ncols': n, 'fields': fields}).encode() + b'\n'
    assert _pad(len(MAGIC) + len(head)) == fields[0]['offset']
    tmp = path + '.tmp'
    with open(tmp, 'wb') as f:
        f.write(MAGIC)
        f.write(head)
        for (name, a), d in zip(arrays, fields):
            f.write(b'\0' * (d['offset'] - f.tell()))
            f.write(a.tobytes(order='F'))
    os.replace(tmp, path)


def load(path):
    """(cfg, state, qrad, gcol) from a restart file; state is a CrmState of
    ncols columns, qrad an (ncols, nx_rad, 1, nz) array."""
    with open(path, 'rb') as f:
        if f.read(len(MAGIC)) != MAGIC:
            raise ValueError('%s: not a CRM checkpoint' % path)
        head = json.loads(f.readline())
        out = {}
        for d in head['fields']:
            f.seek(d['offset'])
            buf = f.read(d['nbytes'])
            if len(buf) != d['nbytes']:
                raise ValueError('%s: truncated field %s' % (path, d['name']))
            out[d['name']] = np.frombuffer(buf, dtype=np.dtype(d['dtype'])).reshape(
                d['shape'], order='F').copy(order='F')
    cfg = T.CrmConfig(**head['config'])
    state = T.CrmState(**{f: out[pb] for f, pb in STATE_NAMES.items()})
    return cfg, state, out['CRM_QRAD'], [int(g) for g in out['GCOL']]
