"""The CRM state in the GCM's own restart file: reader and writer.

The reference keeps each GCM column's CRM state in 'global' physics-buffer
fields between GCM steps (cam/crm_physics.F90:126-191: CRM_U, CRM_V, CRM_W,
CRM_T of shape (pcols, crm_nx, crm_ny, crm_nz), CRM_QRAD of shape (pcols,
crm_nx_rad, crm_ny_rad, crm_nz) and, for sam1mom, CRM_QT, CRM_QP, CRM_QN) and
writes them to the restart file in pbuf_write_restart
(cam/physics_buffer.F90.in:1336-1371, 1440-1457): every non-column dimension
of a field is folded into one dimension named pbuf_NNNNN (NNNNN = their
product, five digits, pbuf_init_restart :1300-1320), so on the file a field
is the variable of the pbuf name with dimensions (ncol, pbuf_NNNNN) in
Fortran order -- netCDF dimensions (pbuf_NNNNN, ncol) -- on the physics
grid's unstructured column dimension, or (lon, lat, pbuf_NNNNN) on a
rectangular grid; the folded index is (i - 1) + nx ((j - 1) + ny (k - 1)).

This module reads and writes that layout in the netCDF classic format
(CDF-1, CDF-2 with 64-bit offsets, CDF-5 with 64-bit sizes; the formats PIO
writes restart files in), with numpy only, so that a serving chunk can be
resumed from a GCM restart and a chunk's state written back into one.
Column ids are the GCM's global column numbers (1-based), as gcol.
"""
import struct

import numpy as np

from . import crm_types as T

# (pbuf name, crm_state_c component) of the sam1mom build
STATE_FIELDS = (('CRM_U', 'u_wind'), ('CRM_V', 'v_wind'), ('CRM_W', 'w_wind'), ('CRM_T', 'temperature'),
                ('CRM_QT', 'qt'), ('CRM_QP', 'qp'), ('CRM_QN', 'qn'))

_NC_DIMENSION, _NC_VARIABLE, _NC_ATTRIBUTE = 10, 11, 12
_TYPES = {1: ('i1', 1), 2: ('S1', 1), 3: ('>i2', 2), 4: ('>i4', 4), 5: ('>f4', 4), 6: ('>f8', 8),
          7: ('u1', 1), 8: ('>u2', 2), 9: ('>u4', 4), 10: ('>i8', 8), 11: ('>u8', 8)}
_CODES = {np.dtype('>f8'): 6, np.dtype('>f4'): 5, np.dtype('>i4'): 4, np.dtype('>i8'): 10}


class NetcdfError(ValueError):
    pass


def pbuf_dim_name(n):
    """The folded dimension of pbuf_init_restart ('pbuf_', i5.5)."""
    return 'pbuf_%05d' % n


class ClassicFile:
    """A netCDF classic-format file opened for reading: dims, variables
    (name -> (dim names, numpy dtype, begin offset, shape)), read(name)."""

    def __init__(self, path):
        self.path = path
        with open(path, 'rb') as f:
            self._buf = f.read()
        b = self._buf
        if b[:3] != b'CDF' or b[3] not in (1, 2, 5):
            raise NetcdfError('%s: not a netCDF classic file' % path)
        self.version = b[3]
        self._off = 4
        self._wide = self.version == 5          # 64-bit counts and sizes
        self.numrecs = self._nonneg()
        self.dims = []                          # [(name, length)] in file order
        tag, n = self._tag()
        if tag == _NC_DIMENSION:
            for _ in range(n):
                name = self._name()
                self.dims.append((name, self._nonneg()))
        self.attrs = self._attrs()
        self.variables = {}
        tag, n = self._tag()
        if tag == _NC_VARIABLE:
            for _ in range(n):
                name = self._name()
                nd = self._nonneg()
                dimids = [self._nonneg() for _ in range(nd)]
                vattrs = self._attrs()
                code = self._int(4)
                self._nonneg()                  # vsize
                begin = self._int(8 if self.version != 1 else 4)
                if code not in _TYPES:
                    raise NetcdfError('variable %s: unknown type %d' % (name, code))
                dnames = [self.dims[d][0] for d in dimids]
                shape = tuple(self.dims[d][1] for d in dimids)
                self.variables[name] = (dnames, np.dtype(_TYPES[code][0]), begin, shape, vattrs)

    def _int(self, size):
        v = int.from_bytes(self._buf[self._off:self._off + size], 'big', signed=False)
        self._off += size
        return v

    def _nonneg(self):
        return self._int(8 if self._wide else 4)

    def _tag(self):
        return self._int(4), self._nonneg()

    def _name(self):
        n = self._nonneg()
        s = self._buf[self._off:self._off + n].decode('utf-8')
        self._off += (n + 3) // 4 * 4
        return s

    def _attrs(self):
        out = {}
        tag, n = self._tag()
        if tag == _NC_ATTRIBUTE:
            for _ in range(n):
                name = self._name()
                code = self._int(4)
                cnt = self._nonneg()
                dt, size = _TYPES[code]
                raw = self._buf[self._off:self._off + cnt * size]
                self._off += (cnt * size + 3) // 4 * 4
                out[name] = raw.decode('utf-8', 'replace') if code == 2 else np.frombuffer(raw, dtype=dt)
        return out

    def read(self, name):
        """The variable's values (C order of its netCDF dimensions)."""
        if name not in self.variables:
            raise KeyError(name)
        dnames, dt, begin, shape, _ = self.variables[name]
        if any(s == 0 for s in shape[:1]) and self.numrecs:
            raise NetcdfError('%s: record variables are not read here' % name)
        n = int(np.prod(shape)) if shape else 1
        a = np.frombuffer(self._buf, dtype=dt, count=n, offset=begin)
        return a.reshape(shape).astype(dt.newbyteorder('='))


def _column_axis(f, name):
    dnames, _, _, shape, _ = f.variables[name]
    pb = [i for i, d in enumerate(dnames) if d.startswith('pbuf_')]
    return dnames, shape, pb


def read_crm_state(path, cfg, gcol):
    """The CRM state of GCM columns gcol (global ids, 1-based) from a restart
    file: (CrmState (len(gcol), nx, ny, nz), qrad (len(gcol), nx_rad, ny_rad,
    nz)).  Unstructured (ncol) and rectangular (lon, lat) physics grids are
    read; on a rectangular grid gcol numbers the columns lon fastest."""
    f = ClassicFile(path)
    nx, ny, nz = cfg.crm_nx, cfg.crm_ny, cfg.crm_nz
    nxr, nyr = cfg.crm_nx_rad or nx, cfg.crm_ny_rad or ny
    g = np.asarray(gcol, dtype=np.int64) - 1
    n = g.size
    st = T.CrmState.zeros(n, nx, ny, nz)

    def columns(name, m):
        if name not in f.variables:
            raise NetcdfError('%s: no variable %s' % (path, name))
        dnames, shape, pb = _column_axis(f, name)
        if len(pb) != 1 or shape[pb[0]] != m:
            raise NetcdfError('%s: %s has dimensions %s, expected %s' % (path, name, dnames, pbuf_dim_name(m)))
        a = f.read(name)
        if pb[0] != 0:
            raise NetcdfError('%s: %s: the folded dimension is not the slowest' % (path, name))
        a = a.reshape(m, -1)                    # (pbuf, columns), columns lon fastest
        if g.size and (g.min() < 0 or g.max() >= a.shape[1]):
            raise NetcdfError('%s: column id out of range 1..%d' % (path, a.shape[1]))
        return a[:, g].T                        # (n, m)

    for pname, field in STATE_FIELDS:
        v = columns(pname, nx * ny * nz)
        getattr(st, field)[...] = v.reshape(n, nz, ny, nx).transpose(0, 3, 2, 1)
    q = columns('CRM_QRAD', nxr * nyr * nz).reshape(n, nz, nyr, nxr).transpose(0, 3, 2, 1)
    return st, np.asfortranarray(q)


def write_crm_state(path, cfg, ncol, gcol, st, qrad, version=2):
    """Write the CRM_* restart variables of columns gcol (1-based ids on an
    unstructured grid of ncol columns; other columns zero) in the layout of
    pbuf_write_restart, netCDF classic (version 1, 2 or 5)."""
    nx, ny, nz = cfg.crm_nx, cfg.crm_ny, cfg.crm_nz
    nxr, nyr = cfg.crm_nx_rad or nx, cfg.crm_ny_rad or ny
    g = np.asarray(gcol, dtype=np.int64) - 1
    n = g.size
    m_st, m_rad = nx * ny * nz, nxr * nyr * nz
    dims = [('ncol', ncol), (pbuf_dim_name(m_st), m_st)]
    if m_rad != m_st:
        dims.append((pbuf_dim_name(m_rad), m_rad))
    did = {d: i for i, (d, _) in enumerate(dims)}
    vars_ = []
    for pname, field in STATE_FIELDS:
        a = np.zeros((m_st, ncol))
        a[:, g] = np.asarray(getattr(st, field))[:n].transpose(0, 3, 2, 1).reshape(n, m_st).T
        vars_.append((pname, [did[pbuf_dim_name(m_st)], did['ncol']], a))
    a = np.zeros((m_rad, ncol))
    a[:, g] = np.asarray(qrad)[:n].transpose(0, 3, 2, 1).reshape(n, m_rad).T
    vars_.append(('CRM_QRAD', [did[pbuf_dim_name(m_rad)], did['ncol']], a))
    vars_.append(('pbuf_time_idx', [], np.array(1, dtype='>i4')))
    _write_classic(path, dims, vars_, version)


def _write_classic(path, dims, variables, version):
    wide = version == 5
    off_size = 4 if version == 1 else 8

    def nonneg(v):
        return struct.pack('>Q' if wide else '>I', v)

    def name(s):
        b = s.encode('utf-8')
        return nonneg(len(b)) + b + b'\0' * ((-len(b)) % 4)

    data = [np.ascontiguousarray(a, dtype=np.dtype('>f8') if a.dtype.kind == 'f' else a.dtype.newbyteorder('>'))
            for _, _, a in variables]

    def header(begins):
        h = b'CDF' + bytes([version]) + nonneg(0)
        h += struct.pack('>I', _NC_DIMENSION) + nonneg(len(dims)) + b''.join(name(d) + nonneg(n) for d, n in dims)
        h += struct.pack('>I', 0) + nonneg(0)                      # no global attributes
        h += struct.pack('>I', _NC_VARIABLE) + nonneg(len(variables))
        for (vname, dids, _), a, b in zip(variables, data, begins):
            vsize = (a.nbytes + 3) // 4 * 4
            h += name(vname) + nonneg(len(dids)) + b''.join(nonneg(d) for d in dids)
            h += struct.pack('>I', 0) + nonneg(0)                  # no variable attributes
            h += struct.pack('>I', _CODES[a.dtype]) + nonneg(min(vsize, 0xFFFFFFFF) if not wide else vsize)
            h += struct.pack('>Q' if off_size == 8 else '>I', b)
        return h

    hlen = len(header([0] * len(variables)))
    begins, pos = [], hlen
    for a in data:
        begins.append(pos)
        pos += (a.nbytes + 3) // 4 * 4
    if off_size == 4 and pos >= 2 ** 31:
        raise NetcdfError('file too large for CDF-1; use version 2 or 5')
    with open(path, 'wb') as fh:
        fh.write(header(begins))
        for a in data:
            b = a.tobytes()
            fh.write(b + b'\0' * ((-len(b)) % 4))
