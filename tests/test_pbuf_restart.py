"""The CRM state in the GCM restart file's layout (pbuf_write_restart:
CRM_* variables of dimensions (pbuf_NNNNN, ncol), netCDF classic): our
reader against files written by scipy's independent netCDF implementation,
scipy against our writer, CDF-5, and a GCM step resumed from a restart file
equal to the step continued in memory (oracle, bit for bit)."""
import numpy as np
import pytest

import oracle
from crm_gb300 import crm_types as T
from crm_gb300 import pbuf_restart as R
from crm_gb300 import synthetic as S

netcdf = pytest.importorskip('scipy.io').netcdf_file


def _state(cfg, n, seed):
    rng = np.random.default_rng(seed)
    st = T.CrmState.zeros(n, cfg.crm_nx, cfg.crm_ny, cfg.crm_nz)
    for name in st.arrays():
        getattr(st, name)[...] = rng.standard_normal(getattr(st, name).shape)
    q = np.asfortranarray(rng.standard_normal((n, cfg.crm_nx_rad, cfg.crm_ny_rad, cfg.crm_nz)))
    return st, q


def _fold(a):
    """(n, nx, ny, nz) -> (nx*ny*nz, n), i fastest, as pbuf_write_restart."""
    n = a.shape[0]
    return a.transpose(0, 3, 2, 1).reshape(n, -1).T


@pytest.mark.parametrize('version', [1, 2])
def test_reads_a_file_written_by_scipy(tmp_path, version):
    cfg = S.config_32x28()
    ncol, gcol = 10, np.array([3, 7, 1, 10])
    st, q = _state(cfg, 4, 1)
    m = cfg.crm_nx * cfg.crm_ny * cfg.crm_nz
    path = str(tmp_path / 'r.nc')
    f = netcdf(path, 'w', version=version)
    f.createDimension('ncol', ncol)
    f.createDimension(R.pbuf_dim_name(m), m)
    for pname, field in R.STATE_FIELDS + (('CRM_QRAD', None),):
        v = f.createVariable(pname, 'd', (R.pbuf_dim_name(m), 'ncol'))
        full = np.zeros((m, ncol))
        full[:, gcol - 1] = _fold(q if field is None else getattr(st, field))
        v[:] = full
    f.close()
    st2, q2 = R.read_crm_state(path, cfg, gcol)
    for name in st.arrays():
        assert np.array_equal(getattr(st2, name), getattr(st, name)), name
    assert np.array_equal(q2, q)


def test_scipy_reads_our_file(tmp_path):
    cfg = S.config_64x58()
    st, q = _state(cfg, 3, 2)
    gcol = np.array([5, 2, 9])
    path = str(tmp_path / 'w.nc')
    R.write_crm_state(path, cfg, 12, gcol, st, q, version=2)
    f = netcdf(path, 'r', mmap=False)
    m = cfg.crm_nx * cfg.crm_nz
    assert f.variables['CRM_T'].dimensions == (R.pbuf_dim_name(m), 'ncol')
    a = f.variables['CRM_T'][:].copy()
    assert np.array_equal(a[:, gcol - 1], _fold(st.temperature))
    assert np.all(np.delete(a, gcol - 1, axis=1) == 0)
    assert np.array_equal(f.variables['CRM_QRAD'][:][:, gcol - 1], _fold(q))
    f.close()


@pytest.mark.parametrize('version', [1, 2, 5])
def test_round_trip_3d_and_formats(tmp_path, version):
    cfg = S.config_3d(nx=16, ny=8, nz=20)
    st, q = _state(cfg, 2, 3)
    path = str(tmp_path / ('v%d.nc' % version))
    R.write_crm_state(path, cfg, 4, [4, 2], st, q, version=version)
    assert R.ClassicFile(path).version == version
    st2, q2 = R.read_crm_state(path, cfg, [4, 2])
    for name in st.arrays():
        assert np.array_equal(getattr(st2, name), getattr(st, name)), name
    assert np.array_equal(q2, q)


def test_refuses_what_it_cannot_map(tmp_path):
    cfg = S.config_32x28()
    st, q = _state(cfg, 1, 4)
    path = str(tmp_path / 'x.nc')
    R.write_crm_state(path, cfg, 3, [2], st, q)
    with pytest.raises(R.NetcdfError):
        R.read_crm_state(path, cfg, [4])                       # column out of range
    with pytest.raises(R.NetcdfError):
        R.read_crm_state(path, S.config_64x58(), [1])           # other CRM size
    (tmp_path / 'bad.nc').write_bytes(b'HDF5....')
    with pytest.raises(R.NetcdfError):
        R.ClassicFile(str(tmp_path / 'bad.nc'))


def test_resume_from_a_restart_file_equals_continuing(tmp_path):
    """Step 1 of 4 columns, their CRM state through a restart file of a
    16-column grid, step 2 from the file equals step 2 from memory."""
    cfg, cin, st, rad, desc = S.workload_32x28(ncrms=4, moist=True)
    desc.dt_gl = 200.0
    gcol = np.array([11, 3, 16, 8])
    rc, _, _ = oracle.run(cfg, desc, cin, st, rad)
    assert rc == 0
    path = str(tmp_path / 'restart.nc')
    R.write_crm_state(path, cfg, 16, gcol, st, rad.qrad)
    st_f, q_f = R.read_crm_state(path, cfg, gcol)
    rad_f = rad.copy()
    rad_f.qrad[...] = q_f
    desc.igstep = 2
    outs = []
    for s_, r_ in ((st.copy(), rad.copy()), (st_f, rad_f)):
        rc, _, out = oracle.run(cfg, desc, cin, s_, r_)
        assert rc == 0
        outs.append((s_, out))
    (a, oa), (b, ob) = outs
    for name in a.arrays():
        assert np.array_equal(getattr(a, name), getattr(b, name)), name
    for name, x in oa.arrays().items():
        assert np.array_equal(x, getattr(ob, name)), name
