"""The C ABI library without a GPU: it loads, exports every function that
include/crm_gb300.h declares, and fails loudly (a status, no fallback) when
no CUDA device is present."""
import ctypes as C
import os
import re

import pytest

from conftest import has_gpu
from crm_gb300 import build
from crm_gb300 import crm_types as T
from crm_gb300 import lib as L
from crm_gb300 import synthetic as S

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(REPO, 'include', 'crm_gb300.h')).read()
    src = re.sub(r'/\*.*?\*/', '', src, flags=re.S)
    names = re.findall(r'^[A-Za-z_][\w \*]*?\b(crm_\w+)\s*\(', src, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope='module')
def lib():
    build.build()
    return L.load()


def test_header_declares_the_bound_functions():
    assert set(header_functions()) == set(L.EXPORTS)


def test_library_exports_every_declared_symbol(lib):
    for name in header_functions():
        assert hasattr(lib, name), name


def test_status_strings_and_version(lib):
    for s in range(10):
        assert lib.crm_status_string(s).decode() not in ('', 'unknown status'), s
    assert lib.crm_status_string(99).decode() == 'unknown status'
    assert b'sm_103a' in lib.crm_version()


def test_struct_sizes_match_the_header():
    # pointers and ints as the header lays them out (LP64)
    assert C.sizeof(T.CCrmOutput) == C.sizeof(C.c_void_p) * len(T.OUTPUT_FIELDS)
    assert C.sizeof(T.CCrmInput) == C.sizeof(C.c_void_p) * len(T.INPUT_FIELDS)
    assert C.sizeof(T.CCrmState) == C.sizeof(C.c_void_p) * 7
    assert C.sizeof(T.CCrmConfig) == 6 * 4 + 3 * 8 + 4 * 4 + 8 + 8 + 8


@pytest.mark.skipif(has_gpu(), reason='checks the no-device path')
def test_create_without_device_fails_loudly(lib):
    cfg = S.config_32x28()
    cfg.max_ncrms = 4
    st = C.c_int(-1)
    h = lib.crm_create(C.byref(cfg.to_c()), C.byref(st))
    assert not h
    assert st.value == T.CRM_ERR_NO_DEVICE
    with pytest.raises(L.CrmError):
        L.CrmContext(cfg)


def test_invalid_configurations_are_rejected(lib):
    for kw in ({'crm_nx': 14}, {'crm_nx': 7}, {'plev': 20}, {'crm_dt': 40.0}, {'crm_ny': 4}):
        cfg = S.config_32x28()
        cfg.max_ncrms = 4
        for k, v in kw.items():
            setattr(cfg, k, v)
        st = C.c_int(-1)
        h = lib.crm_create(C.byref(cfg.to_c()), C.byref(st))
        assert not h
        assert st.value in (T.CRM_ERR_ARG, T.CRM_ERR_UNSUPPORTED), kw
    # not built: 3D transform lengths with a factor 3 or 5, 3D radiation
    # groups coarser than the CRM grid, the two-moment microphysics
    for kw in ({'crm_ny': 12, 'crm_ny_rad': 12}, {'crm_ny': 16, 'crm_ny_rad': 8},
               {'microphysics': T.CRM_MICRO_M2005}):
        cfg = S.config_32x28()
        cfg.max_ncrms = 4
        for k, v in kw.items():
            setattr(cfg, k, v)
        st = C.c_int(-1)
        assert not lib.crm_create(C.byref(cfg.to_c()), C.byref(st))
        assert st.value == T.CRM_ERR_UNSUPPORTED, kw


def test_noalloc_rejects_oversize_before_touching_the_device(lib):
    # set-up values of 100000 columns (257 MB) or crm_nx 2048 exceed the fixed
    # 32 MiB scratch of crm_run_device_noalloc; the check needs no GPU
    cfg = S.config_64x58()
    d = T.CCrmCallDesc(0, 100000, 100000, 100.0, 2, None)
    rc = lib.crm_run_device_noalloc(C.byref(cfg.to_c()), C.byref(d), C.byref(T.CCrmInput()),
                                    C.byref(T.CCrmState()), C.byref(T.CCrmRad()),
                                    C.byref(T.CCrmOutput()), None, None)
    assert rc == T.CRM_ERR_TOO_LARGE
    d = T.CCrmCallDesc(0, 1, 1, 100.0, 2, None)
    rc = lib.crm_run_device_noalloc(C.byref(S.config_64x58(nx=2048).to_c()), C.byref(d),
                                    C.byref(T.CCrmInput()), C.byref(T.CCrmState()),
                                    C.byref(T.CCrmRad()), C.byref(T.CCrmOutput()), None, None)
    assert rc == T.CRM_ERR_TOO_LARGE


def _c_struct_fields(name):
    src = open(os.path.join(REPO, 'include', 'crm_gb300.h')).read()
    src = re.sub(r'/\*.*?\*/', '', src, flags=re.S)
    body = re.search(r'typedef struct %s \{(.*?)\} %s;' % (name, name), src, flags=re.S).group(1)
    fields = []
    for decl in body.split(';'):
        decl = decl.strip()
        if not decl:
            continue
        decl = re.sub(r'^(const\s+)?(int|double|unsigned)\s*', '', decl)
        fields += [f.strip().lstrip('*').strip() for f in decl.split(',')]
    return fields


def _fortran_type_fields(doc, name):
    body = re.search(r'type, bind\(C\) :: %s\n(.*?)\n\s*end type' % name, doc, flags=re.S).group(1)
    body = body.replace('&\n', ' ')
    fields = []
    for line in body.splitlines():
        line = line.split('!')[0]
        if '::' in line:
            fields += [f.strip() for f in line.split('::')[1].split(',') if f.strip()]
    return fields


def test_integration_fortran_binding_mirrors_the_header():
    """The bind(C) types of the Fortran binding module declare the same
    components, in the same order, as the C header."""
    doc = open(os.path.join(REPO, 'include', 'crm_gb300_bind.F90')).read()
    for c_name, f_name in (('crm_config', 'crm_config_c'), ('crm_call_desc', 'crm_call_desc_c'),
                           ('crm_input_c', 'crm_input_c'), ('crm_state_c', 'crm_state_c'),
                           ('crm_rad_c', 'crm_rad_c')):
        assert _fortran_type_fields(doc, f_name) == _c_struct_fields(c_name), c_name
    n = int(re.search(r'field\((\d+)\)', doc).group(1))
    assert n == len(T.OUTPUT_FIELDS)


def test_fortran_binding_interfaces_are_exported(lib):
    """Every bind(C, name=...) interface of the Fortran module names a
    function the header declares and the library exports, with as many
    arguments as the C prototype."""
    doc = open(os.path.join(REPO, 'include', 'crm_gb300_bind.F90')).read()
    hdr = re.sub(r'/\*.*?\*/', '', open(os.path.join(REPO, 'include', 'crm_gb300.h')).read(), flags=re.S)
    names = re.findall(r"(?:function|subroutine)[ \t]+(\w+)[ \t]*\(([^)]*)\)[^\n]*(?:&\s*\n[^\n]*)?bind\(C, name='(\w+)'\)",
                       doc)
    assert {n for _, _, n in names} >= {'crm_create', 'crm_run', 'crm_destroy', 'crm_server_create',
                                       'crm_submit', 'crm_poll', 'crm_chunk_open', 'crm_chunk_close'}
    for fname, args, cname in names:
        assert fname == cname
        assert hasattr(lib, cname), cname
        proto = re.search(r'\b%s\s*\(([^)]*)\)\s*;' % cname, hdr)
        assert proto, cname
        n_c = len([a for a in proto.group(1).split(',') if a.strip() and a.strip() != 'void'])
        n_f = len([a for a in args.split(',') if a.strip()])
        assert n_c == n_f, (cname, n_c, n_f)


def test_launch_shape_table(lib):
    """The shape table the autotuner walks is readable without a device:
    whole warps, at most 1024 threads, register budgets that fit an SM
    (at most 2048 threads per SM), and an
    out-of-range index refused."""
    from crm_gb300.autotune import shapes
    table = shapes()
    assert len(table) == lib.crm_num_launch_shapes() >= 5
    for s, threads, ctas, planes in table:
        assert threads % 32 == 0 and 32 <= threads <= 1024, s
        assert 1 <= ctas and threads * ctas <= 2048, s
        assert planes in (0, 2), s
    t, c, m = C.c_int(), C.c_int(), C.c_int()
    assert lib.crm_launch_shape_info(len(table), C.byref(t), C.byref(c), C.byref(m)) != 0
