"""The oracle reproduces its committed fixtures (tests/golden/, written by
tests/golden/make_golden.py): bit for bit on the platform that wrote them,
to 1e-9 relative elsewhere (host libm values enter the FFT tables and the
gamma constants)."""
import os
import platform

import numpy as np
import pytest

from golden import make_golden as G

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


@pytest.mark.parametrize('name', sorted(G.CASES))
def test_oracle_matches_golden(name):
    ref = np.load(os.path.join(HERE, name + '.npz'))
    got = G.run_case(name)
    assert str(got['inputs_sha256']) == str(ref['inputs_sha256']), 'synthetic inputs changed'
    same_platform = str(ref['platform']) == '%s-%s' % (platform.system(), platform.machine())
    for key in ref.files:
        if key in ('platform', 'inputs_sha256'):
            continue
        a, b = got[key], ref[key]
        if same_platform:
            assert np.array_equal(a, b), key
        else:
            scale = np.max(np.abs(b)) or 1.0
            assert np.max(np.abs(a - b)) <= 1e-9 * scale, key


@pytest.mark.parametrize('nlev', [30, 72])
def test_hybrid_coordinate_tables(nlev):
    """vcoord.json holds the reference's hybrid-coordinate tables
    (components/homme/test/vcoord, converted by data/make_vcoord.py): the
    surface interface is pure sigma (hyai = 0, hybi = 1), pressures increase
    monotonically downwards, and the mid levels lie between the interfaces."""
    from crm_gb300 import synthetic as S
    vc = S.vcoord(nlev)
    hyai, hybi, hyam, hybm = vc['hyai'], vc['hybi'], vc['hyam'], vc['hybm']
    assert len(hyai) == nlev + 1 and len(hyam) == nlev
    assert hyai[-1] == 0.0 and hybi[-1] == 1.0
    pint = hyai * vc['p0'] + hybi * 1.0e5
    pmid = hyam * vc['p0'] + hybm * 1.0e5
    assert np.all(np.diff(pint) > 0)
    assert np.all((pmid > pint[:-1]) & (pmid < pint[1:]))
