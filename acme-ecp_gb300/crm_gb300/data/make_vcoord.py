"""Extract the hybrid vertical-coordinate tables the synthetic workloads use.

Reads the E3SM/CAM hybrid coefficient tables that ship with the reference
(components/homme/test/vcoord/acme-72{i,m}.ascii for 72 levels,
cami-30.ascii / camm-30.ascii for 30 levels) and writes them to vcoord.json
beside this script, so that the library and the tests never need the
reference tree at run time.  Run once:

    python make_vcoord.py /path/to/reference
"""
import json
import os
import sys


def _read_table(path):
    """Return the two arrays (a, b) of one vcoord ascii file."""
    toks = open(path).read().split()
    out, i = [], 0
    while i < len(toks):
        n = int(toks[i])
        i += 1
        while toks[i].startswith('!') or not _isnum(toks[i]):
            i += 1
        vals = [float(t) for t in toks[i:i + n]]
        i += n
        out.append(vals)
    return out


def _isnum(t):
    try:
        float(t)
        return True
    except ValueError:
        return False


def main(ref):
    base = os.path.join(ref, 'components', 'homme', 'test', 'vcoord')
    data = {}
    for name, ifile, mfile in (('L72', 'acme-72i.ascii', 'acme-72m.ascii'),
                               ('L30', 'cami-30.ascii', 'camm-30.ascii')):
        hyai, hybi = _read_table(os.path.join(base, ifile))
        hyam, hybm = _read_table(os.path.join(base, mfile))
        assert len(hyai) == len(hybi) == len(hyam) + 1 == len(hybm) + 1
        data[name] = dict(hyai=hyai, hybi=hybi, hyam=hyam, hybm=hybm, p0=1.0e5,
                          source='components/homme/test/vcoord/' + ifile + ', ' + mfile)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'vcoord.json')
    with open(out, 'w') as f:
        json.dump(data, f, indent=1)
    print('wrote', out)


if __name__ == '__main__':
    if len(sys.argv) != 2:
        sys.exit('usage: python make_vcoord.py <reference checkout>')
    main(sys.argv[1])
