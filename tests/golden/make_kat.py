"""Generate tests/golden/kat.json: known answers for single routines of the
reference, computed here in Python from the reference's own source text.

The numbers in kat.json do not come from the oracle.  This script reads the
constants out of the reference files and evaluates the routines with an
independent Python restatement:

  crm/sat.F90      the four 9-coefficient tables (esatw_crm, dtesatw_crm,
                   esati_crm, dtesati_crm) and the Murphy-Koop constants of
                   the cold branch are parsed from the file; the functions
                   are evaluated as the Fortran does with crm_rknd = 8 and
                   REAL*4 literals (constants rounded to float32, arithmetic
                   in double), the cold branch with Python's exp/log;
  cam/RNG_MT.F90   the generator's parameters (N, M, MATA, UMASK, LMASK,
                   TMASKB, TMASKC) and the seeding multiplier are parsed from
                   the file; the state update, tempering and the (0,1)
                   mapping follow RNG_MT_set_seed / RNG_MT_gen_rand, in
                   Python integers with explicit 32-bit wrap-around.

  crm/gammafff.c   compiled from the reference checkout itself
                   (oracle/build_ref.py) and called: the gamma function of the
                   sam1mom set-up at its ten arguments and on a sweep.

Run once, with the reference checkout as argument:

    python tests/golden/make_kat.py <reference checkout>
"""
import json
import math
import os
import re
import sys

import numpy as np

CRM = os.path.join('components', 'cam', 'src', 'physics', 'crm')
CAM = os.path.join('components', 'cam', 'src', 'physics', 'cam')


def r4(x):
    """A REAL*4 literal widened to double."""
    return float(np.float32(x))


def parse_sat(path):
    src = open(path).read()
    funcs = {}
    for m in re.finditer(r'function\s+(\w+)_crm\s*\(t\)(.*?)end\s*\n', src, re.S | re.I):
        name, body = m.group(1).lower(), m.group(2)
        d = re.search(r'data\s+a0\s*,.*?/\s*&?(.*?)/', body, re.S | re.I)
        if not d:
            continue
        nums = re.findall(r'[-+]?\d*\.\d+(?:[eEdD][-+]?\d+)?', d.group(1))
        funcs[name] = [float(x.replace('d', 'e').replace('D', 'e')) for x in nums]
        assert len(funcs[name]) == 9, (name, nums)
    cold = re.search(r'esatw_crm\s*=\s*([\d.]+)\s*\*\s*([\d.]+)\s*\*\s*exp\(\s*([\d.]+)\s*-\s*([\d.]+)/t\s*\+\s*'
                     r'([\d.]+)\*Log\(t\)\s*-\s*([\d.]+)\*t\)', src, re.I)
    cold_i = re.search(r'esati_crm\s*=\s*([\d.]+)\s*\*\s*exp\(', src, re.I)
    assert cold and cold_i
    return funcs, [float(x) for x in cold.groups()], float(cold_i.group(1))


def sat_functions(funcs, cold, cold_i):
    fw2, fw1, c0, c1, c2, c3 = cold
    t_ref = r4(273.16)

    def poly(a, t):
        a = [r4(x) for x in a]
        dt = t - t_ref
        return a[0] + dt * (a[1] + dt * (a[2] + dt * (a[3] + dt * (a[4] + dt * (a[5] + dt * (a[6] + dt * (a[7] + a[8] * dt)))))))

    def mk(t):
        return math.exp(((r4(c0) - r4(c1) / t) + r4(c2) * math.log(t)) - r4(c3) * t)

    def esatw(t):
        if t - t_ref > -80.:
            return poly(funcs['esatw'], t)
        return float(np.float32(np.float32(fw2) * np.float32(fw1))) * mk(t)

    def esati(t):
        if t - t_ref > -80.:
            return poly(funcs['esati'], t)
        return r4(cold_i) * mk(t)

    def dtesatw(t):
        if t - t_ref > -80.:
            return poly(funcs['dtesatw'], t)
        return esatw(t + 1.0) - esatw(t)

    def dtesati(t):
        if t - t_ref > -80.:
            return poly(funcs['dtesati'], t)
        return esati(t + 1.0) - esati(t)

    def qsat(es, p):
        return (r4(0.622) * es) / (p - es if p - es > es else es)

    return {
        'esatw': lambda t, p: esatw(t), 'esati': lambda t, p: esati(t),
        'dtesatw': lambda t, p: dtesatw(t), 'dtesati': lambda t, p: dtesati(t),
        'qsatw': lambda t, p: qsat(esatw(t), p), 'qsati': lambda t, p: qsat(esati(t), p),
        'dtqsatw': lambda t, p: (r4(0.622) * dtesatw(t)) / p,
        'dtqsati': lambda t, p: (r4(0.622) * dtesati(t)) / p,
    }


def parse_rng(path):
    src = open(path).read()
    par = {}
    for name in ('N', 'M', 'MATA', 'UMASK', 'LMASK', 'TMASKB', 'TMASKC'):
        m = re.search(r'parameter\s*::\s*%s\s*=\s*(-?\d+)' % name, src)
        par[name] = int(m.group(1))
    m = re.search(r'mt\(mti\)\s*=\s*iand\(\s*(\d+)\s*\*\s*mt\(mti\s*-\s*1\)', src)
    par['SEEDMUL'] = int(m.group(1))
    return par


def rng_draws(par, seed, n):
    """RNG_MT_set_seed(seed) then n calls of RNG_MT_gen_rand."""
    M32 = 0xFFFFFFFF
    N, M = par['N'], par['M']
    u = lambda x: x & M32
    s = lambda x: x - (1 << 32) if x & 0x80000000 else x
    mt = [0] * N
    mt[0] = u(seed)
    for i in range(1, N):
        mt[i] = u(par['SEEDMUL'] * mt[i - 1])
    mti = N
    um, lm, mata = u(par['UMASK']), u(par['LMASK']), u(par['MATA'])
    tb, tc = u(par['TMASKB']), u(par['TMASKC'])
    mag = (0, mata)
    out = []
    for _ in range(n):
        if mti >= N:
            for kk in range(N):
                y = (mt[kk] & um) | (mt[(kk + 1) % N] & lm)
                mt[kk] = mt[(kk + M) % N] ^ (y >> 1) ^ mag[y & 1]
            mti = 0
        y = mt[mti]
        mti += 1
        y ^= y >> 11
        y ^= (y << 7) & tb
        y ^= (y << 15) & tc
        y ^= y >> 18
        y = u(y)
        ys = s(y)
        out.append((ys + 2.0 ** 32) / 2.0 ** 32 if ys < 0 else (ys + 0.5) / 2.0 ** 32)
    return out


def gamma_values(ref):
    """gammafff(x) of the reference's compiled gammafff.c: the ten arguments
    of precip_init.F90 / microphysics.F90 (3 + b, (5 + b) / 2, 4 + b for
    rain, snow, graupel, and 3) and a sweep of 0.5..12."""
    import ctypes as C
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))),
                                    'oracle'))
    import build_ref
    lib = C.CDLL(build_ref.build(ref))
    f = lib.gammafff
    f.restype = C.c_float
    f.argtypes = [C.POINTER(C.c_float)]
    b = {'rain': r4(0.8), 'snow': 0.25, 'grau': 0.5}
    xs = [3.0]
    for v in b.values():
        xs += [3.0 + v, (5.0 + v) / 2.0, 4.0 + v]
    xs = [float(np.float32(x)) for x in xs] + [float(x) for x in np.linspace(0.5, 12.0, 47, dtype=np.float32)]
    return {'x': xs, 'value': [float(f(C.byref(C.c_float(x)))) for x in xs]}


def main(ref):
    funcs, cold, cold_i = parse_sat(os.path.join(ref, CRM, 'sat.F90'))
    f = sat_functions(funcs, cold, cold_i)
    temps = [float(x) for x in np.round(np.linspace(160.0, 320.0, 81), 6)] + [193.16, 193.17, 273.16]
    press = [float(1000.0 - 4.0 * i) for i in range(len(temps))]
    sat = {name: [fn(t, p) for t, p in zip(temps, press)] for name, fn in f.items()}
    par = parse_rng(os.path.join(ref, CAM, 'RNG_MT.F90'))
    seeds = [1000, 17000, 1024000, 12345000]
    rng = {str(sd): rng_draws(par, sd, 700) for sd in seeds}
    data = {'source': {'sat': 'components/cam/src/physics/crm/sat.F90',
                       'rng': 'components/cam/src/physics/cam/RNG_MT.F90',
                       'gammafff': 'components/cam/src/physics/crm/gammafff.c (compiled, gcc, glibc libm)'},
            'sat_t': temps, 'sat_p': press, 'sat': sat, 'sat_coefficients': funcs,
            'rng_parameters': par, 'rng': rng, 'gammafff': gamma_values(ref)}
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'kat.json')
    with open(out, 'w') as fh:
        json.dump(data, fh, indent=0)
    print('wrote', out)


if __name__ == '__main__':
    if len(sys.argv) != 2:
        sys.exit('usage: python make_kat.py <reference checkout>')
    main(sys.argv[1])
