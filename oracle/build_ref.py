"""Recipe: the reference's own C source of this path, compiled from where it
lies in the reference checkout into oracle/_ref/ (never committed; built only
where the checkout exists).

  components/cam/src/physics/crm/gammafff.c -> oracle/_ref/libgammafff_ref.so
      gammafff(float *x) = (float)exp(lgamma(*x)), the gamma function the
      sam1mom set-up calls (precip_init.F90, microphysics.F90)

The rest of the path is Fortran and cannot be compiled here (no Fortran
compiler on either machine).  Usage: python oracle/build_ref.py [checkout].
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, '_ref')
GAMMA_SRC = os.path.join('components', 'cam', 'src', 'physics', 'crm', 'gammafff.c')
GAMMA_LIB = os.path.join(OUT, 'libgammafff_ref.so')


def reference_root(root=None):
    root = root or os.environ.get('CRM_REFERENCE_ROOT') or '/root/reference'
    return root if os.path.exists(os.path.join(root, GAMMA_SRC)) else None


def build(root=None):
    """Compile the reference's gammafff.c; returns the library path or None
    when the checkout is absent."""
    root = reference_root(root)
    if root is None:
        return None
    src = os.path.join(root, GAMMA_SRC)
    if os.path.exists(GAMMA_LIB) and os.path.getmtime(GAMMA_LIB) >= os.path.getmtime(src):
        return GAMMA_LIB
    os.makedirs(OUT, exist_ok=True)
    subprocess.check_call(['gcc', '-O2', '-fPIC', '-shared', '-o', GAMMA_LIB, src, '-lm'])
    return GAMMA_LIB


if __name__ == '__main__':
    print(build(sys.argv[1] if len(sys.argv) > 1 else None))
