"""Compile the reference vegas Cython module out of tree into ``oracle/_ref/``.

TEST INFRASTRUCTURE ONLY: the compiled reference is used in the development
container to check the oracle restatement and to generate the golden vectors
under ``tests/golden/``.  It is never imported by the product package, and it
does not travel to the GPU host (the reference sources are not there).

Recipe (nothing is written into the reference tree):

1. copy ``src/vegas/_vegas.pyx`` and ``_vegas.pxd`` from the reference into a
   temporary directory laid out as package ``vegas``;
2. apply a 4-line compile fix: Cython 3.3 rejects memoryview slices held
   across a ``yield`` in ``Integrator._random_batch`` (_vegas.pyx:1753-1758,
   "C struct/union member cannot be a memory view").  The four yielded slices
   are wrapped in ``numpy.asarray(...)``; no arithmetic changes;
3. cythonize + compile with gcc through setuptools, then copy the extension
   and an empty ``vegas/__init__.py`` into ``oracle/_ref/vegas/``.

The reference's pure-Python ``vegas/__init__.py`` (restratify, PDFIntegrator
etc.) is not compiled; ``import_reference_package`` loads it straight from the
reference tree on top of the compiled module when a golden generator needs
``restratify``.  ``gvar`` (not installed) is replaced by ``oracle/gvar_stub``.

The reference tree is taken from ``--reference``, else from the environment
variable ``VEGAS_REFERENCE``, else from a directory named ``reference`` beside
this repository's root (``default_reference()``).

Usage:  python oracle/build_ref.py [--reference DIR]
"""
import argparse
import glob
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, '_ref', 'vegas')


def default_reference():
    """The reference tree: $VEGAS_REFERENCE, else ``reference`` beside the repository root."""
    env = os.environ.get('VEGAS_REFERENCE')
    if env:
        return env
    return os.path.join(os.path.dirname(os.path.dirname(HERE)), 'reference')

PATCHES = [
    ("answer = (x[:neval_batch, :],)", "answer = (numpy.asarray(x[:neval_batch, :]),)"),
    ("answer += (y[:neval_batch, :],)", "answer += (numpy.asarray(y[:neval_batch, :]),)"),
    ("answer += (jac[:neval_batch],)", "answer += (numpy.asarray(jac[:neval_batch]),)"),
    ("answer += (hcube_array[:neval_batch],)", "answer += (numpy.asarray(hcube_array[:neval_batch]),)"),
]

SETUP = r'''
from setuptools import setup, Extension
from Cython.Build import cythonize
setup(ext_modules=cythonize([Extension("vegas._vegas", ["vegas/_vegas.pyx"])],
                            language_level=3, quiet=True))
'''


def built():
    return bool(glob.glob(os.path.join(OUT, '_vegas*.so')))


def build(reference=None, force=False):
    if built() and not force:
        return OUT
    reference = reference or default_reference()
    src = os.path.join(reference, 'src', 'vegas')
    if not os.path.isdir(src):
        raise FileNotFoundError('reference sources not found at %s' % src)
    tmp = tempfile.mkdtemp(prefix='vegas_ref_build_')
    try:
        pkg = os.path.join(tmp, 'vegas')
        os.makedirs(pkg)
        with open(os.path.join(src, '_vegas.pyx')) as f:
            text = f.read()
        for old, new in PATCHES:
            if text.count(old) != 1:
                raise RuntimeError('patch anchor not found exactly once: %r' % old)
            text = text.replace(old, new)
        with open(os.path.join(pkg, '_vegas.pyx'), 'w') as f:
            f.write(text)
        shutil.copy(os.path.join(src, '_vegas.pxd'), os.path.join(pkg, '_vegas.pxd'))
        open(os.path.join(pkg, '__init__.py'), 'w').close()
        with open(os.path.join(tmp, 'setup.py'), 'w') as f:
            f.write(SETUP)
        subprocess.run([sys.executable, 'setup.py', 'build_ext', '--inplace'],
                       cwd=tmp, check=True, stdout=subprocess.DEVNULL)
        os.makedirs(OUT, exist_ok=True)
        for so in glob.glob(os.path.join(pkg, '_vegas*.so')):
            shutil.copy(so, OUT)
        open(os.path.join(OUT, '__init__.py'), 'w').close()
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    return OUT


def import_reference():
    """Import the compiled reference module ``vegas._vegas`` with the gvar stand-in."""
    for p in (os.path.join(HERE, 'gvar_stub'), os.path.join(HERE, '_ref')):
        if p not in sys.path:
            sys.path.insert(0, p)
    from vegas import _vegas  # noqa: E402
    return _vegas


def import_reference_package(reference=None):
    """The reference package ``vegas`` (src/vegas/__init__.py, read from the
    reference tree) with ``vegas._vegas`` resolved to the compiled module."""
    import importlib.util
    reference = reference or default_reference()
    stub = os.path.join(HERE, 'gvar_stub')
    if stub not in sys.path:
        sys.path.insert(0, stub)
    spec = importlib.util.spec_from_file_location(
        'vegas', os.path.join(reference, 'src', 'vegas', '__init__.py'),
        submodule_search_locations=[OUT])
    mod = importlib.util.module_from_spec(spec)
    sys.modules['vegas'] = mod
    spec.loader.exec_module(mod)
    return mod


if __name__ == '__main__':
    ap = argparse.ArgumentParser()
    ap.add_argument('--reference', default=None)
    ap.add_argument('--force', action='store_true')
    a = ap.parse_args()
    print(build(a.reference, a.force))
