"""Import the unmodified reference spdepy in this container (test infrastructure only).

Used by ``make_golden.py`` to produce the committed fixtures; nothing in the GPU
tests, ``smoke()`` or ``bench.py`` imports this module (the reference tree is not
present on the GPU machine).

Three workarounds make the reference's own code importable here:

1. ``spdepy/__init__.py`` needs installed package metadata plus netCDF4/pandas
   (reference ``src/spdepy/__init__.py:2-3,11``).  A stub ``spdepy`` module whose
   ``__path__`` points at a temporary copy of ``src/spdepy`` bypasses it; the
   submodules (grids, spdes, model, optim) are the reference's own files.
2. The stencil libraries are prebuilt by ``oracle/Makefile`` (the reference's
   runtime ``g++ -shared -W1, lib.so -o lib.so`` fails on g++ 13) and placed in
   the temporary copy's ``spdes/ccode`` so ``setClib`` finds them and does not
   try to compile.
3. CHOLMOD (scikit-sparse 0.4.12, ``poetry.lock:582-589``) is not installed.  A
   ``sksparse.cholmod`` stand-in with the five methods the reference calls
   (``cholesky``, ``logdet``, ``solve_A``, ``solve_Lt``, ``apply_Pt``) uses a dense
   LAPACK Cholesky with the identity permutation, which is exact to rounding for
   the small fixture sizes.
"""
from __future__ import annotations

import os
import shutil
import sys
import tempfile
import types

import numpy as np

# the reference project root: $SPDEPY_REFERENCE, by default where this container mounts it
REF_ROOT = os.environ.get("SPDEPY_REFERENCE", "/root/reference")
REF_SRC = os.path.join(REF_ROOT, "src", "spdepy")
HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF_LIBS = os.path.join(REPO, "oracle", "_ref")

_CHOLMOD_STANDIN = '''
import numpy as np
import scipy.linalg as sla
from scipy import sparse


class CholmodNotPositiveDefiniteError(Exception):
    pass


class Factor:
    def __init__(self, A):
        A = sparse.csc_matrix(A)
        D = A.toarray()
        try:
            self.L = np.linalg.cholesky(D)
        except np.linalg.LinAlgError as e:
            raise CholmodNotPositiveDefiniteError(str(e))

    def logdet(self):
        return 2.0 * np.log(np.diag(self.L)).sum()

    def solve_A(self, b):
        b = b.toarray() if sparse.issparse(b) else np.asarray(b, dtype=float)
        y = sla.solve_triangular(self.L, b, lower=True)
        return sla.solve_triangular(self.L.T, y, lower=False)

    def solve_Lt(self, b, use_LDLt_decomposition=True):
        return sla.solve_triangular(self.L.T, np.asarray(b, dtype=float), lower=False)

    def apply_Pt(self, b):
        return np.asarray(b)


def cholesky(A, *args, **kwargs):
    return Factor(A)
'''


def load_reference():
    """Return the reference ``spdepy`` module tree imported from a temp copy."""
    if "spdepy" in sys.modules and getattr(sys.modules["spdepy"], "_is_ref_stub", False):
        return sys.modules["spdepy"]
    if not os.path.isdir(REF_LIBS) or not os.listdir(REF_LIBS):
        raise RuntimeError("run `make -C oracle` first to build the reference stencils")
    tmp = tempfile.mkdtemp(prefix="spdepy_ref_")
    pkg = os.path.join(tmp, "spdepy")
    shutil.copytree(REF_SRC, pkg)
    for f in os.listdir(REF_LIBS):
        if f.endswith(".so"):
            shutil.copy(os.path.join(REF_LIBS, f), os.path.join(pkg, "spdes", "ccode", f))
    sk = os.path.join(tmp, "sksparse")
    os.makedirs(sk)
    open(os.path.join(sk, "__init__.py"), "w").close()
    with open(os.path.join(sk, "cholmod.py"), "w") as fh:
        fh.write(_CHOLMOD_STANDIN)
    sys.path.insert(0, tmp)
    stub = types.ModuleType("spdepy")
    stub.__path__ = [pkg]
    stub._is_ref_stub = True
    sys.modules["spdepy"] = stub
    import spdepy.grids  # noqa: F401
    import spdepy.spdes  # noqa: F401
    import spdepy.model  # noqa: F401
    stub.grid = spdepy.grids.grid
    stub.spde_init = spdepy.spdes.spde_init
    stub.Model = spdepy.model.Model
    return stub
