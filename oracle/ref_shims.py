"""Oracle test infrastructure: import the reference's own Python under import shims.

This module is only used on the development machine that holds a read-only
checkout of RigidMultiblobsWall; it is never imported by the product and never
runs on a GPU machine.  It exists to generate the golden fixtures under
``tests/golden/`` from the reference's own FP64 functions.

The reference does not import as-is on Python 3.12 / scipy 1.18.  The shims
below are installed in ``sys.modules`` only (nothing is written into the
reference tree):

* ``imp`` (removed in Python 3.12; used by ``mobility/mobility.py:7``) - a stub
  whose ``find_module`` raises ImportError for pycuda and succeeds for numba;
* ``numba`` - ``njit`` becomes the identity decorator and ``prange`` is
  ``range``, so ``mobility/mobility_numba.py`` runs as plain IEEE Python
  (no fastmath);
* ``visit.visit_writer_interface`` (unbuilt native module);
* ``scipy.sparse.linalg._isolve._iterative`` and ``scipy._lib._util._aligned_zeros``
  (private scipy names imported by ``quaternion_integrator/gmres.py:6-10``);
* ``scipy.sparse.linalg.gmres`` accepting the old ``tol=`` keyword
  (``general_application_utils.py:598,627``) mapped to ``rtol=`` with
  ``atol=0`` and ``callback_type='legacy'``.
"""
import importlib
import os
import sys
import types

# The checkout is named by the environment (RMW_REFERENCE_ROOT); without it the
# reference counts as absent and nothing here imports it.
REFERENCE_ROOT = os.environ.get("RMW_REFERENCE_ROOT", "")


def reference_available():
    if not REFERENCE_ROOT:
        return False
    return os.path.isfile(os.path.join(REFERENCE_ROOT, "mobility", "mobility_numba.py"))


def _install_shims():
    if getattr(_install_shims, "done", False):
        return
    # imp: find_module('pycuda') must fail, find_module('numba') must succeed.
    imp = types.ModuleType("imp")

    def find_module(name, *args, **kwargs):
        if name == "numba":
            return (None, "numba", None)
        raise ImportError(name)

    imp.find_module = find_module
    sys.modules["imp"] = imp

    numba = types.ModuleType("numba")

    def njit(*args, **kwargs):
        if len(args) == 1 and callable(args[0]) and not kwargs:
            return args[0]
        return lambda f: f

    numba.njit = njit
    numba.jit = njit
    numba.prange = range
    sys.modules["numba"] = numba

    visit = types.ModuleType("visit")
    vwi = types.ModuleType("visit.visit_writer_interface")
    visit.visit_writer_interface = vwi
    sys.modules.setdefault("visit", visit)
    sys.modules["visit.visit_writer_interface"] = vwi

    import scipy._lib._util as su
    import numpy as np
    if not hasattr(su, "_aligned_zeros"):
        su._aligned_zeros = lambda shape, dtype=float, order="C", align=None: np.zeros(shape, dtype=dtype, order=order)
    sys.modules.setdefault("scipy.sparse.linalg._isolve._iterative",
                           types.ModuleType("scipy.sparse.linalg._isolve._iterative"))

    import scipy.sparse.linalg as spla
    orig_gmres = spla.gmres
    if not getattr(orig_gmres, "_rmw_shim", False):
        def gmres(A, b, x0=None, tol=None, restart=None, maxiter=None, M=None,
                  callback=None, atol=0.0, rtol=1e-5, callback_type=None, **kw):
            if tol is not None:
                rtol = tol
            if callback is not None and callback_type is None:
                callback_type = "legacy"
            return orig_gmres(A, b, x0=x0, rtol=rtol, atol=atol, restart=restart,
                              maxiter=maxiter, M=M, callback=callback,
                              callback_type=callback_type)
        gmres._rmw_shim = True
        spla.gmres = gmres
    _install_shims.done = True


def _prepare():
    if not reference_available():
        raise RuntimeError("reference checkout not found: set RMW_REFERENCE_ROOT to a RigidMultiblobsWall "
                           "checkout (found %r)" % REFERENCE_ROOT)
    # The reference tree is read-only: never write bytecode caches into it.
    sys.dont_write_bytecode = True
    _install_shims()
    if REFERENCE_ROOT not in sys.path:
        sys.path.insert(0, REFERENCE_ROOT)
    p = os.path.join(REFERENCE_ROOT, "multi_bodies")
    if p not in sys.path:
        sys.path.append(p)


def load(module_path):
    """Import a reference package module (e.g. 'mobility.mobility') under the shims."""
    _prepare()
    return importlib.import_module(module_path)


def load_script(relpath, name):
    """Import a reference script file (e.g. 'multi_bodies/multi_bodies.py') as module `name`."""
    _prepare()
    if name in sys.modules:
        return sys.modules[name]
    import importlib.util
    spec = importlib.util.spec_from_file_location(name, os.path.join(REFERENCE_ROOT, relpath))
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod
