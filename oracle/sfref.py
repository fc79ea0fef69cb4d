"""Loader for the reference Strawberry Fields code -- TEST INFRASTRUCTURE ONLY.

The reference (a pure-Python package) imports several modules that are absent
here and on the GPU host: ``numba`` (two ``@jit`` loops in
``fockbackend/circuit.py:307-365``), ``thewalrus`` (gate matrices,
``fockbackend/ops.py:30-36``), ``blackbird``/``xir``/``xcc`` (IO and remote
API), ``toml``, ``dateutil``, ``plotly`` and, on some hosts, ``networkx`` and
``sympy``.  This loader puts a meta-path finder in front of the import system
that turns each missing module into a permissive stub, makes ``numba.jit`` an
identity decorator (the jitted loops then run as plain numpy), and serves
``thewalrus.fock_gradients`` from the oracle's FP64 restatement in
``oracle/fock_oracle.py`` -- in thewalrus's own index order
``[out1, out2, in1, in2]`` so the reference's transposes at
``fockbackend/ops.py:269,329,343`` still apply.

Two entry points:

* :func:`load_fock_circuit` loads only ``fockbackend/ops.py`` and
  ``fockbackend/circuit.py`` as a private package (needs numpy and scipy);
  this is the reference CPU implementation timed by ``bench.py --impl
  reference`` and the generator of ``tests/golden``.
* :func:`import_strawberryfields` imports the whole package (frontend,
  ``sf.Engine``) for end-to-end tests of the drop-in backend.
"""

import importlib.abc
import importlib.machinery
import importlib.util
import os
import sys
import types

import numpy as np

from . import fock_oracle as fo

_HERE = os.path.dirname(os.path.abspath(__file__))
_REPO = os.path.dirname(_HERE)


def find_reference():
    """Return the directory holding the ``strawberryfields`` package of the
    reference: ``$SF_REFERENCE_ROOT`` when set, else the offline install under
    ``baseline/_ref``; ``None`` when neither holds it."""
    cands = [os.path.join(_REPO, "baseline", "_ref")]
    env = os.environ.get("SF_REFERENCE_ROOT")
    if env:
        cands.insert(0, env)
    for c in cands:
        if os.path.isfile(os.path.join(c, "strawberryfields", "backends", "fockbackend", "circuit.py")):
            return c
    return None


# ---------------------------------------------------------------------------
# thewalrus.fock_gradients restated (thewalrus index order for 2-mode gates)
# ---------------------------------------------------------------------------

def _tw_displacement(r, phi, cutoff, dtype=np.complex128):
    return fo.displacement(float(r), float(phi), int(cutoff)).astype(dtype)


def _tw_squeezing(r, theta, cutoff, dtype=np.complex128):
    return fo.squeezing(float(r), float(theta), int(cutoff)).astype(dtype)


def _tw_beamsplitter(theta, phi, cutoff, dtype=np.complex128):
    return fo.beamsplitter(float(theta), float(phi), int(cutoff)).transpose(0, 2, 1, 3).astype(dtype)


def _tw_two_mode_squeezing(r, theta, cutoff, dtype=np.complex128):
    return fo.two_mode_squeeze(float(r), float(theta), int(cutoff)).transpose(0, 2, 1, 3).astype(dtype)


def _tw_mzgate(theta, phi, cutoff, dtype=np.complex128):
    return fo.mzgate(float(theta), float(phi), int(cutoff)).transpose(0, 2, 1, 3).astype(dtype)


def _make_fock_gradients():
    m = types.ModuleType("thewalrus.fock_gradients")
    m.displacement = _tw_displacement
    m.squeezing = _tw_squeezing
    m.beamsplitter = _tw_beamsplitter
    m.two_mode_squeezing = _tw_two_mode_squeezing
    m.mzgate = _tw_mzgate

    def _unavailable(*a, **k):
        raise NotImplementedError("thewalrus gradient builders are not restated")

    for name in ("grad_displacement", "grad_squeezing", "grad_beamsplitter",
                 "grad_two_mode_squeezing", "grad_mzgate"):
        setattr(m, name, _unavailable)
    return m


def _make_symplectic():
    """``thewalrus.symplectic`` helpers the reference's state tests import
    (published definitions: a phase-space rotation by theta, the symplectic
    form, and the reordering between (x1, p1, x2, p2, ...) and
    (x1, x2, ..., p1, p2, ...) phase-space orderings)."""
    m = types.ModuleType("thewalrus.symplectic")

    def rotation(theta):
        c, s = np.cos(theta), np.sin(theta)
        return np.array([[c, -s], [s, c]])

    def sympmat(n):
        z, i = np.zeros((n, n)), np.identity(n)
        return np.block([[z, i], [-i, z]])

    def _xxpp_order(n2):
        return np.concatenate([np.arange(0, n2, 2), np.arange(1, n2, 2)])

    def xpxp_to_xxpp(S):
        S = np.asarray(S)
        ind = _xxpp_order(S.shape[0])
        return S[ind] if S.ndim == 1 else S[ind][:, ind]

    def xxpp_to_xpxp(S):
        S = np.asarray(S)
        ind = np.argsort(_xxpp_order(S.shape[0]))
        return S[ind] if S.ndim == 1 else S[ind][:, ind]

    m.rotation, m.sympmat, m.xpxp_to_xxpp, m.xxpp_to_xpxp = rotation, sympmat, xpxp_to_xxpp, xxpp_to_xpxp
    return m


# ---------------------------------------------------------------------------
# permissive stubs for absent modules
# ---------------------------------------------------------------------------

class _StubMeta(type):
    """Metaclass of stub classes: attribute access yields further stub classes."""

    def __getattr__(cls, name):
        if name.startswith("__") and name.endswith("__"):
            raise AttributeError(name)
        return _stub_class(name)

    def __getitem__(cls, k):
        return _stub_class("item")

    def __iter__(cls):
        return iter(())


class _Anything(metaclass=_StubMeta):
    """Stand-in for any attribute of a stubbed module: a class (so isinstance
    and subclassing work) whose instances accept any call or attribute."""

    def __init__(self, *a, **k):
        pass

    def __call__(self, *a, **k):
        return _Anything()

    def __getattr__(self, name):
        if name.startswith("__") and name.endswith("__"):
            raise AttributeError(name)
        return _Anything()

    def __getitem__(self, k):
        return _Anything()

    def __iter__(self):
        return iter(())


def _stub_class(name):
    return _StubMeta(str(name), (_Anything,), {})


def _identity_jit(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]
    return lambda f: f


class _StubModule(types.ModuleType):
    def __getattr__(self, name):
        if name.startswith("__") and name.endswith("__"):
            raise AttributeError(name)
        if self.__name__.split(".")[0] == "numba" and name in ("jit", "njit", "vectorize", "guvectorize"):
            return _identity_jit
        return _stub_class(name)


class _StubFinder(importlib.abc.MetaPathFinder, importlib.abc.Loader):
    def __init__(self, roots):
        self.roots = set(roots)

    def find_spec(self, fullname, path=None, target=None):
        if fullname.split(".")[0] in self.roots:
            return importlib.machinery.ModuleSpec(fullname, self, is_package=True)
        return None

    def create_module(self, spec):
        if spec.name == "thewalrus.fock_gradients":
            return _make_fock_gradients()
        if spec.name == "thewalrus.symplectic":
            return _make_symplectic()
        mod = _StubModule(spec.name)
        mod.__path__ = []
        return mod

    def exec_module(self, module):
        if module.__name__ == "numba":
            module.jit = _identity_jit
            module.njit = _identity_jit
        if module.__name__ == "thewalrus":
            module.__version__ = "0.22.0"


_ALWAYS_STUB = ("numba", "thewalrus", "blackbird", "xcc", "xir", "toml", "dateutil", "plotly",
                "quantum_blackbird")
_STUB_IF_MISSING = ("networkx", "sympy", "tensorflow_probability")


def _install_stubs():
    roots = list(_ALWAYS_STUB)
    for name in _STUB_IF_MISSING:
        if importlib.util.find_spec(name) is None:
            roots.append(name)
    for f in sys.meta_path:
        if isinstance(f, _StubFinder):
            f.roots |= set(roots)
            return
    sys.meta_path.insert(0, _StubFinder(roots))


# ---------------------------------------------------------------------------
# entry points
# ---------------------------------------------------------------------------

_FOCK_PKG = "_sfref_fockbackend"


def load_fock_circuit(ref_root=None):
    """Load the reference's ``fockbackend/ops.py`` and ``fockbackend/circuit.py``
    as package ``_sfref_fockbackend``; return ``(ops_module, Circuit)``."""
    if _FOCK_PKG + ".circuit" in sys.modules:
        mod = sys.modules[_FOCK_PKG + ".circuit"]
        return sys.modules[_FOCK_PKG + ".ops"], mod.Circuit
    ref_root = ref_root or find_reference()
    if ref_root is None:
        raise ImportError("reference strawberryfields sources not found")
    _install_stubs()
    fdir = os.path.join(ref_root, "strawberryfields", "backends", "fockbackend")
    pkg = types.ModuleType(_FOCK_PKG)
    pkg.__path__ = [fdir]
    sys.modules[_FOCK_PKG] = pkg
    mods = {}
    for name in ("ops", "circuit"):
        spec = importlib.util.spec_from_file_location(f"{_FOCK_PKG}.{name}", os.path.join(fdir, f"{name}.py"))
        mod = importlib.util.module_from_spec(spec)
        sys.modules[spec.name] = mod
        spec.loader.exec_module(mod)
        mods[name] = mod
    return mods["ops"], mods["circuit"].Circuit


def import_strawberryfields(ref_root=None):
    """Import the full reference package (with stubs for absent modules) and
    return the ``strawberryfields`` module."""
    if "strawberryfields" in sys.modules:
        return sys.modules["strawberryfields"]
    ref_root = ref_root or find_reference()
    if ref_root is None:
        raise ImportError("reference strawberryfields sources not found")
    _install_stubs()
    if ref_root not in sys.path:
        sys.path.insert(0, ref_root)
    import strawberryfields  # noqa: E402

    return strawberryfields
