"""Fixtures for running the reference's ``tests/backend`` files against the
GB300 backend (installed as ``conftest.py`` beside the staged files by
``tests/refsuite/stage.py``).

It provides the fixtures of the reference's ``tests/conftest.py`` that the
backend tests use -- ``tol``, ``cutoff``, ``alpha``, ``hbar``, ``pure``,
``batch_size``, ``setup_backend``, ``setup_backend_pars``, ``setup_eng`` --
with the same defaults (TOL 1e-3, CUTOFF 6, ALPHA 0.1, HBAR 1.7; conftest.py
:64-71) and the same backend selection by marks (``pytest_runtest_setup``,
conftest.py:215-245), but with one backend: ``fock_gb300``, marked ``fock``
so every test written for the reference's Fock backend runs on it.

``FOCK_REFSUITE_BACKEND=fock`` puts the reference's own ``FockBackend`` in
its place (a check of this shim that needs no GPU).
"""
import os
import sys

import pytest

_REPO = os.environ.get("FOCK_GB300_REPO") or os.path.dirname(
    os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))
if _REPO not in sys.path:
    sys.path.insert(0, _REPO)

from oracle import sfref  # noqa: E402  (loads the reference with stubs for its absent dependencies)

sf = sfref.import_strawberryfields()

from strawberryfields.engine import LocalEngine  # noqa: E402
from strawberryfields.program import Program  # noqa: E402

BACKEND = os.environ.get("FOCK_REFSUITE_BACKEND", "fock_gb300")


def _backend_class():
    if BACKEND == "fock":
        from strawberryfields.backends.fockbackend import FockBackend

        return FockBackend
    from strawberryfields_gb300 import sf_backend

    return type(sf_backend())


TOL = 1e-3
CUTOFF = 6
ALPHA = 0.1
HBAR = 1.7


@pytest.fixture(scope="session")
def tol():
    return float(os.environ.get("TOL", TOL))


@pytest.fixture(scope="session")
def cutoff():
    return int(os.environ.get("CUTOFF", CUTOFF))


@pytest.fixture(scope="session")
def alpha():
    return float(os.environ.get("ALPHA", ALPHA))


@pytest.fixture(scope="session")
def hbar():
    sf.hbar = float(os.environ.get("HBAR", HBAR))
    return sf.hbar


@pytest.fixture(params=[pytest.param(True, marks=pytest.mark.pure), pytest.param(False, marks=pytest.mark.mixed)])
def pure(request):
    return request.param


@pytest.fixture(scope="session")
def batch_size():
    """None, or ``BATCHSIZE`` from the environment (as in the reference's
    conftest.py:100-114): the backend then runs with its batch_size option."""
    return int(os.environ["BATCHSIZE"]) if "BATCHSIZE" in os.environ else None


@pytest.fixture(params=[pytest.param(BACKEND, marks=pytest.mark.fock)])
def setup_backend(request, cutoff, pure, batch_size):
    cls = _backend_class()

    def _setup_backend(num_subsystems):
        backend = cls()
        backend.begin_circuit(num_subsystems=num_subsystems, cutoff_dim=cutoff, pure=pure, batch_size=batch_size)
        return backend

    return _setup_backend


@pytest.fixture(params=[pytest.param(BACKEND, marks=pytest.mark.fock)])
def setup_backend_pars(request, cutoff, pure, batch_size):
    backend = "fock" if BACKEND == "fock" else _backend_class()()
    return backend, {"cutoff_dim": cutoff, "pure": pure, "batch_size": batch_size}


@pytest.fixture
def setup_eng(setup_backend_pars):
    def _setup_eng(num_subsystems, **kwargs):
        prog = Program(num_subsystems)
        backend, options = setup_backend_pars
        options = dict(options, **kwargs)
        return LocalEngine(backend=backend, backend_options=options), prog

    return _setup_eng


def pytest_runtest_setup(item):
    marks = {m.name for m in item.iter_markers() if m.name in ("fock", "gaussian", "bosonic", "tf")}
    wanted = [m.args for m in item.iter_markers(name="backends")]
    allowed = set(wanted[0]) if wanted else {"fock", "gaussian", "bosonic", "tf"}
    for b in marks:
        if b not in allowed:
            pytest.skip(f"test runs with {sorted(allowed)} backends only")
    for m in item.iter_markers(name="broken"):
        pytest.skip("broken test skipped: {}".format(m.args[0] if m.args else ""))
