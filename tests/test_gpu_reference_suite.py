"""The reference's own backend unit tests run against ``fock_gb300``.

``tests/refsuite/stage.py`` copies the reference's ``tests/backend`` files for
the Fock backend's interface (gates, preparations, measurements, states,
add/del modes) into ``baseline/_ref_tests/backend``, and its engine-level
``tests/integration`` files into ``baseline/_ref_tests/integration``, with the
fixture shim
``tests/refsuite/conftest_gb300.py`` as their conftest; this test runs them
unmodified in a child pytest with the GB300 backend in place of the
reference's ``FockBackend``, pure and mixed, at the reference's default
tolerances (TOL 1e-3, CUTOFF 6, HBAR 1.7).
"""
import os
import re
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STAGED = os.path.join(ROOT, "baseline", "_ref_tests", "backend")
STAGED_INTEGRATION = os.path.join(ROOT, "baseline", "_ref_tests", "integration")


def _summary(text):
    counts = {}
    for n, what in re.findall(r"(\d+) (passed|failed|skipped|errors?|deselected)", text):
        counts[what.rstrip("s") if what.startswith("error") else what] = int(n)
    return counts


def _run(staged, min_passed, extra=()):
    if not os.path.isfile(os.path.join(staged, "conftest.py")):
        pytest.skip("reference tests not staged (python tests/refsuite/stage.py REFERENCE_ROOT)")
    env = dict(os.environ, FOCK_REFSUITE_BACKEND="fock_gb300", FOCK_GB300_REPO=ROOT)
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-p", "no:cacheprovider", "-rfE", *extra, "."],
                       cwd=staged, env=env, capture_output=True, text=True, timeout=1800)
    counts = _summary(r.stdout.splitlines()[-1] if r.stdout else "")
    report = "\n".join(r.stdout.splitlines()[-60:]) + r.stderr[-2000:]
    assert r.returncode == 0, report
    assert counts.get("failed", 0) == 0 and counts.get("error", 0) == 0, report
    assert counts.get("passed", 0) >= min_passed, report


def test_reference_backend_suite_on_gb300(cuda):
    _run(STAGED, 1500)


def test_reference_integration_suite_on_gb300(cuda):
    """The reference's tests/integration files that run programs through an
    engine (setup_eng) on the Fock interface: decompositions, engine,
    hbar, measurements, operations, parameters, utils.  The
    utils.extract_unitary tests are left out: that utility accepts only the
    backend names 'fock' and 'tf' (strawberryfields/utils/program_functions.py),
    whatever backend the fixture provides."""
    _run(STAGED_INTEGRATION, 230, ("-m", "not gaussian and not bosonic and not tf", "-k", "not TestExtractUnitary"))
