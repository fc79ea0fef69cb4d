"""The fixture shim that runs the reference's backend tests on fock_gb300
(tests/refsuite/conftest_gb300.py), checked without a GPU: with the
reference's own FockBackend in place of the GB300 backend the staged files
must pass as they do under the reference's conftest."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STAGED = os.path.join(ROOT, "baseline", "_ref_tests", "backend")


def test_shim_runs_reference_backend_files():
    if not os.path.isfile(os.path.join(STAGED, "conftest.py")):
        pytest.skip("reference backend tests not staged (python tests/refsuite/stage.py REFERENCE_ROOT)")
    env = dict(os.environ, FOCK_REFSUITE_BACKEND="fock", FOCK_GB300_REPO=ROOT)
    files = ["test_modes.py", "test_displacement_operation.py", "test_states_probabilities.py"]
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-p", "no:cacheprovider"] + files, cwd=STAGED,
                       env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]
    assert " passed" in r.stdout
