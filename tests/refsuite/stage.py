"""Stage the reference's backend test files for a run against ``fock_gb300``.

The reference's own unit tests of the backend interface
(``tests/backend/test_*.py`` in the Strawberry Fields source tree) and its
integration tests that run programs through an engine
(``tests/integration/test_*.py``) are the strongest evidence that the GB300
backend is a drop-in for the ``fock`` backend.  They are not copied into this
repository: this script copies them from a reference checkout into
``baseline/_ref_tests/backend`` and ``baseline/_ref_tests/integration`` (git-ignored,
like the reference install under ``baseline/_ref``), next to the fixture shim
``tests/refsuite/conftest_gb300.py`` installed as their ``conftest.py``.  The
files run unmodified; the shim replaces the reference's
``tests/conftest.py`` (its ``setup_backend`` fixture, conftest.py:160-186,
parametrised with the GB300 backend instead of Fock/Gaussian/Bosonic).

Usage: ``python tests/refsuite/stage.py [REFERENCE_ROOT]`` (default
``$SF_REFERENCE_ROOT``).
"""
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
DEST = os.path.join(REPO, "baseline", "_ref_tests", "backend")
DEST_INTEGRATION = os.path.join(REPO, "baseline", "_ref_tests", "integration")

# the reference's test files that exercise the BaseFock surface; files for
# the Gaussian/bosonic/TF backends only are left out (their marks would skip
# every test anyway)
FILES = [
    "test_beamsplitter_operation.py",
    "test_displaced_squeezed_state_preparation.py",
    "test_displacement_operation.py",
    "test_fock_measurement.py",
    "test_homodyne.py",
    "test_is_vacuum.py",
    "test_loss_channel.py",
    "test_modes.py",
    "test_multimode_state_preparations.py",
    "test_mzgate_operation.py",
    "test_nongaussian_gates.py",
    "test_postselection.py",
    "test_rotation_operation.py",
    "test_squeeze_operation.py",
    "test_squeezed_state_preparation.py",
    "test_state_preparations.py",
    "test_states.py",
    "test_states_polyquad.py",
    "test_states_probabilities.py",
    "test_states_wigner.py",
    "test_twomode_squeezing_operation.py",
]

# the reference's integration tests that run whole programs through an engine
# (setup_eng) on the Fock backend interface
INTEGRATION = [
    "test_decompositions_integration.py",
    "test_engine_integration.py",
    "test_hbar_integration.py",
    "test_measurement_integration.py",
    "test_ops_integration.py",
    "test_parameters_integration.py",
    "test_utils_integration.py",
]

PYTEST_INI = """[pytest]
markers =
    backends(name1, name2, ...): test applies to named backends only
    fock: fock backend
    gaussian: gaussian backend
    bosonic: bosonic backend
    tf: tf backend
    pure: pure states
    mixed: mixed states
    broken: broken test
"""


def _stage_dir(src, dest, files):
    if not os.path.isdir(src):
        raise SystemExit(f"{src} does not exist")
    os.makedirs(dest, exist_ok=True)
    for name in files:
        shutil.copyfile(os.path.join(src, name), os.path.join(dest, name))
    shutil.copyfile(os.path.join(HERE, "conftest_gb300.py"), os.path.join(dest, "conftest.py"))
    with open(os.path.join(dest, "pytest.ini"), "w") as f:
        f.write(PYTEST_INI)


def stage(ref_root=None, dest=DEST, dest_integration=DEST_INTEGRATION):
    """Copy the test files and the shim (backend tests to ``dest``,
    integration tests to ``dest_integration``); returns ``dest``."""
    ref_root = ref_root or os.environ.get("SF_REFERENCE_ROOT")
    if not ref_root:
        raise SystemExit("usage: stage.py REFERENCE_ROOT (or set SF_REFERENCE_ROOT)")
    _stage_dir(os.path.join(ref_root, "tests", "backend"), dest, FILES)
    _stage_dir(os.path.join(ref_root, "tests", "integration"), dest_integration, INTEGRATION)
    return dest


if __name__ == "__main__":
    print(stage(sys.argv[1] if len(sys.argv) > 1 else None))
