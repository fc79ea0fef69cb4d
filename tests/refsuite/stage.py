"""Stage the reference's backend test files for a run against ``fock_gb300``.

The reference's own unit tests of the backend interface
(``tests/backend/test_*.py`` in the Strawberry Fields source tree) are the
strongest evidence that the GB300 backend is a drop-in for the ``fock``
backend.  They are not copied into this repository: this script copies them
from a reference checkout into ``baseline/_ref_tests/backend`` (git-ignored,
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


def stage(ref_root=None, dest=DEST):
    """Copy the test files and the shim; returns the staged directory."""
    ref_root = ref_root or os.environ.get("SF_REFERENCE_ROOT")
    if not ref_root:
        raise SystemExit("usage: stage.py REFERENCE_ROOT (or set SF_REFERENCE_ROOT)")
    src = os.path.join(ref_root, "tests", "backend")
    if not os.path.isdir(src):
        raise SystemExit(f"{src} does not exist")
    os.makedirs(dest, exist_ok=True)
    for name in FILES:
        shutil.copyfile(os.path.join(src, name), os.path.join(dest, name))
    shutil.copyfile(os.path.join(HERE, "conftest_gb300.py"), os.path.join(dest, "conftest.py"))
    with open(os.path.join(dest, "pytest.ini"), "w") as f:
        f.write(PYTEST_INI)
    return dest


if __name__ == "__main__":
    print(stage(sys.argv[1] if len(sys.argv) > 1 else None))
