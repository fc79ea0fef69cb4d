"""GB300-native Fock-basis circuit simulator with a Strawberry Fields
``BaseFock`` backend face.

The compute path is ``libfockgb300.so`` (hand-written sm_103a CUDA behind a
C ABI, ``include/fock_gb300.h``); this package is the host side:

* :mod:`.backend` -- ``FockGB300Backend`` / ``sf_backend()``, the drop-in
  ``BaseFock`` backend (reference ``fockbackend/backend.py``);
* :mod:`.circuit` -- ``DeviceCircuit``, device state updates (reference
  ``fockbackend/circuit.py``);
* :mod:`.states` -- ``FockStateGB300`` readouts (reference ``states.py``);
* :mod:`.autograd` -- ``CompiledCircuit``, fused forward sweep + adjoint
  gradients as a ``torch.autograd.Function``;
* :mod:`.qnn` -- CV-QNN gate lists (reference ``examples/quantum_neural_network.py``).
"""

from . import _lib
from ._lib import load as load_library
from .backend import FockGB300Backend, register, sf_backend
from .circuit import DeviceCircuit
from .states import FockStateGB300
from .autograd import CompiledCircuit

__all__ = ["FockGB300Backend", "sf_backend", "register", "DeviceCircuit", "FockStateGB300", "CompiledCircuit",
           "load_library"]
