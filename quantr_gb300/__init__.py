"""quantr_gb300 — GB300-native state-vector engine behind quantr's simulate path.

Public names mirror the quantr crate's root re-exports (src/lib.rs:78-84): `Gate`, `Circuit`,
`SimulatedCircuit`, `Measurement` (`Observable` / `NonObservable`), `QuantrError` and
`states` (`Qubit`, `ProductState`, `SuperPosition`). Simulation runs in libquantr_gpu
(hand-written sm_103a kernels behind the C ABI of include/qgpu.h); there is no CPU fallback.
"""
from . import states
from .circuit import (Circuit, Measurement, NonObservable, Observable, SimulatedCircuit,
                      set_default_backend)
from .errors import QuantrError
from .gate import Gate
from .rng import seed
from .states import ProductState, Qubit, SuperPosition

__all__ = ["Circuit", "Gate", "Measurement", "NonObservable", "Observable", "ProductState",
           "QuantrError", "Qubit", "SimulatedCircuit", "SuperPosition", "seed",
           "set_default_backend", "states"]
