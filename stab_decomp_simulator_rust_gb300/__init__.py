"""GB300-native stabilizer-decomposition engine with NECSTAR's Python surface.

``QuantumCircuit`` → ``QuantumState.from_circuit`` compiles a Clifford+T
circuit into χ CH-form terms held in HBM; ``exp_value``, ``norm``,
``inner_product``, projection, measurement and sampling evaluate the χ² pair
sums with hand-written sm_103a kernels (libnecstar_gpu.so, C ABI in
include/necstar_gpu.h).
"""
from .circuit import QuantumCircuit, QuantumGate
from .pauli import PauliString
from .state import PRECISION_FP64, PRECISION_MIXED, BatchPlan, QuantumState, exp_values_multi, zero_screen_circuit
from ._ffi import NecstarError

__all__ = ["QuantumCircuit", "QuantumGate", "PauliString", "QuantumState", "NecstarError",
           "PRECISION_FP64", "PRECISION_MIXED", "exp_values_multi", "BatchPlan", "zero_screen_circuit"]
