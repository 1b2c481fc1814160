"""ctypes binding of ``libnecstar_gpu.so`` (the C ABI of include/necstar_gpu.h).

The library must have been built (``stab_decomp_simulator_rust_gb300.build``
or ``__graft_entry__.build()``); importing the API without it raises — there
is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import re

from . import build as _build

HEADER = os.path.join(os.path.dirname(_build.PKG), "include", "necstar_gpu.h")

_lib = None


class Gate(C.Structure):
    _fields_ = [("op", C.c_uint32), ("q0", C.c_uint32), ("q1", C.c_uint32), ("q2", C.c_uint32)]


class PauliABI(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("len", C.c_uint32),
                ("ops", C.POINTER(C.c_uint8)), ("qubits", C.POINTER(C.c_uint32))]


def header_symbols() -> list[str]:
    """Names of every function declared in include/necstar_gpu.h."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(nsg_[a-z_0-9]+)\s*\(", text)))


def header_constants() -> dict[str, int]:
    text = open(HEADER).read()
    return {k: int(v) for k, v in re.findall(r"#define\s+(NSG_[A-Z_0-9]+)\s+(-?\d+)", text)}


def load(path: str | None = None):
    """Loads the library (once) and declares the signatures."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or _build.LIB
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build the CUDA library first (python -c 'import __graft_entry__ as g; g.build()')")
    L = C.CDLL(path)
    vp, sz, u32, u64, i32, dbl = C.c_void_p, C.c_size_t, C.c_uint32, C.c_uint64, C.c_int32, C.c_double
    P = C.POINTER
    L.nsg_version.restype = C.c_char_p
    L.nsg_last_error_message.restype = C.c_char_p
    L.nsg_last_error_args.argtypes = [P(C.c_int64)]
    L.nsg_state_from_circuit.argtypes = [u32, vp, sz, P(vp)]
    L.nsg_state_from_terms.argtypes = [u32, u64] + [vp] * 11 + [P(vp)]
    L.nsg_state_free.argtypes = [vp]
    L.nsg_state_free.restype = None
    L.nsg_state_clone.argtypes = [vp, P(vp)]
    L.nsg_num_qubits.argtypes = [vp, P(u32)]
    L.nsg_stabilizer_rank.argtypes = [vp, P(u64)]
    L.nsg_state_set_stream.argtypes = [vp, vp]
    L.nsg_apply_gates.argtypes = [vp, vp, sz]
    L.nsg_exp_value.argtypes = [vp, P(PauliABI), P(dbl)]
    L.nsg_exp_value_batch.argtypes = [vp, P(PauliABI), sz, u32, vp]
    L.nsg_exp_value_noalloc.argtypes = [vp, P(PauliABI), P(dbl)]
    L.nsg_exp_value_multi.argtypes = [vp, sz, P(PauliABI), vp, u32, vp]
    L.nsg_plan_create.argtypes = [vp, sz, P(PauliABI), vp, u32, P(vp)]
    L.nsg_plan_run.argtypes = [vp, vp]
    L.nsg_plan_info.argtypes = [vp, vp, vp, vp, P(i32)]
    L.nsg_plan_free.argtypes = [vp]
    L.nsg_plan_free.restype = None
    L.nsg_inner_product.argtypes = [vp, vp, vp]
    L.nsg_norm.argtypes = [vp, P(dbl)]
    L.nsg_project_normalized.argtypes = [vp, u32, i32]
    L.nsg_project_unnormalized.argtypes = [vp, u32, i32]
    L.nsg_discard.argtypes = [vp, u32]
    L.nsg_measure.argtypes = [vp, vp, sz, vp, vp]
    L.nsg_measure_all.argtypes = [vp, vp, vp]
    L.nsg_sample.argtypes = [vp, vp, sz, u64, vp, vp, vp, sz, P(sz)]
    L.nsg_to_statevector.argtypes = [vp, vp, sz]
    L.nsg_export_terms.argtypes = [vp] + [vp] * 11
    L.nsg_debug_pair_values.argtypes = [vp, vp, vp, vp]
    L.nsg_debug_t_tensor.argtypes = [u32, P(vp)]
    L.nsg_state_kron.argtypes = [vp, vp, P(vp)]
    L.nsg_random_clifford.argtypes = [u32, vp, vp, sz, P(sz)]
    L.nsg_random_words.argtypes = [vp, vp, sz]
    L.nsg_debug_chacha_block.argtypes = [vp, i32, vp]
    L.nsg_profile_enable.argtypes = [i32]
    L.nsg_profile_read.argtypes = [P(dbl), P(u64), P(u64)]
    L.nsg_probe_int_ops.argtypes = [u64, P(dbl), P(u64)]
    L.nsg_exp_value_counts.argtypes = [vp, P(PauliABI), sz, vp, P(dbl)]
    L.nsg_zero_screen.argtypes = [vp, P(PauliABI), sz, vp]
    L.nsg_zero_screen_circuit.argtypes = [u32, vp, sz, P(PauliABI), sz, vp]
    L.nsg_set_pair_tiling.argtypes = [i32, i32]
    L.nsg_debug_compile_keep.argtypes = [u32, vp, sz, vp, sz, P(u64)]
    L.nsg_state_select.argtypes = [vp, vp, sz, P(vp)]
    L.nsg_debug_set_wait.argtypes = [u32, u32]
    L.nsg_states_from_circuits.argtypes = [sz, vp, vp, vp, vp]
    L.nsg_toffoli_tensor_state.argtypes = [u32, P(vp)]
    for name in header_symbols():
        fn = getattr(L, name)
        if name not in ("nsg_version", "nsg_last_error_message", "nsg_state_free", "nsg_plan_free"):
            fn.restype = C.c_int32
    _lib = L
    return L


class NecstarError(ValueError):
    """Raised for every non-zero status; the reference's Python layer maps
    every Rust error to ValueError (python/src/state.rs:22-40)."""

    def __init__(self, code: int, message: str, args3):
        super().__init__(message or f"necstar error {code}")
        self.code = code
        self.args3 = tuple(args3)


def check(rc: int):
    if rc != 0:
        L = load()
        a = (C.c_int64 * 3)()
        L.nsg_last_error_args(a)
        raise NecstarError(rc, (L.nsg_last_error_message() or b"").decode(), list(a))
