"""ctypes binding of ``libtedq_gb300.so`` (declarations: include/tedq_gb300.h).

The library is built in-tree by ``ted-q_gb300/csrc/build.py`` (or
``__graft_entry__.build()``).  There is no fallback: if the library is
missing every backend call raises ``RuntimeError``.
"""

import ctypes
import os
from ctypes import POINTER, c_char_p, c_double, c_int32, c_int64, c_size_t, c_void_p

from .errors import BackendError

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libtedq_gb300.so")
ABI_VERSION = 1

# status codes
OK, ERR_ARG, ERR_OOM, ERR_CUDA, ERR_TIMEOUT, ERR_UNSUPPORTED, ERR_STATE = range(7)

# gate opcodes (TEDQ_OP_*)
OP = {"I": 0, "Hadamard": 1, "PauliX": 2, "PauliY": 3, "PauliZ": 4, "S": 5, "T": 6, "SX": 7,
      "CNOT": 8, "CZ": 9, "CY": 10, "SWAP": 11, "CSWAP": 12, "Toffoli": 13,
      "RX": 14, "RY": 15, "RZ": 16, "Rot": 17, "PhaseShift": 18, "ControlledPhaseShift": 19,
      "CRX": 20, "CRY": 21, "CRZ": 22}
OP_MATRIX = 23
OBS = {"I": 0, "PauliX": 1, "PauliY": 2, "PauliZ": 3, "Hadamard": 4}
OBS_MATRIX = 5
MEAS_EXPVAL, MEAS_PROBS, MEAS_STATE = 0, 1, 2
PREC_C64, PREC_C128 = 0, 1


class Gate(ctypes.Structure):
    _fields_ = [("op", c_int32), ("n_qubits", c_int32), ("qubits", c_int32 * 3), ("param_slot", c_int32 * 3),
                ("fixed", c_double * 3), ("matrix", POINTER(c_double))]


class ObsFactor(ctypes.Structure):
    _fields_ = [("obs", c_int32), ("n_qubits", c_int32), ("qubits", c_int32 * 3), ("matrix", POINTER(c_double))]


class Meas(ctypes.Structure):
    _fields_ = [("kind", c_int32), ("n_factors", c_int32), ("factors", POINTER(ObsFactor)),
                ("n_qubits", c_int32), ("qubits", POINTER(c_int32))]


class Options(ctypes.Structure):
    _fields_ = [("precision", c_int32), ("fuse", c_int32), ("tile_qubits", c_int32), ("jit", c_int32),
                ("exact_phase", c_int32), ("reserved", c_int32 * 3)]


class ProgramInfo(ctypes.Structure):
    _fields_ = [("n_qubits", c_int32), ("state_qubits", c_int32), ("n_params", c_int32),
                ("n_real_outputs", c_int32), ("n_terms", c_int32), ("n_fwd_passes", c_int32),
                ("n_bwd_passes", c_int32), ("n_fwd_phases", c_int32), ("n_bwd_phases", c_int32),
                ("n_fused_gates", c_int32), ("n_elem_gates", c_int32), ("precision", c_int32),
                ("workspace_per_circuit", c_int64), ("jit_state", c_int32), ("pad", c_int32),
                ("jit_modules_loaded", c_int64), ("reserved", c_int64 * 2)]


class Profile(ctypes.Structure):
    _fields_ = [("fwd_launches", c_int64), ("fwd_ms", c_double), ("bwd_launches", c_int64), ("bwd_ms", c_double),
                ("meas_launches", c_int64), ("meas_ms", c_double), ("lam_launches", c_int64), ("lam_ms", c_double),
                ("fwd_amp_passes", c_int64), ("bwd_amp_passes", c_int64), ("reserved", c_int64 * 4)]


class ServerOptions(ctypes.Structure):
    _fields_ = [("device", c_int32), ("n_streams", c_int32), ("max_batch", c_int32), ("max_wait_us", c_int32),
                ("memory_budget_bytes", c_int64), ("paused", c_int32), ("lane_qubits", c_int32),
                ("reserved", c_int64 * 3)]


class RequestResult(ctypes.Structure):
    _fields_ = [("status", c_int32), ("batch_size", c_int32), ("queue_us", c_double), ("total_us", c_double)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", c_int64), ("completed", c_int64), ("failed", c_int64), ("cancelled", c_int64),
                ("batches", c_int64), ("in_flight_bytes", c_int64), ("peak_in_flight_bytes", c_int64),
                ("reserved", c_int64 * 4)]


class TnOptions(ctypes.Structure):
    _fields_ = [("precision", c_int32), ("gemm", c_int32), ("max_rank", c_int32), ("repeats", c_int32),
                ("seed", ctypes.c_uint64), ("graphs", c_int32), ("reserved", c_int32 * 3)]


class TnInfo(ctypes.Structure):
    _fields_ = [("n_qubits", c_int32), ("n_params", c_int32), ("n_meas", c_int32), ("n_steps", c_int32),
                ("max_rank", c_int32), ("n_sliced", c_int32), ("gates_kept", c_int32), ("precision", c_int32),
                ("log2_flops", c_double), ("workspace_per_circuit", c_int64), ("workspace_fixed", c_int64),
                ("reserved", c_int64 * 4)]


class TnProfile(ctypes.Structure):
    _fields_ = [("leaf_launches", c_int64), ("leaf_ms", c_double), ("gather_launches", c_int64),
                ("gather_ms", c_double), ("gather_bytes", c_double), ("gemm_launches", c_int64),
                ("gemm_ms", c_double), ("gemm_flops", c_double), ("root_launches", c_int64), ("root_ms", c_double),
                ("tc_launches", c_int64), ("tc_ms", c_double), ("tc_flops", c_double), ("gemm_error", c_int32),
                ("pad", c_int32)]


TN_GEMM = {"fp32": 0, "tc32": 1, "tf32": 2, "auto": 3}

# every symbol the header declares, with (restype, argtypes)
SIGNATURES = {
    "tedq_abi_version": (c_int32, []),
    "tedq_last_error": (c_int32, [c_char_p, c_size_t]),
    "tedq_program_create": (c_int32, [POINTER(Gate), c_int32, c_int32, POINTER(Meas), c_int32, POINTER(Options),
                                      POINTER(c_void_p)]),
    "tedq_program_destroy": (c_int32, [c_void_p]),
    "tedq_program_info": (c_int32, [c_void_p, POINTER(ProgramInfo)]),
    "tedq_program_workspace_bytes": (c_int64, [c_void_p, c_int64]),
    "tedq_program_jit_wait": (c_int32, [c_void_p]),
    "tedq_program_describe": (c_int64, [c_void_p, c_int32, c_char_p, c_int64]),
    "tedq_run": (c_int32, [c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p, c_void_p, c_size_t,
                           c_void_p]),
    "tedq_run_adjoint": (c_int32, [c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p, c_void_p,
                                   c_void_p, c_void_p, c_size_t, c_void_p]),
    "tedq_run_noalloc": (c_int32, [c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p, c_void_p]),
    "tedq_server_create": (c_int32, [POINTER(ServerOptions), POINTER(c_void_p)]),
    "tedq_server_destroy": (c_int32, [c_void_p]),
    "tedq_server_submit": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p, c_int32, POINTER(c_int64)]),
    "tedq_server_wait": (c_int32, [c_void_p, c_int64, c_int64, c_void_p, c_void_p, POINTER(RequestResult)]),
    "tedq_server_cancel": (c_int32, [c_void_p, c_int64]),
    "tedq_server_stats": (c_int32, [c_void_p, POINTER(ServerStats)]),
    "tedq_server_resume": (c_int32, [c_void_p]),
    "tedq_profile_enable": (c_int32, [c_void_p, c_int32]),
    "tedq_profile_read": (c_int32, [c_void_p, POINTER(Profile)]),
    "tedq_tn_plan_create": (c_int32, [POINTER(Gate), c_int32, c_int32, POINTER(Meas), c_int32, POINTER(TnOptions),
                                      POINTER(c_void_p)]),
    "tedq_tn_plan_destroy": (c_int32, [c_void_p]),
    "tedq_tn_plan_info": (c_int32, [c_void_p, POINTER(TnInfo)]),
    "tedq_tn_plan_describe": (c_int64, [c_void_p, c_char_p, c_int64]),
    "tedq_tn_workspace_bytes": (c_int64, [c_void_p, c_int64]),
    "tedq_tn_contract": (c_int32, [c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_size_t, c_void_p]),
    "tedq_tn_profile_enable": (c_int32, [c_void_p, c_int32]),
    "tedq_tn_profile_read": (c_int32, [c_void_p, POINTER(TnProfile)]),
    "tedq_tn_gemm": (c_int32, [c_int32, c_int32, c_void_p, c_void_p, c_void_p, c_int64, c_int64, c_int64, c_int64,
                               c_int64, c_int64, c_int64, c_void_p, c_void_p]),
}

_lib = None


def lib():
    """The loaded library; raises RuntimeError when it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python ted-q_gb300/csrc/build.py` "
                               "(or __graft_entry__.build()); the GB300 backend has no fallback path")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        if L.tedq_abi_version() != ABI_VERSION:
            raise RuntimeError(f"libtedq_gb300 ABI {L.tedq_abi_version()} != expected {ABI_VERSION}")
        _lib = L
    return _lib


def last_error():
    buf = ctypes.create_string_buffer(4096)
    lib().tedq_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(status, what):
    if status == OK:
        return
    msg = last_error()
    if status == ERR_ARG:
        raise ValueError(f"{what}: {msg}")
    if status == ERR_UNSUPPORTED:
        raise NotImplementedError(f"{what}: {msg}")
    raise BackendError(f"{what} failed with status {status}: {msg}")
