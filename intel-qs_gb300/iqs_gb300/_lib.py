"""ctypes binding of libiqsg.so (include/iqsg.h).

The library is required: importing this module without it, or on a machine without a
CUDA device when a register is created, raises. There is no CPU implementation behind
this package.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "libiqsg.so"

IQSG_OK, IQSG_EINVAL, IQSG_ENOMEM, IQSG_EDEVICE, IQSG_ETIMEOUT, IQSG_ENOTSUP = range(6)
COMPLEX_DP, COMPLEX_SP = 0, 1
MATH_NATIVE, MATH_EMULATED = 0, 1
OPT_SWEEP_WIDTH, OPT_SWEEP_PIPELINE, OPT_TILE_QUBITS, OPT_NATIVE_SHARE, OPT_DF_STORAGE = 0, 1, 2, 3, 4

_P = C.c_void_p
_U = C.c_uint
_U64 = C.c_uint64
_D = C.c_double
_DP = C.POINTER(C.c_double)
_UP = C.POINTER(C.c_uint)
_IP = C.POINTER(C.c_int)

OP_1Q, OP_CTRL, OP_2Q, OP_SWAPLIKE, OP_DIAG2, OP_PHASE, OP_GRAD1, OP_GRAD2 = range(8)
HIST_INTEGER, HIST_ROUNDED, HIST_BINNED = 0, 1, 2


class Op(C.Structure):
    """iqsg_op (include/iqsg.h): one gate of a stream for iqsg_apply_ops."""
    _fields_ = [("kind", C.c_int32), ("t0", C.c_uint32), ("t1", C.c_uint32), ("nctrl", C.c_uint32),
                ("ctrl", C.c_uint32 * 4), ("mask", C.c_uint64), ("value", C.c_uint64), ("m", C.c_double * 32)]


assert C.sizeof(Op) == 304, "iqsg_op layout mismatch"


class SweepInfo(C.Structure):
    """iqsg_sweep_info (include/iqsg.h): one fused sweep of a planned gate stream."""
    _fields_ = [("k", C.c_uint), ("pos", C.c_uint * 4), ("ops", C.c_uint), ("one_qubit", C.c_uint),
                ("two_qubit", C.c_uint), ("diagonal", C.c_uint)]


class PauliTerm(C.Structure):
    """iqsg_pauli_term (include/iqsg.h)."""
    _fields_ = [("xmask", C.c_uint64), ("zmask", C.c_uint64), ("ny", C.c_int32), ("pad", C.c_int32),
                ("coeff", C.c_double)]


assert C.sizeof(PauliTerm) == 32, "iqsg_pauli_term layout mismatch"

# name -> argtypes (every function returns int status unless listed in _RESTYPES)
SIGNATURES = {
    "iqsg_last_error": [],
    "iqsg_version": [],
    "iqsg_create": [_U, C.c_int, _P, C.POINTER(_P)],
    "iqsg_create_from_device": [_U, C.c_int, _P, _P, C.POINTER(_P)],
    "iqsg_clone": [_P, C.POINTER(_P)],
    "iqsg_destroy": [_P],
    "iqsg_info": [_P, _UP, C.POINTER(C.c_int), C.POINTER(_P)],
    "iqsg_set_math": [_P, C.c_int],
    "iqsg_synchronize": [_P],
    "iqsg_fill": [_P, _D, _D],
    "iqsg_init_basis": [_P, _U64],
    "iqsg_set_amplitude": [_P, _U64, _D, _D],
    "iqsg_get_amplitude": [_P, _U64, _DP],
    "iqsg_upload": [_P, _P, _U64, _U64],
    "iqsg_download": [_P, _P, _U64, _U64],
    "iqsg_init_uniform_random": [_P, _U64, _U64, _D, _D],
    "iqsg_counters": [_P, C.POINTER(_U64)],
    "iqsg_plan_ops": [C.c_uint, C.c_int, C.c_int, C.c_uint, C.c_void_p, C.c_uint, C.POINTER(SweepInfo), C.c_uint,
                      C.POINTER(C.c_uint), C.POINTER(C.c_int)],
    "iqsg_rng_create": [C.POINTER(_P)],
    "iqsg_rng_destroy": [_P],
    "iqsg_rng_clone": [_P, C.c_int, C.POINTER(_P)],
    "iqsg_rng_set_seed": [_P, _U64],
    "iqsg_rng_set_seed_pool": [_P, _U64, C.c_uint, C.c_uint, C.c_uint],
    "iqsg_rng_skip": [_P, C.c_int, _U64, C.c_int],
    "iqsg_rng_uniform": [_P, C.c_int, _DP, _U64, _D, _D, C.c_int],
    "iqsg_rng_gaussian": [_P, C.c_int, _DP, _U64, C.c_int],
    "iqsg_rng_integers": [_P, C.c_int, C.POINTER(C.c_int), _U64, C.c_int, C.c_int, C.c_int],
    "iqsg_rng_info": [_P, C.POINTER(_U64), C.POINTER(_U64)],
    "iqsg_init_random": [_P, _P, C.c_int],
    "iqsg_noise_gate_matrix": [C.c_int, _D, _D, _D, _DP, _DP],
    "iqsg_noise_gate_draw": [_P, C.c_int, _D, _D, _D, _DP],
    "iqsg_noise_engine_create": [C.c_uint32, C.POINTER(_P)],
    "iqsg_noise_engine_destroy": [_P],
    "iqsg_noise_engine_gaussian": [_P, C.c_int, _DP, _U64],
    "iqsg_chi_eigensystem": [C.c_int, C.c_uint, _DP, _DP, _DP, _DP, _DP],
    "iqsg_chi_normalize": [C.c_int, C.c_uint, _DP, _DP, _DP, _DP],
    "iqsg_channel_gate": [_P, C.c_int, C.c_uint, _DP, _DP, _DP, _DP, C.POINTER(C.c_uint), C.POINTER(C.c_int)],
    "iqsg_upload_async": [_P, _P, _U64, _U64],
    "iqsg_download_async": [_P, _P, _U64, _U64],
    "iqsg_copy": [_P, _P],
    "iqsg_apply_1q": [_P, _U, _DP],
    "iqsg_apply_controlled_1q": [_P, _U, _U, _DP],
    "iqsg_apply_multi_controlled_1q": [_P, _U, _UP, _U, _DP],
    "iqsg_apply_2q": [_P, _U, _U, _DP],
    "iqsg_apply_swaplike": [_P, _U, _U, _DP],
    "iqsg_apply_diag_2q": [_P, _U, _U, _DP],
    "iqsg_apply_cost_phase": [_P, _P, _D],
    "iqsg_collapse": [_P, _U, C.c_int],
    "iqsg_scale": [_P, _D, _D],
    "iqsg_axpy": [_P, _P, _D, _D],
    "iqsg_permute": [_P, _UP, _UP],
    "iqsg_probability": [_P, _U, _DP],
    "iqsg_expectation_pauli": [_P, _U, _UP, _UP, _DP, _DP],
    "iqsg_norm2": [_P, _DP],
    "iqsg_overlap": [_P, _P, _DP],
    "iqsg_max_abs_diff": [_P, _P, _D, _D, _DP],
    "iqsg_l2_diff": [_P, _P, _DP],
    "iqsg_cost_expectation": [_P, _P, C.c_int, _DP],
    "iqsg_maxcut_cost": [_P, _IP, _UP, _IP],
    "iqsg_weighted_maxcut_cost": [_P, _DP, _UP, _DP],
    "iqsg_state_stats": [_P, _DP],
    "iqsg_cost_histogram": [_P, _P, C.c_int, _D, _D, _DP, _U],
    "iqsg_apply_ops": [_P, C.POINTER(Op), _U, _UP],
    "iqsg_adjoint_ops": [_P, _P, C.POINTER(Op), _U, _DP, _U, _UP],
    "iqsg_set_sweep_width": [_P, _U],
    "iqsg_set_option": [_P, C.c_int, C.c_int],
    "iqsg_qaoa_layer": [_P, _U, _UP, _IP, _D, _D],
    "iqsg_qaoa_observable": [_P, _P, _U, _UP, _IP, _DP, _DP],
    "iqsg_qaoa_layer_backward": [_P, _P, _U, _UP, _IP, _D, _D, _DP, _DP],
    "iqsg_qaoa_layer_ckpt": [_P, _P, _P, _U, _UP, _IP, _D, _D],
    "iqsg_qaoa_layer_backward_ckpt": [_P, _P, _P, _U, _UP, _IP, _D, _D, _DP, _DP],
    "iqsg_batch_create": [_U, _UP, _UP, _UP, C.POINTER(PauliTerm), C.c_int, _P, C.POINTER(_P)],
    "iqsg_batch_destroy": [_P],
    "iqsg_batch_run": [_P, _DP, C.c_int, _DP, _DP],
    "iqsg_batch_set_launch": [_P, _U, _U],
    "iqsg_batch_info": [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)],
    "iqsg_probability_static": [_P, _U, C.c_int, _U, _P, _P],
}
_RESTYPES = {"iqsg_last_error": C.c_char_p, "iqsg_rng_destroy": None, "iqsg_noise_engine_destroy": None}


def _load() -> C.CDLL:
    if not LIB_PATH.exists():
        raise ImportError(
            f"libiqsg.so not found at {LIB_PATH}; build it first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = C.CDLL(str(LIB_PATH))
    for name, argtypes in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = argtypes
        fn.restype = _RESTYPES.get(name, C.c_int)
    return lib


lib = _load()


class IqsgError(RuntimeError):
    """A CUDA-side failure reported by libiqsg (status IQSG_EDEVICE / IQSG_ETIMEOUT / ...)."""

    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status


def check(status: int) -> None:
    """Raise the Python exception matching an iqsg_status (EINVAL -> ValueError,
    ENOMEM -> MemoryError, others -> IqsgError)."""
    if status == IQSG_OK:
        return
    msg = (lib.iqsg_last_error() or b"").decode(errors="replace")
    if status == IQSG_EINVAL:
        raise ValueError(msg)
    if status == IQSG_ENOMEM:
        raise MemoryError(msg)
    raise IqsgError(status, msg)


def dptr(a) -> "C.POINTER(C.c_double)":
    return a.ctypes.data_as(_DP)


def uptr(a) -> "C.POINTER(C.c_uint)":
    return a.ctypes.data_as(_UP)


def iptr(a) -> "C.POINTER(C.c_int)":
    return a.ctypes.data_as(_IP)
