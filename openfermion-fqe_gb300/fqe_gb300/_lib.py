"""ctypes binding of libfqegpu.so (the C ABI declared in include/fqegpu.h).

This is the analogue of the reference's ``fqe/lib/__init__.py`` (which loads
``libfqe.so`` with ctypes) and of the ndpointer/argtypes wrappers in
``fqe/lib/fci_graph.py`` and ``_fqe_data.pyx``.  There is no CPU fallback:
if the library is missing or no CUDA device is present, every call raises.
"""

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libfqegpu.so")

OK = 0
ERR_INVALID = 1
ERR_NOMEM = 2
ERR_CUDA = 3
ERR_UNSUPPORTED = 4
ERR_TIMEOUT = 5
ERR_NUMERIC = 6

PREC_FP64 = 0
PREC_OZAKI = 1

_P = ctypes.c_void_p
_I = ctypes.c_int
_L = ctypes.c_int64
_D = ctypes.c_double

_SIGNATURES = {
    "fqegpu_version": [],
    "fqegpu_last_error": [ctypes.c_char_p, _I],
    "fqegpu_sync": [_P],
    "fqegpu_graph_create": [_I, _I, _I, _P, ctypes.POINTER(_P)],
    "fqegpu_graph_destroy": [_P],
    "fqegpu_graph_dims": [_P, ctypes.POINTER(_L), ctypes.POINTER(_L),
                          ctypes.POINTER(_I), ctypes.POINTER(_I)],
    "fqegpu_graph_strings": [_P, _I, _P],
    "fqegpu_graph_zmatrix": [_P, _I, _P],
    "fqegpu_graph_dexc": [_P, _I, _P],
    "fqegpu_graph_map_lengths": [_P, _I, _P],
    "fqegpu_graph_maps": [_P, _I, _P],
    "fqegpu_ham_create": [_P, _P, _P, _P, ctypes.POINTER(_P)],
    "fqegpu_ham_create_spin": [_P, _P, _P, _P, ctypes.POINTER(_P)],
    "fqegpu_ham_destroy": [_P],
    "fqegpu_ham_info": [_P, _P],
    "fqegpu_ham_set_scratch_limit": [_P, _L],
    "fqegpu_ham_set_timing": [_P, _I],
    "fqegpu_ham_stage_ms": [_P, _P],
    "fqegpu_apply": [_P, _P, _P, _D, _D, _D, _D, _I, _P],
    "fqegpu_apply_host": [_P, _P, _P, _D, _D, _D, _D, _I],
    "fqegpu_ham_check": [_P, _P],
    "fqegpu_ham_set_tuning": [_P, _I, _I],
    "fqegpu_ham_test_injection": [_P, _L, _I],
    "fqegpu_debug_fail_allocs": [_I],
    "fqegpu_apply_noalloc": [_I, _I, _I, _P, _P, _P, _P, _D, _D, _D, _D, _P],
    "fqegpu_make_dvec": [_P, _P, _P, _P],
    "fqegpu_make_coeff": [_P, _P, _P, _I, _P],
    "fqegpu_diagonal_coulomb": [_P, _P, _P, _P, _I, _P],
    "fqegpu_axpy": [_L, _D, _D, _P, _P, _P],
    "fqegpu_scale": [_L, _D, _D, _P, _P],
    "fqegpu_vdot": [_L, _P, _P, _P, _P],
    "fqegpu_norm2": [_L, _P, _P, _P],
    "fqegpu_block_vdot": [_L, _I, _P, _P, _P, _P],
    "fqegpu_block_axpy": [_L, _I, _P, _P, _P, _P],
    "fqegpu_taylor": [_P, _P, _D, _D, _D, _D, _I, _I,
                      ctypes.POINTER(_I), _P],
    "fqegpu_diagonal": [_P, _P, _P],
    "fqegpu_rdm1": [_P, _P, _P, _P, _P],
    "fqegpu_rdm2_gram": [_P, _P, _P, _P, _P],
    "fqegpu_transform": [_P, _P, _P, _P, _P, _P],
    "fqegpu_evolve_diagonal": [_P, _P, _P, _P, _P],
    "fqegpu_batch_create": [_I, _P, _P, _P, _D, _D, _D, _D, _I, _P,
                            ctypes.POINTER(_P)],
    "fqegpu_batch_launch": [_P, _P],
    "fqegpu_batch_check": [_P, _P],
    "fqegpu_batch_destroy": [_P],
    "fqegpu_batch_taylor_create": [_I, _P, _P, _D, _D, _I, _I, _P,
                                   ctypes.POINTER(_P)],
    "fqegpu_batch_taylor_terms": [_P, _P, _P],
    "fqegpu_precondition": [_L, _P, _P, _D, _D, _P, _P],
    "fqegpu_mlp_create": [ctypes.POINTER(_P)],
    "fqegpu_mlp_destroy": [_P],
    "fqegpu_mlp_nparams": [],
    "fqegpu_mlp_set_params": [_P, _P, _L],
    "fqegpu_mlp_get_params": [_P, _P, _L],
    "fqegpu_mlp_get_grad": [_P, _P, _L],
    "fqegpu_mlp_precondition": [_P, _P, _P, _P, _D, _D, _D, _D, _P, _P],
    "fqegpu_mlp_multiplier": [_P, _P, _P, _D, _D, _D, _P, _P],
    "fqegpu_mlp_loss_grad": [_P, _P, _P, _P, _P, _P, _D, _D, _D, _I, _P, _P],
    "fqegpu_mlp_adam": [_P, _D, _D, _D, _D, _D, _P],
}

_lib = None


class FqeGpuError(RuntimeError):
    """Raised for CUDA-level failures of the library."""


def exported_symbols():
    return sorted(_SIGNATURES)


def load(path: str = LIB_PATH):
    """Load the shared library (no CUDA call is made)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FqeGpuError(
            f"libfqegpu.so not found at {path}: build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'`")
    lib = ctypes.CDLL(path)
    for name, args in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _I
    _lib = lib
    return lib


def last_error() -> str:
    buf = ctypes.create_string_buffer(1024)
    load().fqegpu_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(status: int, what: str = "") -> None:
    """Map an fqegpu_status to the exception type the reference raises."""
    if status == OK:
        return
    msg = f"{what}: {last_error()}" if what else last_error()
    if status == ERR_INVALID:
        raise ValueError(msg)
    if status == ERR_NOMEM:
        raise MemoryError(msg)
    if status == ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    if status == ERR_TIMEOUT:
        raise TimeoutError(msg)
    if status == ERR_NUMERIC:
        raise RuntimeError(msg)
    raise FqeGpuError(msg)


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args), name)
