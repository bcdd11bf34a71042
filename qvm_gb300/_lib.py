"""ctypes binding of libqvmgpu.so (declared in include/qvmgpu.h).

The library is built in-tree by ``qvm_gb300.build``; there is no fallback:
if the shared library is missing or a call fails, an exception is raised.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libqvmgpu.so")

FP64 = 0
FP32 = 1
MEASURE_INTERPRETED = 0
MEASURE_COMPILED = 1
SAMPLE_BISECT = 0
SAMPLE_CDF = 1
RUN_PLAIN = 0
RUN_FUSED = 1

_i = ctypes.c_int
_ip = ctypes.POINTER(ctypes.c_int)
_dp = ctypes.POINTER(ctypes.c_double)
_u64 = ctypes.c_uint64
_u64p = ctypes.POINTER(ctypes.c_uint64)
_i64p = ctypes.POINTER(ctypes.c_int64)
_vp = ctypes.c_void_p
_vpp = ctypes.POINTER(ctypes.c_void_p)

# name -> (restype, argtypes); every entry point of include/qvmgpu.h
SIGNATURES = {
    "qvmg_last_error": (ctypes.c_char_p, []),
    "qvmg_abi_version": (_i, []),
    "qvmg_debug_fail_alloc": (_i, [_i]),
    "qvmg_debug_tc_withhold": (_i, [_i]),
    "qvmg_device_info": (_i, [_ip, _u64p, _u64p]),
    "qvmg_state_bytes": (_u64, [_i, _i]),
    "qvmg_state_create": (_i, [_i, _i, _vpp]),
    "qvmg_state_free": (_i, [_vp]),
    "qvmg_state_info": (_i, [_vp, _ip, _ip]),
    "qvmg_state_set_priority": (_i, [_vp, _i]),
    "qvmg_device_reserve": (_i, [_u64]),
    "qvmg_state_reset": (_i, [_vp]),
    "qvmg_state_upload": (_i, [_vp, _dp]),
    "qvmg_state_download": (_i, [_vp, _dp]),
    "qvmg_state_copy": (_i, [_vp, _vp]),
    "qvmg_state_sync": (_i, [_vp]),
    "qvmg_apply_dense": (_i, [_vp, _i, _ip, _dp]),
    "qvmg_apply_permutation": (_i, [_vp, _i, _ip, _i64p]),
    "qvmg_apply_diagonal": (_i, [_vp, _i, _ip, _dp]),
    "qvmg_prob_excited": (_i, [_vp, _i, _dp]),
    "qvmg_prob_ground": (_i, [_vp, _i, _dp]),
    "qvmg_force_measurement": (_i, [_vp, _i, _i, ctypes.c_double]),
    "qvmg_measure": (_i, [_vp, _i, ctypes.c_double, _i, _ip, _ip, _dp]),
    "qvmg_measure_all": (_i, [_vp, ctypes.c_double, _u64p]),
    "qvmg_sample": (_i, [_vp, _dp, _u64, _i, _u64p]),
    "qvmg_sample_noalloc": (_i, [_vp, _i, _i, _vp, _u64, _i, _vp, _vp]),
    "qvmg_probabilities": (_i, [_vp, _dp]),
    "qvmg_marginal_probabilities": (_i, [_vp, _i, _ip, _dp]),
    "qvmg_reduced_density_matrix": (_i, [_vp, _i, _ip, _dp]),
    "qvmg_density_diagonal": (_i, [_vp, _dp]),
    "qvmg_apply_kraus": (_i, [_vp, _i, _ip, _i, _dp, ctypes.c_double, _ip, _dp]),
    "qvmg_measure_sequence": (_i, [_vp, _i, _ip, _i, _i, _dp, _u64, _vp, _u64p]),
    "qvmg_wavefunction_octets": (_i, [_vp, _vp]),
    "qvmg_probabilities_octets": (_i, [_vp, _vp]),
    "qvmg_norm": (_i, [_vp, _dp]),
    "qvmg_normalize": (_i, [_vp]),
    "qvmg_inner": (_i, [_vp, _vp, _dp, _dp]),
    "qvmg_fidelity": (_i, [_vp, _vp, _dp, _dp]),
    "qvmg_program_create": (_i, [_vpp]),
    "qvmg_program_free": (_i, [_vp]),
    "qvmg_program_add_dense": (_i, [_vp, _i, _ip, _dp]),
    "qvmg_program_add_dense_many": (_i, [_vp, _i, _ip, _ip, _dp]),
    "qvmg_program_add_permutation": (_i, [_vp, _i, _ip, _i64p]),
    "qvmg_program_add_diagonal": (_i, [_vp, _i, _ip, _dp]),
    "qvmg_program_num_ops": (_i, [_vp, _ip]),
    "qvmg_program_plan": (_i, [_vp, _i, _i, _i, _i, _i, _ip]),
    "qvmg_program_plan_stats": (_i, [_vp, _i64p, _i]),
    "qvmg_program_set_option": (_i, [_vp, _i, _i]),
    "qvmg_program_plan_describe": (_i, [_vp, ctypes.c_char_p, _u64, _u64p]),
    "qvmg_program_run": (_i, [_vp, _vp, _i]),
    "qvmg_program_run_profiled": (_i, [_vp, _vp, _i, ctypes.POINTER(ctypes.c_float), _ip, _i, _ip]),
    "qvmg_state_stream": (_i, [_vp, _vpp]),
    "qvmg_qaoa_batch_create": (_i, [_i, _ip, _ip, _ip, _i, _dp, _dp, _vpp]),
    "qvmg_qaoa_batch_set_angles": (_i, [_vp, _dp, _dp]),
    "qvmg_qaoa_batch_run": (_i, [_vp, _dp, _i, _dp, ctypes.POINTER(ctypes.c_uint32)]),
    "qvmg_qaoa_batch_state": (_i, [_vp, _i, _dp]),
    "qvmg_qaoa_batch_bytes": (_u64, [_vp]),
    "qvmg_qaoa_batch_free": (_i, [_vp]),
    "qvmg_sbatch_create": (_i, [_i, _i, _ip, _ip, _ip, _ip, _dp, _ip, _vpp]),
    "qvmg_sbatch_run": (_i, [_vp, _dp, _u64p]),
    "qvmg_sbatch_shot_offset": (_i, [_vp, _i, _u64p]),
    "qvmg_sbatch_state": (_i, [_vp, _i, _dp]),
    "qvmg_sbatch_bytes": (_u64, [_vp]),
    "qvmg_sbatch_free": (_i, [_vp]),
}

STATUS = {
    1: "invalid argument",
    2: "CUDA error",
    3: "out of device memory",
    4: "probability out of range",
    5: "unsupported",
    6: "device wait timed out",
}


class QVMGError(RuntimeError):
    """A libqvmgpu call returned a nonzero status."""

    def __init__(self, code: int, message: str):
        super().__init__(f"{STATUS.get(code, 'error')} ({code}): {message}")
        self.code = code


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is not built; run `python -m qvm_gb300.build` "
                "(the statevector engine has no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(rc: int):
    if rc != 0:
        msg = lib().qvmg_last_error()
        raise QVMGError(rc, msg.decode() if msg else "")
    return rc


def call(name: str, *args):
    return check(getattr(lib(), name)(*args))
