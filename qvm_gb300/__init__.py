"""qvm_gb300: a GB300 (sm_103a) statevector engine for the QVM's pure-state path.

The compute lives in ``libqvmgpu.so`` (C ABI, include/qvmgpu.h); this
package is the host-side mirror of the reference's pure-state API.
"""
from ._lib import QVMGError  # noqa: F401
from .state import CudaPureState, Program, device_info, state_bytes  # noqa: F401
from .qvm import PureStateQVM, make_qvm, run_program  # noqa: F401

__all__ = ["QVMGError", "CudaPureState", "Program", "PureStateQVM", "make_qvm",
           "run_program", "device_info", "state_bytes"]
