"""The names of mpx/utils/mpc_wrapper_srbd.py, so that a caller switches by
its import line alone:

    # from mpx.utils.mpc_wrapper_srbd import BatchedMPCControllerWrapper
    from mpx_gb300.mpc_wrapper_srbd import BatchedMPCControllerWrapper

BatchedMPCControllerWrapper is the batched SRBD controller
(mpc_wrapper_srbd.py:19-175: run, torch_run, whole_body_run,
torch_whole_body_run, reset), the class of mpx_gb300.wrappers.
"""
from .wrappers import BatchedMPCControllerWrapper

__all__ = ["BatchedMPCControllerWrapper"]
