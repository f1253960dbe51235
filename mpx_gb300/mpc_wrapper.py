"""The names of mpx/utils/mpc_wrapper.py, so that a caller switches by its
import line alone:

    # from mpx.utils.mpc_wrapper import BatchedMPCControllerWrapper, MPCControllerWrapper, mpx_data
    from mpx_gb300.mpc_wrapper import BatchedMPCControllerWrapper, MPCControllerWrapper, mpx_data

BatchedMPCControllerWrapper is the data-record form (make_data / run(data,
x0, input) / reset, mpc_wrapper.py:29-192), MPCControllerWrapper the single
instance (mpc_wrapper.py:194-468), mpx_data the record (mpc_wrapper.py:16-27).
The classes are those of mpx_gb300.wrappers.
"""
from .wrappers import BatchedDataMPCWrapper as BatchedMPCControllerWrapper
from .wrappers import MPCControllerWrapper, mpx_data

__all__ = ["BatchedMPCControllerWrapper", "MPCControllerWrapper", "mpx_data"]
