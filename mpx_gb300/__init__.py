"""mpx_gb300: GB300-native batched primal-dual iLQR MPC (SRBD hot path)."""
from .problem import (MODEL_BIPED_WRENCH12, MODEL_GENERIC_LQ, MODEL_SRBD_QUAT13, MODEL_SRBD_RPY12, ModelDesc,
                      SolverOptions)
