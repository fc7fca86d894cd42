"""sw2d -- GB300-native SW2D shallow-water time-stepping core.

Python front end of libsw2d.so (C ABI in include/sw2d.h).  The numerical
work runs in hand-written sm_103a CUDA kernels; this package only binds the
ABI, builds synthetic scenarios and drives runs.
"""
from .native import (  # noqa: F401
    DT_CFL, DT_FIXED, KERNEL_AUTO, KERNEL_STREAM, KERNEL_TILE, FIELD_DEPTH, FIELD_ELEVATION, FIELD_UM, FIELD_UU, FIELD_VN, FIELD_VV,
    PREC_F32, PREC_F64, RAIN_COMPAT, RAIN_LINEAR, RAIN_NONE, RAIN_STEP, RAIN_STORM,
    REQ_CANCELLED, REQ_DONE, REQ_FAILED, REQ_PENDING, REQ_RUNNING, REQ_UNKNOWN,
    Batch, BatchConfig, Config, ServerConfig, ServerHandle, SW2DError, Solver, batch_config, batch_scenario_bytes,
    default_config, device_bytes, evaporation_series, load, server_config,
)
