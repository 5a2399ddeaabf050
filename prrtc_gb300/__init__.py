"""GB300-native (sm_103a) implementation of pRRTC's GPU RRT-Connect hot path.

The product is the shared library ``libprrtc_gb300.so`` (C ABI in
``include/prrtc/prrtc.h``); ``api`` is its Python host mirror.
"""
from .api import (Batch, BatchSettings, Context, EnvHandle, PlannerResult, PrrtcError, Settings,  # noqa: F401
                  SmoothSettings, dof, num_spheres, robot_id)
from .env import Environment  # noqa: F401
