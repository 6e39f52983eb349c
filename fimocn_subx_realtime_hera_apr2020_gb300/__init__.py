"""GB300 implementation of FIM's horizontal dynamics step.

The compute path is libfimgpu.so (hand-written CUDA for sm_103a behind the
C-ABI of include/fim_gpu.h); this package is its host-side mirror of the
reference interface: grid tables, configuration, synthetic states and the
per-routine / fused-step calls.
"""
from .config import FimConfig, WORKLOADS, default_dt, vertical_tables  # noqa: F401
from .grid import Grid  # noqa: F401
from .dycore import Dycore, DycoreState, FIELDS  # noqa: F401
from .state import synthetic_state, synthetic_state_device  # noqa: F401
