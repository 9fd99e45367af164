"""GB300-native sweep-and-tiniest-queue broad phase.

The product is the native library libstq_gb300.so behind include/stq_abi.h;
this package holds its CUDA sources (csrc/), its build recipe (build.py) and
a thin Python binding (stq.py) used by the tests and the benchmark.
"""
from . import stq  # noqa: F401
from .stq import (AABB_DTYPE, Context, Mesh, STQError, SweepResult,  # noqa: F401
                  cloth_pair, crumpled_sheets, load_library, random_boxes)
