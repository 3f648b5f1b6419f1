"""canvas_ity_gb300 -- a GB300-native rasteriser behind the canvas_ity API.

The C++ drop-in (`include/canvas_ity.hpp`, implemented in
`canvas_ity_gb300/csrc/`) records drawing state on the host and renders with
hand-written sm_103a CUDA kernels.  This Python package builds the shared
library, loads it, and drives it with recorded call lists (`trace`), seeded
benchmark scenes (`scenes`), the batched many-canvas engine and the serving
loop.  The library is loaded lazily; every entry point raises if the CUDA
library is missing -- there is no CPU fallback.
"""
from . import trace  # noqa: F401
