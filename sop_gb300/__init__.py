"""sop_gb300 -- a GB300-native (sm_103a) SOP coarse-grained molecular-dynamics engine.

The compute path is the CUDA library libsopgpu.so behind the C ABI in
include/sop_gpu.h; this package holds its Python binding (engine), the
molecule topology and the reference's input files (system), the reference's
output files (outputs), and the build recipe (build).
"""
from .system import Molecule, generate, ensemble_spec, request_stream  # noqa: F401

__all__ = ["Molecule", "generate", "ensemble_spec", "request_stream"]
