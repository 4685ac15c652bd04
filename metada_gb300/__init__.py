"""metada_gb300: GB300-native (sm_103a) ensemble Kalman analysis for METADA.

The compute path is the CUDA library libmetada_gb300.so behind the C-ABI in
include/metada_gb300.h; this package holds its build recipe, a ctypes
binding, tensor-level wrappers (kernels), the reference-interface mirror
(algorithms) and the seeded synthetic-input generators.
"""

__version__ = "0.1.0"
