"""szx_gb300: SZx's blocked error-bounded codec on one GB300 (sm_103a).

The product is the native library libszx_gb300.so (CUDA kernels behind the C
ABI of include/szx_gb300.h); this package builds it (``build``) and exposes it
to Python (``api``).
"""
from .api import (ABS, FXR, NO_BLOCK, OPENMP, RANDOM_ACCESS, REL, SZx_DOUBLE, SZx_FLOAT, WITH_BLOCK,  # noqa: F401
                  DeviceCodec, SZxError, compress_blocked, compress_host, compute_data_length, compute_dimension,
                  compute_value_range, decompress_host, fast_compress_args, fast_decompress, filter_dimension)
