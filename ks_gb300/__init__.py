"""GB300-native GSKS: general stride kernel summation on sm_103a.

The product is the C-ABI library ``ks_gb300/lib/libgsks.so`` (headers in
``include/ks.h`` and ``include/gsks.h``); this package is its Python host
interface (``ks_gb300.gsks``) and build recipe (``ks_gb300.build``).
"""
from .gsks import (  # noqa: F401
    KS_GAUSSIAN, KS_POLYNOMIAL, KS_LAPLACE, KS_GAUSSIAN_VAR_BANDWIDTH, KS_TANH,
    KS_QUARTIC, KS_MULTIQUADRATIC, KS_EPANECHNIKOV, GSKS_FP64, GSKS_SPLIT_BF16X3,
    GsksError, KsT, load, make_kernel, dgsks, dgsks_ref, dgsks_status, dgsks_ref_call,
    dgsks_device, dgsks_list, norms_device, set_precision, get_precision, last_error,
    last_launch_count, error_string,
)
