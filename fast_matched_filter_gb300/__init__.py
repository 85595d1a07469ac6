"""GB300-native matched filter with the interface of fast_matched_filter.

    from fast_matched_filter_gb300 import matched_filter
    cc_sums = matched_filter(templates, moveouts, weights, data, step, arch="gpu")

The exported names mirror the reference package's
(fast_matched_filter/__init__.py:11-16).
"""
from .fast_matched_filter import (  # noqa: F401
    Batch,
    CPU_LOADED,
    last_precision,
    matched_filter,
    matched_filter_device,
    test_matched_filter,
)
from ._lib import FMFError  # noqa: F401
from .sharding import matched_filter_sharded, template_block  # noqa: F401
from .detection import (  # noqa: F401
    Detections,
    detect,
    matched_filter_detect,
    valid_lag_range,
)

__version__ = "0.1.0"


def __getattr__(name):
    # GPU_LOADED loads the library on first read (importing maps no native code)
    if name == "GPU_LOADED":
        from . import fast_matched_filter
        return fast_matched_filter.GPU_LOADED
    raise AttributeError("module %r has no attribute %r" % (__name__, name))
