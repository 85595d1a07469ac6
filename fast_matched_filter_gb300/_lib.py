"""ctypes binding of libfmf_gb300.so (the C ABI declared in include/fmf_gb300.h).

The reference binds its GPU library the same way
(fast_matched_filter/fast_matched_filter.py:19-63); the argument list of
``fmf_matched_filter`` is the reference's 13 + 2 arguments
(matched_filter.cu:171-176).  Loading fails loudly: there is no CPU
fallback in this package.
"""
import ctypes as ct
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libfmf_gb300.so")

FMF_OK = 0
FMF_ERR_ARG = 1
FMF_ERR_OOM = 2
FMF_ERR_SMEM = 3
FMF_ERR_CUDA = 4
FMF_ERR_TIMEOUT = 5
FMF_ERR_UNSUPPORTED = 6
STATUS_NAMES = {0: "OK", 1: "BAD_ARG", 2: "OOM", 3: "SMEM", 4: "CUDA_ERR",
                5: "TIMEOUT", 6: "UNSUPPORTED"}

PREC_FP32 = 0
PREC_SPLIT_BF16 = 1
PREC_BF16 = 2
PREC_AUTO = 3  # split bf16 where its error model allows 1e-5, else fp32
PRECISIONS = {"fp32": PREC_FP32, "split_bf16": PREC_SPLIT_BF16, "bf16": PREC_BF16,
              "auto": PREC_AUTO}
PRECISION_NAMES = {v: k for k, v in PRECISIONS.items()}

FLAG_DEVICE_POINTERS = 1


def flag_tile(lag_blocks):
    """FMF_FLAG_TILE: tensor-core lag blocks per tile (0 = library choice)."""
    return ((int(lag_blocks) // 16) & 0xFF) << 8


def flag_template_group(n):
    """FMF_FLAG_TEMPLATE_GROUP: templates interleaved per group of tile-queue items."""
    return (int(n) & 0xFF) << 16


def flag_precision(precision):
    """FMF_FLAG_PRECISION: numerator precision of fmf_matched_filter_variable_ex."""
    return (PRECISIONS[precision] & 3) << 24

_fp = ct.POINTER(ct.c_float)
_ip = ct.POINTER(ct.c_int)
_sz = ct.c_size_t
ARGTYPES = [_fp, _fp, _ip, _fp, _fp, _sz, _sz, _sz, _sz, _sz, _sz, _sz, _fp, ct.c_int, ct.c_int]
# same 15 arguments, then precision, flags, stream -- addresses as integers
ARGTYPES_EX = [ct.c_void_p] * 5 + [_sz] * 7 + [ct.c_void_p, ct.c_int, ct.c_int,
                                               ct.c_int, ct.c_int, ct.c_void_p]

# every symbol declared in include/fmf_gb300.h
EXPORTS = ("fmf_matched_filter", "matched_filter", "fmf_matched_filter_ex",
           "fmf_last_error", "fmf_version", "fmf_last_launch_count",
           "fmf_release_cache", "fmf_timing_begin", "fmf_timing_end", "fmf_timing_end_ex",
           "fmf_device_errors", "fmf_matched_filter_noalloc", "fmf_batch_create",
           "fmf_batch_add", "fmf_batch_set_tiles", "fmf_batch_run", "fmf_batch_launch_count",
           "fmf_batch_destroy", "fmf_selftest_wait_timeout", "fmf_matched_filter_variable",
           "fmf_matched_filter_variable_ex", "fmf_detect", "fmf_matched_filter_detect",
           "fmf_template_energies", "fmf_matched_filter_check_zeros", "fmf_eval_atanh",
           "fmf_last_precision", "fmf_measure_fp32_fma")

DETECT_CAPACITY = 16384  # FMF_DETECT_CAPACITY
# detection arguments after the rows: n_mad, min_separation, max_detections, six outputs,
# flags, stream
_DETECT_TAIL = [ct.c_float, _sz, _sz] + [ct.c_void_p] * 6 + [ct.c_int, ct.c_void_p]
ARGTYPES_DETECT = [ct.c_void_p, _sz, _sz, ct.c_void_p, ct.c_void_p] + _DETECT_TAIL
ARGTYPES_SEARCH_DETECT = [ct.c_void_p] * 5 + [_sz] * 7 + [ct.c_int, ct.c_int] + _DETECT_TAIL


class FMFError(RuntimeError):
    """A non-zero status returned by the library."""

    def __init__(self, status, message):
        self.status = status
        super().__init__("fmf_gb300 status %d (%s): %s"
                         % (status, STATUS_NAMES.get(status, "?"), message))


_lib = None
_load_error = None


def load(path=None):
    """Load (once) and return the library; raise OSError if it is missing."""
    global _lib, _load_error
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    lib = ct.CDLL(p)
    lib.fmf_matched_filter.argtypes = ARGTYPES
    lib.fmf_matched_filter.restype = ct.c_int
    lib.matched_filter.argtypes = ARGTYPES
    lib.matched_filter.restype = ct.c_int
    lib.fmf_matched_filter_ex.argtypes = ARGTYPES_EX
    lib.fmf_matched_filter_ex.restype = ct.c_int
    lib.fmf_last_error.argtypes = [ct.c_char_p, _sz]
    lib.fmf_last_error.restype = ct.c_int
    lib.fmf_version.restype = ct.c_char_p
    lib.fmf_last_launch_count.restype = ct.c_int
    lib.fmf_last_precision.restype = ct.c_int
    lib.fmf_measure_fp32_fma.argtypes = [ct.POINTER(ct.c_double)]
    lib.fmf_measure_fp32_fma.restype = ct.c_int
    lib.fmf_release_cache.restype = ct.c_int
    lib.fmf_timing_begin.restype = ct.c_int
    lib.fmf_device_errors.restype = ct.c_int
    lib.fmf_selftest_wait_timeout.argtypes = [ct.c_uint]
    lib.fmf_matched_filter_variable_ex.argtypes = [ct.c_void_p] * 5 + [_sz, ct.c_void_p] + [_sz] * 5 + [
        ct.c_void_p, ct.c_int, ct.c_int, ct.c_void_p]
    lib.fmf_matched_filter_variable_ex.restype = ct.c_int
    lib.fmf_selftest_wait_timeout.restype = ct.c_int
    lib.fmf_batch_create.argtypes = [ct.POINTER(ct.c_void_p), ct.c_int]
    lib.fmf_batch_create.restype = ct.c_int
    lib.fmf_batch_add.argtypes = [ct.c_void_p] + ARGTYPES_EX[:15]
    lib.fmf_batch_add.restype = ct.c_int
    lib.fmf_batch_set_tiles.argtypes = [ct.c_void_p, ct.c_int, ct.c_int]
    lib.fmf_batch_set_tiles.restype = ct.c_int
    lib.fmf_batch_run.argtypes = [ct.c_void_p, ct.c_void_p]
    lib.fmf_batch_run.restype = ct.c_int
    lib.fmf_batch_launch_count.argtypes = [ct.c_void_p]
    lib.fmf_batch_launch_count.restype = ct.c_int
    lib.fmf_batch_destroy.argtypes = [ct.c_void_p]
    lib.fmf_batch_destroy.restype = ct.c_int
    lib.fmf_timing_end.argtypes = [ct.POINTER(ct.c_double), ct.POINTER(ct.c_double),
                                   ct.POINTER(ct.c_int)]
    lib.fmf_timing_end.restype = ct.c_int
    lib.fmf_timing_end_ex.argtypes = [ct.POINTER(ct.c_double), ct.c_int, ct.POINTER(ct.c_int)]
    lib.fmf_timing_end_ex.restype = ct.c_int
    lib.fmf_detect.argtypes = ARGTYPES_DETECT
    lib.fmf_detect.restype = ct.c_int
    lib.fmf_matched_filter_detect.argtypes = ARGTYPES_SEARCH_DETECT
    lib.fmf_matched_filter_detect.restype = ct.c_int
    lib.fmf_matched_filter_check_zeros.argtypes = ARGTYPES_EX + [ct.c_longlong, ct.c_void_p]
    lib.fmf_matched_filter_check_zeros.restype = ct.c_int
    lib.fmf_template_energies.argtypes = [ct.c_void_p, _sz, _sz, ct.c_void_p, ct.c_int, ct.c_void_p]
    lib.fmf_template_energies.restype = ct.c_int
    lib.fmf_eval_atanh.argtypes = [ct.c_void_p, ct.c_void_p, _sz, ct.c_void_p]
    lib.fmf_eval_atanh.restype = ct.c_int
    if path is None:
        _lib = lib
    return lib


def try_load():
    """Load the library if it exists; return (lib or None, error text)."""
    global _load_error
    try:
        return load(), None
    except (OSError, AttributeError) as e:  # not built, stale, or not loadable here
        _load_error = str(e)
        return None, _load_error


def last_error(lib=None):
    lib = lib or load()
    buf = ct.create_string_buffer(512)
    st = lib.fmf_last_error(buf, 512)
    return st, buf.value.decode(errors="replace")


def check(status, lib=None):
    if status != FMF_OK:
        _, msg = last_error(lib)
        raise FMFError(status, msg)
