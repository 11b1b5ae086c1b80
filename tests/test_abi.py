"""The C-ABI library builds, loads and exports every entry point declared in include/qiw.h."""
import ctypes as C
import os
import re

from qiw import _lib, build

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "qiw.h")


def declared():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(qiw_[A-Za-z_0-9]+)\s*\(", text)))


def test_header_and_library_exports():
    lib = C.CDLL(build.build())
    names = declared()
    assert set(_lib.EXPORTS) <= set(names)
    for n in names:
        assert hasattr(lib, n), n


def test_ctx_create_reports_missing_device_without_crashing():
    import torch
    if torch.cuda.is_available():
        return
    lib = _lib.load()
    h = C.c_void_p()
    rc = lib.qiw_ctx_create(C.byref(h), 0)
    assert rc == _lib.QIW_ERR_CUDA and not h.value
    b = C.c_void_p()
    assert lib.qiw_batch_create(C.byref(b), 0) == _lib.QIW_ERR_CUDA and not b.value


def test_null_arguments_are_rejected():
    lib = _lib.load()
    assert lib.qiw_integrate(None, 0, None, 0, None) == _lib.QIW_ERR_ARG
    assert lib.qiw_problem_set(None, None) == _lib.QIW_ERR_ARG
    assert lib.qiw_last_error(None) == b"null context"
    assert lib.qiw_batch_add(None, None, None) == _lib.QIW_ERR_ARG
    assert lib.qiw_batch_run(None, 0, 0, None, 0) == _lib.QIW_ERR_ARG
    assert lib.qiw_batch_last_error(None) == b"null batch"
    assert lib.qiw_integrate_samples_batch(None, 1, None, 0, None, None) == _lib.QIW_ERR_ARG
    assert lib.qiw_integrate_sample_norms(None, 1, None, 0, None, None) == _lib.QIW_ERR_ARG
    assert lib.qiw_warp_train_batch(None, 1, None, None, None, None, 10, 64, 1e-3, None) == _lib.QIW_ERR_ARG


def test_plan_cache_calls_need_no_device():
    """qiw_plan_cache_info / qiw_plan_cache_clear touch host memory only."""
    lib = _lib.load()
    assert lib.qiw_plan_cache_clear() == _lib.QIW_OK
    e, h, b = C.c_int64(-1), C.c_int64(-1), C.c_int64(-1)
    assert lib.qiw_plan_cache_info(C.byref(e), C.byref(h), C.byref(b)) == _lib.QIW_OK
    assert e.value == 0 and b.value == 0 and h.value >= 0
    assert lib.qiw_plan_cache_info(None, None, None) == _lib.QIW_OK
