"""The C ABI library: loads, exports every declared symbol, behaves without a GPU (CPU only)."""
import re

import numpy as np
import pytest

from conftest import ROOT, kernel_spec, load_golden


def _declared():
    text = (ROOT / "include" / "morefit_cuda.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mf_[a-z0-9_]+)\s*\(", text)))


def test_header_symbols_exported():
    from morefit_gb300 import _lib as L
    declared = _declared()
    assert len(declared) >= 25
    for name in declared:
        assert hasattr(L.lib, name), f"{name} declared in morefit_cuda.h but not exported"
    assert sorted(L.exported_symbols()) == declared


def test_version_and_stride():
    from morefit_gb300 import _lib as L
    assert b"sm_103a" in L.lib.mf_version()
    assert L.lib.mf_column_stride(0) == 64
    assert L.lib.mf_column_stride(1) == 64
    assert L.lib.mf_column_stride(64) == 64
    assert L.lib.mf_column_stride(65) == 128
    assert L.lib.mf_column_stride(1000000) == 1000000


def test_no_device_is_an_error_not_a_crash():
    import ctypes as C
    from morefit_gb300 import _lib as L
    n = C.c_int(-1)
    assert L.lib.mf_device_count(C.byref(n)) == 0
    if n.value > 0:
        pytest.skip("a GPU is visible")
    h = L.c_ctx()
    rc = L.lib.mf_context_create(0, 0, C.byref(h))
    assert rc == L.MF_ERR_NO_DEVICE
    assert b"no CUDA device" in L.lib.mf_last_error()


def test_null_arguments_rejected():
    from morefit_gb300 import _lib as L
    assert L.lib.mf_kernel_reduce(None, None, 0, 0, None, 0, None) == L.MF_ERR_INVALID
    assert L.lib.mf_buffer_h2d(None, 0, None, 8) == L.MF_ERR_INVALID
    assert L.lib.mf_context_create(0, 0, None) == L.MF_ERR_INVALID
    assert L.lib.mf_kernel_reduce_segments_chunked(None, None, 0, 1, None, None, None, 0, 0, None) == L.MF_ERR_INVALID
    assert L.lib.mf_kernel_generate_splitmix_async(None, 1, 16, 100, 7, None, 0, None, 128, 0) == L.MF_ERR_INVALID
    assert L.lib.mf_context_set_resident(None, 2000) == L.MF_ERR_INVALID
    assert L.lib.mf_context_resident_stats(None, None, None, None, None) == L.MF_ERR_INVALID
    assert L.lib.mf_compile_check_resident(None, 1, None, None, None, 0) == L.MF_ERR_INVALID


def test_device_properties_without_a_device():
    import ctypes as C
    from morefit_gb300 import _lib as L
    n = C.c_int(-1)
    assert L.lib.mf_device_count(C.byref(n)) == 0
    if n.value > 0:
        pytest.skip("a GPU is visible")
    name = C.create_string_buffer(64)
    assert L.lib.mf_device_properties(0, name, 64, None, None, None) == L.MF_ERR_NO_DEVICE


@pytest.mark.parametrize("workload,kernel", [("pwave", "lh_grad_kernel"), ("mass", "lh_hessian_kernel")])
def test_parameter_buffers_match_reference(workload, kernel):
    """Host evaluation of hoisted parameter buffers equals the reference fitter's vectors."""
    from morefit_gb300.backend import eval_expressions
    g = load_golden(f"{workload}_n1000.json")
    bufs = {"lh_kernel": g["lh_buffers"], "lh_grad_kernel": g["grad_buffers"],
            "lh_hessian_kernel": g["hessian_buffers"]}[kernel]
    for pt in g["points"]:
        got = eval_expressions(g["parameters"], pt["params"], [e for _, e in bufs])
        ref = np.array(pt["kernel_params"][kernel][len(g["parameters"]):])
        np.testing.assert_allclose(got, ref, rtol=1e-12)


def test_expression_errors_are_reported():
    from morefit_gb300 import _lib as L
    from morefit_gb300.backend import eval_expressions
    with pytest.raises(L.MFError, match="PARSE"):
        eval_expressions(["a"], [1.0], ["a+unknown_name"])
    with pytest.raises(L.MFError, match="PARSE"):
        eval_expressions(["a"], [1.0], ["(a+1"])
    assert eval_expressions(["a"], [2.0], ["((a==0.0) ? 5.0 : 1.0/(a))"])[0] == 0.5
    assert eval_expressions(["a"], [0.0], ["((a==0.0) ? 5.0 : 1.0/(a))"])[0] == 5.0
    assert eval_expressions(["a"], [3.0], ["pow(a,2.000000000000000e+00)+-(a)"])[0] == 6.0
