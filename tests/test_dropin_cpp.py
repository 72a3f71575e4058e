"""include/compute_cuda.hh under the reference's unchanged fitter (CPU only).

The drop-in C++ backend is compiled against the reference's own headers and
vendored Minuit2 (tests/cpp/Makefile; only where the reference sources are
present: MOREFIT_REFERENCE or the copy staged under oracle/_ref/src).
Without a GPU the reference fitter's make_kernels still drives every
MakeComputeKernel call, and the backend prints the CUDA source it lowers
(print_kernel). That source must be byte-identical to what the C ABI lowers
from the frozen kernel specs, which are the kernels the GPU tests run: the
C++ drop-in and the GPU-tested path build the same kernels.
"""
import subprocess

import pytest

from conftest import build_dropin, kernel_spec, load_golden, reference_sources

pytestmark = pytest.mark.skipif(reference_sources() is None, reason="reference sources not present")


@pytest.fixture(scope="module")
def dropin():
    return build_dropin()


def _sources(text):
    out = []
    for chunk in text.split("CUDA KERNEL SOURCECODE:\n")[1:]:
        out.append(chunk.split("END KERNEL SOURCECODE")[0])
    return out


@pytest.mark.parametrize("workload", ["pwave", "mass"])
def test_cpp_dropin_builds_the_gpu_tested_kernels(dropin, workload):
    from morefit_gb300 import _lib as L
    from morefit_gb300.backend import lower_source
    r = subprocess.run([str(dropin), "lower", workload], capture_output=True, text=True, check=True)
    got = _sources(r.stdout)
    g = load_golden(f"{workload}_n1000.json")
    names = (["precompute_kernel"] if workload == "pwave" else []) + ["lh_kernel", "lh_grad_kernel",
                                                                      "lh_hessian_kernel"]
    assert len(got) == len(names)
    for src, name in zip(got, names):
        k = kernel_spec(g, name)
        kind = L.MF_KERNEL_STORE if name == "precompute_kernel" else L.MF_KERNEL_REDUCE
        want = lower_source(name, kind, L.MF_F64, k["inputs"], k["params"], k["exprs"])
        assert src == want, f"{workload}/{name}: C++ drop-in lowers a different kernel"
