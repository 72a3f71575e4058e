"""Shared fixtures. GPU tests carry @pytest.mark.gpu; everything else runs on CPU."""
import json
import os
import platform
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"
ARCH = platform.machine()


def reference_sources():
    """The reference sources the C++ drop-in compiles against: the tree named by
    MOREFIT_REFERENCE, else the copy staged by `make -C oracle stage` (which
    travels with the working tree to hosts that have no reference tree), else None."""
    env = os.environ.get("MOREFIT_REFERENCE")
    if env and (Path(env) / "include" / "fitter.hh").exists():
        return Path(env)
    staged = ROOT / "oracle" / "_ref" / "src"
    return staged if (staged / "include" / "fitter.hh").exists() else None


def build_dropin() -> Path:
    """Builds Minuit2, the oracle kit and tests/cpp/_build/<arch>/dropin from the reference sources."""
    from morefit_gb300.build import build_library
    build_library()
    jobs = f"-j{os.cpu_count() or 4}"
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "ref", jobs], check=True)
    subprocess.run(["make", "-s", "-C", str(ROOT / "tests" / "cpp"), jobs], check=True)
    return ROOT / "tests" / "cpp" / "_build" / ARCH / "dropin"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU (sm_103)")


def load_golden(name: str) -> dict:
    return json.loads((GOLDEN / name).read_text())


def golden_events(workload: str, n: int) -> np.ndarray:
    raw = np.fromfile(GOLDEN / f"{workload}_n{n}_events.f64", dtype=np.float64)
    ndim = len(load_golden(f"{workload}_n{n}.json")["dimensions"])
    return raw.reshape(ndim, n)


def kernel_spec(g: dict, name: str) -> dict:
    return {k["name"]: k for k in g["kernels"]}[name]


def assert_sums_close(got, ref, abs_scale, rtol=1e-10, stol=1e-12, what=""):
    """|got - ref| <= rtol*|ref| + stol*sum_i|x_i| per output.

    abs_scale[j] = sum over events of |per-event value of output j|; the stol
    term bounds summation-order differences, which scale with it."""
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    tol = rtol * np.abs(ref) + stol * np.asarray(abs_scale, dtype=np.float64)
    bad = ~(np.abs(got - ref) <= tol)  # NaN counts as a mismatch
    assert not bad.any(), (f"{what}: outputs {np.nonzero(bad)[0].tolist()} differ: got {got[bad]}, "
                           f"ref {ref[bad]}, |diff| {np.abs(got - ref)[bad]}, tol {tol[bad]}")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import mforacle
    mforacle.build()
    return mforacle
