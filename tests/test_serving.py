"""Serving loop: coalesced evaluations of concurrent fits (GPU).

Every result must be the same alone and in the mix: the batched launches
give bit-identical sums per evaluation, so a fit's trajectory does not depend
on which other fits share its launches. The bar is exact equality of the
fitted values and errors.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def server():
    from morefit_gb300.backend import CUDABackend
    from morefit_gb300.serving import FitServer
    b = CUDABackend(0)
    yield FitServer(b, hbm_budget=8 << 30, max_active=64)
    b.close()


def _requests():
    from morefit_gb300.serving import FitRequest
    sizes = [3000, 52000, 7100, 20000, 140000, 1000, 33000, 9000]
    models = ["mass", "spwave", "mass", "spwave", "mass", "mass", "spwave", "spwave"]
    return [FitRequest(i, m, n, 1234 + i) for i, (m, n) in enumerate(zip(models, sizes))]


def test_results_same_alone_and_in_the_mix(server):
    mix = {o.id: o for o in server.run(_requests(), realtime=False).outcomes}
    assert len(mix) == 8
    for r in _requests():
        alone = server.run([r], realtime=False).outcomes[0]
        assert np.array_equal(alone.values, mix[r.id].values), r
        assert np.array_equal(alone.errors, mix[r.id].errors), r
        assert alone.evaluations == mix[r.id].evaluations


def test_fits_converge_near_truth(server):
    from morefit_gb300.workloads import load_spec
    out = server.run(_requests(), realtime=False).outcomes
    for o in out:
        truth = np.array(load_spec(o.model)["truth"])
        assert o.converged, o
        assert np.all(np.abs(o.values - truth) < 6.0 * o.errors), (o.model, o.nevents, (o.values - truth) / o.errors)


def test_admission_respects_the_budget(server):
    """With room for about two of the larger datasets, fits wait for memory
    to free up, never exceed the budget, and give the same results."""
    from morefit_gb300.serving import FitServer
    small = FitServer(server.backend, hbm_budget=int(60e6), max_active=64)
    small.models = server.models
    st = small.run(_requests(), realtime=False)
    assert st.peak_bytes <= 60e6 or st.max_active == 1
    ref = {o.id: o for o in server.run(_requests(), realtime=False).outcomes}
    for o in st.outcomes:
        assert np.array_equal(o.values, ref[o.id].values)


@pytest.mark.parametrize("model,n", [("mass", 70001), ("spwave", 5000)])
def test_device_seeded_generation_equals_seed_table(server, model, n):
    """A request's dataset is generated with its streams seeded on the device
    (mf_kernel_generate_splitmix_async): the events equal, bit for bit, those
    generated from the seed table splitmix_seed_rows builds on the host."""
    from morefit_gb300.workloads import splitmix_seed_rows
    gen = server.models[model].gen
    nseeds = int(min(65536, n))
    gen.SetNevents(n)
    gen.SubmitGenerateSplitmixAsync(99, nseeds, -(-n // nseeds))
    a = gen.output.download()
    gen.CopyToSeedBuffer(splitmix_seed_rows(nseeds, 99))
    gen.SetNevents(n)
    gen.SubmitKernelAsync(-(-n // nseeds))
    b = gen.output.download()
    assert a.shape == b.shape and np.array_equal(a, b)
