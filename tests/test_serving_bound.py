"""The ideal-server model the bench's serving section reports beside each
load level (bench.fluid_latencies, bench.fluid_max_load): worked cases by
hand, and the properties the bound relies on; and the wrapper that keeps
the garbage collector off while that section submits (bench._without_gc)."""
import numpy as np

import bench


def test_fifo_by_hand():
    # 1 ms of work at 0, 1 ms at 0.5 ms, 2 us at 1 ms
    lat = bench.fluid_latencies([0.0, 0.5e-3, 1e-3], [16000, 16000, 32], 16e6, "fifo")
    assert np.allclose(lat, [1e-3, 1.5e-3, 1.002e-3])


def test_srpt_by_hand():
    # the 2-us request preempts the waiting 1-ms one; the running request
    # keeps the server while its remaining work is the least
    lat = bench.fluid_latencies([0.0, 0.5e-3, 1e-3], [16000, 16000, 32], 16e6, "srpt")
    assert np.allclose(lat, [1e-3, 1.502e-3, 2e-6])


def test_properties_on_a_heavy_tailed_stream():
    rng = np.random.default_rng(1)
    rate = 16e6
    sizes = np.floor(np.exp(rng.uniform(0, np.log(20000), 3000))) + 1
    arr = np.cumsum(rng.exponential(sizes.mean() / (0.8 * rate), 3000))
    fifo = np.array(bench.fluid_latencies(arr, sizes, rate, "fifo"))
    srpt = np.array(bench.fluid_latencies(arr, sizes, rate, "srpt"))
    own = sizes / rate
    assert (fifo >= own - 1e-12).all() and (srpt >= own - 1e-12).all()
    assert srpt.mean() <= fifo.mean()
    # both policies are work-conserving: the last completion is the same
    assert np.isclose((arr + fifo).max(), (arr + srpt).max())


def test_max_load():
    # equal small requests: the queue stays short almost to full load
    assert bench.fluid_max_load([32] * 10, 16e6)["fifo"] > 0.95
    # requests that alone take longer than the target never meet it
    assert bench.fluid_max_load([64000] * 10, 16e6) == {"fifo": 0.0, "srpt": 0.0}


def test_without_gc_restores_the_collector():
    import gc

    @bench._without_gc
    def inside(fail=False):
        if fail:
            raise ValueError("x")
        return gc.isenabled()

    assert gc.isenabled()
    assert inside() is False and gc.isenabled()
    try:
        inside(fail=True)
    except ValueError:
        pass
    assert gc.isenabled()
