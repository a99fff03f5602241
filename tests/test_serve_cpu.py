"""Host logic of the serving driver (fall3d_gb300/serve.py) that needs no
GPU: the single-server FIFO that turns the measured FP64 service times of
the requests into their latencies on the same arrivals."""
import numpy as np

from fall3d_gb300 import serve


def test_fifo_latencies():
    # idle server: each request is served on arrival
    lat, fin = serve.fifo_latencies([0.0, 10.0, 20.0], [1.0, 2.0, 3.0])
    assert lat.tolist() == [1.0, 2.0, 3.0] and fin == 23.0
    # a queue builds up: the second waits for the first, the third for both
    lat, fin = serve.fifo_latencies([0.0, 1.0, 2.0], [5.0, 5.0, 5.0])
    assert lat.tolist() == [5.0, 9.0, 13.0] and fin == 15.0
    # against a direct simulation on random arrivals
    rng = np.random.default_rng(3)
    arr = np.cumsum(rng.exponential(0.5, 200))
    svc = rng.uniform(0.1, 1.5, 200)
    lat, fin = serve.fifo_latencies(arr, svc)
    free = 0.0
    for i in range(200):
        start = max(free, arr[i])
        free = start + svc[i]
        assert abs(lat[i] - (free - arr[i])) < 1e-9
    assert abs(fin - free) < 1e-9
    assert np.all(lat >= svc - 1e-12)
    assert serve.fifo_latencies([], [])[0].size == 0
