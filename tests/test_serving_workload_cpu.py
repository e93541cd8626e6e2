"""The serving workload's definition (no GPU): a 1024-input net of 120 layers
at 3 % density with N(0, 0.3^2) values and a dense 1024 x 10 head, U[0, 1)
inputs, seeded Poisson arrivals at 2000 requests/s with sizes log-uniform in
[1, 4096] -- the shape the serving loop is measured on."""
import numpy as np

from snicit_gb300.serving import mlp_inputs, request_stream, sparse_mlp


def test_request_stream_is_seeded_poisson_with_log_uniform_sizes():
    a1, s1 = request_stream(7, 20000)
    a2, s2 = request_stream(7, 20000)
    assert np.array_equal(a1, a2) and np.array_equal(s1, s2)   # seeded
    assert not np.array_equal(request_stream(8, 20000)[1], s1)
    assert np.all(np.diff(a1) > 0)
    rate = len(a1) / a1[-1]
    assert abs(rate - 2000.0) / 2000.0 < 0.03                   # Poisson at 2000 req/s
    gaps = np.diff(a1) * 2000.0                                  # exponential(1): cv ~ 1
    assert abs(gaps.std() / gaps.mean() - 1.0) < 0.05
    assert s1.min() >= 1 and s1.max() <= 4096
    logs = np.log(s1 + 0.5)
    assert abs(np.median(logs) - np.log(4097) / 2) < 0.1         # log-uniform
    assert 450 < s1.mean() < 580                                 # mean (4096 - 1) / ln 4097 ~ 492


def test_serving_net_and_inputs_have_the_configured_shape():
    layers, head_w, head_b = sparse_mlp(3, L=4)
    assert len(layers) == 4 and head_w.shape == (1024, 10) and np.all(head_b == 0)
    for ro, cols, vals in layers:
        nnz = ro[-1]
        assert abs(nnz / 1024 ** 2 - 0.03) < 0.002               # 3 % density
        assert abs(vals.std() - 0.3) < 0.01 and abs(vals.mean()) < 0.01
        assert np.all(np.diff(ro) >= 0) and cols.min() >= 0 and cols.max() < 1024
    x = mlp_inputs(3, 5, 64)
    assert x.shape == (64, 1024) and x.dtype == np.float32
    assert 0.0 <= x.min() and x.max() < 1.0 and abs(x.mean() - 0.5) < 0.01
    assert np.array_equal(x, mlp_inputs(3, 5, 64)) and not np.array_equal(x, mlp_inputs(3, 6, 64))
