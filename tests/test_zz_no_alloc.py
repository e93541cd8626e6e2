"""sdnn_layer_noalloc: the entry point for callers that cannot allocate.

Some callers may not call cudaMalloc once they are running (code inside a
CUDA-graph capture, fixed-budget or real-time serving threads, hosts whose
allocator belongs to another framework).  sdnn_layer_noalloc runs one plain
layer of an engine whose weights are already resident on caller-owned device
buffers, with its scratch in a static device array (at most 65536 rows).
These tests check it against the engine's regular entry point (sdnn_infer_host
on a one- and a two-layer engine), within the tolerance the parity tests use
(1e-5 relative, the category flags exactly), on two calls in a row.
"""
import ctypes

import numpy as np
import pytest

import snicit_gb300 as sg
from snicit_gb300 import _lib

pytestmark = pytest.mark.gpu
RTOL = 1e-5


def _noalloc(eng, layer, d_in, d_out, rows, d_alive):
    return sg.load().sdnn_layer_noalloc(eng._h, int(layer), ctypes.c_void_p(d_in.data_ptr()),
                                        ctypes.c_void_p(d_out.data_ptr()), int(rows),
                                        ctypes.c_void_p(d_alive.data_ptr()), None)


def _close(a, b):
    err = np.abs(a.astype(np.float64) - b) / np.maximum(1.0, np.abs(b.astype(np.float64)))
    return err.max() <= RTOL


@pytest.mark.parametrize("N,B", [(1024, 700), (4096, 130)])
def test_noalloc_layer_matches_regular_entry(N, B):
    torch = pytest.importorskip("torch")
    seed = 31 + N
    bias = sg.load().sdnn_reference_bias(N)
    Y0 = sg.generate_inputs(N, seed, 0, B)
    # regular entry point: a one-layer engine
    with sg.Engine(N, 1, mode="SNIG", batch=B, bias=bias, placement=False) as ref:
        ref.generate_weights(seed)
        flags_ref, _ = ref.infer(Y0)
        y_ref = ref.activations(B)
    with sg.Engine(N, 2, mode="SNIG", batch=B, bias=bias, placement=False) as eng:
        eng.generate_weights(seed)
        eng.finalize()  # weights on the device: the only allocation, before the calls
        d_in = torch.from_numpy(Y0).cuda()
        d_out = torch.empty_like(d_in)
        d_alive = torch.empty(B, dtype=torch.int32, device="cuda")
        for _ in range(2):  # two calls in a row share the static scratch
            d_out.fill_(-1.0)
            d_alive.fill_(7)
            assert _noalloc(eng, 0, d_in, d_out, B, d_alive) == 0, _lib.load().sdnn_last_error(eng._h)
            torch.cuda.synchronize()
            assert np.array_equal(d_alive.cpu().numpy(), flags_ref)
            assert _close(d_out.cpu().numpy(), y_ref)


def test_noalloc_chain_matches_two_layer_engine():
    torch = pytest.importorskip("torch")
    N, B, seed = 1024, 300, 57
    Y0 = sg.generate_inputs(N, seed, 0, B)
    with sg.Engine(N, 2, mode="SNIG", batch=B, bias=-0.3, placement=False) as ref:
        ref.generate_weights(seed)
        flags_ref, _ = ref.infer(Y0)
        y_ref = ref.activations(B)
    with sg.Engine(N, 2, mode="SNIG", batch=B, bias=-0.3, placement=False) as eng:
        eng.generate_weights(seed)
        eng.finalize()
        a = torch.from_numpy(Y0).cuda()
        b = torch.empty_like(a)
        alive = torch.empty(B, dtype=torch.int32, device="cuda")
        for _ in range(2):
            assert _noalloc(eng, 0, a, b, B, alive) == 0
            c = torch.empty_like(a)
            assert _noalloc(eng, 1, b, c, B, alive) == 0
            torch.cuda.synchronize()
            # the regular path keeps dead rows at zero; so does the layer (all outputs <= 0 clamp to 0)
            assert np.array_equal(alive.cpu().numpy(), flags_ref)
            assert _close(c.cpu().numpy(), y_ref)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    N = 1024
    with sg.Engine(N, 1, mode="SNIG", batch=16, bias=-0.3, placement=False) as eng:
        eng.generate_weights(1)
        eng.finalize()
        x = torch.zeros((16, N), device="cuda")
        alive = torch.zeros(16, dtype=torch.int32, device="cuda")
        rc = sg.load().sdnn_layer_noalloc(eng._h, 0, ctypes.c_void_p(x.data_ptr()),
                                          ctypes.c_void_p(x.data_ptr()), 65537,
                                          ctypes.c_void_p(alive.data_ptr()), None)
        assert rc == 1
        assert b"65536" in sg.load().sdnn_last_error(eng._h)
