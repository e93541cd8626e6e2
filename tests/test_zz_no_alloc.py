"""sdnn_layer_noalloc: the entry point for callers that cannot allocate.

Some callers may not call cudaMalloc once they are running: code inside a
CUDA-graph capture (an allocation there breaks the capture), serving threads
with a fixed memory budget or a real-time deadline, and hosts whose device
allocator belongs to another framework.  sdnn_layer_noalloc runs one plain
layer of an engine whose weights are already resident, on caller-owned device
buffers, with its scratch in a static device array (at most 65536 rows).

These tests compare it with the engine's regular entry point (sdnn_infer_host
on a one- or two-layer engine).  It runs the same layer kernel with the same
slots, so the activations must agree bit for bit and the survivor flags
exactly, on two calls in a row (the calls share the static scratch).  Every
call is issued on torch's current stream, so the sentinel fills before it are
ordered with it.  This file is collected last.
"""
import ctypes

import numpy as np
import pytest

import snicit_gb300 as sg
from snicit_gb300 import _lib

pytestmark = pytest.mark.gpu


def _stream():
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _noalloc(eng, layer, d_in, d_out, rows, d_alive):
    return sg.load().sdnn_layer_noalloc(eng._h, int(layer), ctypes.c_void_p(d_in.data_ptr()),
                                        ctypes.c_void_p(d_out.data_ptr()), int(rows),
                                        ctypes.c_void_p(d_alive.data_ptr()), _stream())


def _bits_equal(a, b):
    return np.array_equal(np.ascontiguousarray(a, np.float32).view(np.uint32),
                          np.ascontiguousarray(b, np.float32).view(np.uint32))


def _run_twice(eng, layer, d_in, rows, check):
    import torch
    d_out = torch.empty_like(d_in)
    d_alive = torch.empty(rows, dtype=torch.int32, device="cuda")
    for _ in range(2):  # two calls in a row share the static scratch
        d_out.fill_(-1.0)
        d_alive.fill_(7)
        rc = _noalloc(eng, layer, d_in, d_out, rows, d_alive)
        assert rc == 0, sg.load().sdnn_last_error(eng._h)
        torch.cuda.synchronize()
        check(d_out.cpu().numpy(), d_alive.cpu().numpy())


@pytest.mark.parametrize("N,B", [(1024, 700), (4096, 130), (65536, 300)])
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
    assert 0 < flags_ref.sum() < B
    with sg.Engine(N, 2, mode="SNIG", batch=B, bias=bias, placement=False) as eng:
        eng.generate_weights(seed)
        eng.finalize()  # weights on the device: the only allocation, before the calls
        d_in = torch.from_numpy(Y0).cuda()

        def check(y, alive):
            assert np.array_equal(alive, flags_ref)
            assert _bits_equal(y, y_ref)
        _run_twice(eng, 0, d_in, B, check)


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
            assert _bits_equal(c.cpu().numpy(), y_ref)


def test_noalloc_with_placement_matches_through_the_position_map(tmp_path):
    """With neuron placement the layer writes its outputs in the packer's
    storage order; the packed-weight file's position map turns them back into
    neuron order."""
    torch = pytest.importorskip("torch")
    import packed_layout as pl
    N, B, seed = 4096, 200, 77
    bias = sg.load().sdnn_reference_bias(N)
    Y0 = sg.generate_inputs(N, seed, 0, B)
    with sg.Engine(N, 1, mode="SNIG", batch=B, bias=bias) as ref:
        ref.generate_weights(seed)
        flags_ref, _ = ref.infer(Y0)
        y_ref = ref.activations(B)
    path = tmp_path / "w.sdnnw"
    with sg.Engine(N, 1, mode="SNIG", batch=B, bias=bias) as eng:
        eng.generate_weights(seed)
        eng.finalize()
        eng.save_packed(path)
        pos = pl.read_packed(path)["layers"][0]["pos"]
        assert pos is not None
        d_in = torch.from_numpy(Y0).cuda()

        def check(y, alive):
            assert np.array_equal(alive, flags_ref)
            assert _bits_equal(y[:, pos], y_ref)
        _run_twice(eng, 0, d_in, B, check)


def test_noalloc_general_weights_and_per_neuron_bias():
    """Per-edge weight values (the general-value kernel instances) and a
    per-neuron bias."""
    torch = pytest.importorskip("torch")
    N, B = 1024, 257
    rng = np.random.default_rng(5)
    rows = np.repeat(np.arange(N, dtype=np.int32), 24)
    cols = rng.integers(0, N, rows.size).astype(np.int32)
    vals = rng.normal(0.0, 0.3, rows.size).astype(np.float32)
    bias = rng.normal(-0.05, 0.02, N).astype(np.float32)
    Y0 = rng.uniform(0.0, 1.0, (B, N)).astype(np.float32)
    results = []
    for L in (1, 2):
        eng = sg.Engine(N, L, mode="SNIG", batch=B, bias=0.0, placement=False)
        for l in range(L):
            eng.set_layer_coo(l, rows, cols, vals)
            eng.set_layer_bias(l, bias)
        results.append(eng)
    ref, eng = results
    try:
        flags_ref, _ = ref.infer(Y0)
        y_ref = ref.activations(B)
        assert 0 < flags_ref.sum()
        eng.finalize()
        d_in = torch.from_numpy(Y0).cuda()

        def check(y, alive):
            assert np.array_equal(alive, flags_ref)
            assert _bits_equal(y, y_ref)
        _run_twice(eng, 0, d_in, B, check)
    finally:
        ref.close()
        eng.close()


def test_noalloc_rejects_sizes_beyond_its_scratch_and_overlap():
    torch = pytest.importorskip("torch")
    N = 1024
    with sg.Engine(N, 1, mode="SNIG", batch=16, bias=-0.3, placement=False) as eng:
        eng.generate_weights(1)
        eng.finalize()
        x = torch.zeros((16, N), device="cuda")
        alive = torch.zeros(16, dtype=torch.int32, device="cuda")
        L = sg.load()
        rc = L.sdnn_layer_noalloc(eng._h, 0, ctypes.c_void_p(x.data_ptr()),
                                  ctypes.c_void_p(x.data_ptr()), 65537,
                                  ctypes.c_void_p(alive.data_ptr()), _stream())
        assert rc == 1
        assert b"65536" in L.sdnn_last_error(eng._h)
        # in place, and overlapping by one row: rejected
        for off_rows in (0, 1):
            rc = L.sdnn_layer_noalloc(eng._h, 0, ctypes.c_void_p(x.data_ptr()),
                                      ctypes.c_void_p(x[off_rows].data_ptr()), 8,
                                      ctypes.c_void_p(alive.data_ptr()), _stream())
            assert rc == 1
            assert b"overlap" in L.sdnn_last_error(eng._h)
        # adjacent, not overlapping: accepted
        rc = L.sdnn_layer_noalloc(eng._h, 0, ctypes.c_void_p(x.data_ptr()),
                                  ctypes.c_void_p(x[8].data_ptr()), 8,
                                  ctypes.c_void_p(alive.data_ptr()), _stream())
        assert rc == 0, L.sdnn_last_error(eng._h)
        torch.cuda.synchronize()


def test_noalloc_reports_a_device_wait_that_gave_up():
    """A device wait of the call that runs out (here a wait nothing completes,
    through the same bounded-wait helper the layer kernel uses) shows as -1 in
    every d_alive entry; the next call works normally."""
    torch = pytest.importorskip("torch")
    N, B, seed = 1024, 100, 9
    Y0 = sg.generate_inputs(N, seed, 0, B)
    with sg.Engine(N, 1, mode="SNIG", batch=B, bias=-0.3, placement=False) as ref:
        ref.generate_weights(seed)
        flags_ref, _ = ref.infer(Y0)
    with sg.Engine(N, 1, mode="SNIG", batch=B, bias=-0.3, placement=False) as eng:
        eng.generate_weights(seed)
        eng.finalize()
        alive = torch.zeros(B, dtype=torch.int32, device="cuda")
        rc = sg.load().sdnn_selftest_noalloc_timeout(eng._h, ctypes.c_void_p(alive.data_ptr()), B,
                                                     100000, _stream())
        assert rc == 0, sg.load().sdnn_last_error(eng._h)
        torch.cuda.synchronize()
        assert (alive.cpu().numpy() == -1).all()
        d_in = torch.from_numpy(Y0).cuda()
        _run_twice(eng, 0, d_in, B, lambda y, a: np.testing.assert_array_equal(a, flags_ref))
        assert torch.cuda.current_device() == 0
