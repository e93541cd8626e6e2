"""Serving loop (sdnn_server_*): continuous batching of requests.

Checks, through the C ABI on the GPU:
  * a request's result is the same alone and in a mix of co-resident requests
    (bitwise in the plain modes: every row is computed independently of the
    other rows of its pass, in a fixed FP32 order);
  * the dense head's logits agree with the FP64 oracle within 1e-5 relative
    (|gpu - ref| / max(1, |ref|)) and argmax is exact wherever the oracle's
    top-two margin exceeds that tolerance -- on a short net; on the full
    120-layer net the FP32 recurrence itself drifts from FP64 (it amplifies
    rounding), so there the comparison is alone-vs-mix;
  * SNICIT mode (clustering across co-resident requests) keeps the category
    flags and agrees with the oracle within the FP32 bound;
  * admission errors: a request larger than a slot, a full queue.
"""
import numpy as np
import pytest

import snicit_gb300 as sg
from oracle import oracle as orc
from snicit_gb300._lib import SdnnError

pytestmark = pytest.mark.gpu
RTOL = 1e-5


def _engine(layers, N, mode="SNIG", threshold=4, centroids=16, bias=-0.05):
    eng = sg.Engine(N, len(layers), mode=mode, threshold=threshold, batch=4096, bias=bias,
                    num_centroids=centroids)
    for l, (ro, c, v) in enumerate(layers):
        eng.set_layer_csr(l, ro, c, v)
    return eng


def _rel(a, b):
    return np.abs(a.astype(np.float64) - b) / np.maximum(1.0, np.abs(b))


@pytest.mark.parametrize("mode", ["SNIG", "BF"])
def test_alone_equals_mix_full_depth(mode):
    """120-layer serving net: each request bitwise equal alone and in the mix."""
    N, seed = 1024, 5
    layers, hw, hb = sg.sparse_mlp(seed)
    sizes = [1, 7, 300, 1024, 64, 2500, 3]
    reqs = [sg.mlp_inputs(seed, i, n) for i, n in enumerate(sizes)]
    # a 100 ms batching window: requests submitted back to back share passes
    with _engine(layers, N, mode) as eng, \
            sg.Server(eng, hw, hb, slots=2, max_rows=4096, max_delay_us=100000) as sv:
        alone = [sv.wait(sv.submit(x)) for x in reqs]
        ids = [sv.submit(x) for x in reqs]
        mix = [sv.wait(i) for i in ids]
        st = sv.stats()
    assert st["max_rows_in_pass"] > max(sizes), "requests were never co-resident"
    for a, m in zip(alone, mix):
        assert np.array_equal(a.flags, m.flags)
        assert np.array_equal(a.logits, m.logits)
        assert np.array_equal(a.argmax, m.argmax)
        assert a.latency_s > 0 and m.latency_s > 0


def test_head_matches_fp64_oracle():
    N, L, seed = 1024, 8, 11
    layers, hw, hb = sg.sparse_mlp(seed, L=L)
    hb = np.linspace(-0.1, 0.1, 10).astype(np.float32)
    sizes = [5, 900, 130]
    reqs = [sg.mlp_inputs(seed, i, n) for i, n in enumerate(sizes)]
    with _engine(layers, N) as eng, sg.Server(eng, hw, hb, slots=3, max_rows=2048) as sv:
        out = [sv.wait(i) for i in [sv.submit(x) for x in reqs]]
    for x, r in zip(reqs, out):
        Y, alive, _ = orc.infer(layers, N, -0.05, x, precision=64)
        lref, aref = orc.head(Y, hw, hb)
        assert np.array_equal(r.flags, alive.astype(np.int32))
        assert _rel(r.logits, lref).max() <= RTOL
        top2 = np.sort(lref, axis=1)[:, -2:]
        clear = (top2[:, 1] - top2[:, 0]) > 2 * RTOL * np.maximum(1.0, np.abs(top2[:, 1]))
        assert np.array_equal(r.argmax[clear], aref[clear])


def test_snicit_mode_clusters_across_requests():
    N, L, seed = 1024, 10, 17
    layers, hw, hb = sg.sparse_mlp(seed, L=L)
    sizes = [40, 600, 9]
    reqs = [sg.mlp_inputs(seed, i, n) for i, n in enumerate(sizes)]
    with _engine(layers, N, mode="SNICIT", threshold=4, centroids=16) as eng, \
            sg.Server(eng, hw, hb, slots=1, max_rows=2048, max_delay_us=100000) as sv:
        out = [sv.wait(i) for i in [sv.submit(x) for x in reqs]]
        assert sv.stats()["max_rows_in_pass"] == sum(sizes)
    for x, r in zip(reqs, out):
        Y, alive, _ = orc.infer(layers, N, -0.05, x, precision=64)
        Y32, _, _ = orc.infer(layers, N, -0.05, x, precision=32)
        lref, _ = orc.head(Y, hw, hb)
        l32, _ = orc.head(Y32, hw, hb)
        assert np.array_equal(r.flags, alive.astype(np.int32))
        tol = np.maximum(RTOL, 4.0 * _rel(l32, lref).max(axis=1))
        assert np.all(_rel(r.logits, lref).max(axis=1) <= tol)


def test_admission_errors():
    N, seed = 1024, 3
    layers, hw, hb = sg.sparse_mlp(seed, L=2)
    with _engine(layers, N) as eng:
        with sg.Server(eng, hw, hb, slots=1, max_rows=256) as sv:
            assert sv.capacity == 256
            with pytest.raises(SdnnError) as ei:
                sv.submit(sg.mlp_inputs(seed, 0, 257))
            assert ei.value.code == 1
            r = sv.wait(sv.submit(sg.mlp_inputs(seed, 1, 256)))
            assert r.flags.shape == (256,)
        with sg.Server(eng, hw, hb, slots=1, max_rows=256, max_pending=0) as sv:
            with pytest.raises(SdnnError) as ei:
                sv.submit(sg.mlp_inputs(seed, 2, 4))
            assert ei.value.code == 9


def test_slots_share_the_model_weights_and_grow_at_admission():
    """One device copy of the weights serves every slot: the model's weights
    cannot change while a server reads them.  Slots start with buffers for
    4096 rows and grow when a larger request is admitted (free device memory
    read at admission); the results equal the model engine's own."""
    N, seed = 1024, 23
    layers, hw, hb = sg.sparse_mlp(seed, L=12)
    big = sg.mlp_inputs(seed, 0, 10000)
    small = sg.mlp_inputs(seed, 1, 37)
    with sg.Engine(N, len(layers), mode="SNIG", batch=len(big), bias=-0.05) as ref:
        for l, (ro, c, v) in enumerate(layers):
            ref.set_layer_csr(l, ro, c, v)
        f_big, _ = ref.infer(big)
        y_big = ref.activations(len(big))
    with _engine(layers, N) as eng:
        with sg.Server(eng, hw, hb, slots=3, max_rows=16384) as sv:
            st0 = sv.stats()
            assert st0["slot_rows"] == 4096
            with pytest.raises(SdnnError) as ei:
                eng.set_layer_csr(0, *layers[0])
            assert ei.value.code == 6  # SDNN_ERR_STATE: in use by the server
            r_small = sv.wait(sv.submit(small))
            r_big = sv.wait(sv.submit(big))
            st = sv.stats()
        assert st["slot_rows"] >= len(big)
        assert np.array_equal(r_big.flags, f_big)
        lref, aref = orc.head(y_big, hw, hb)
        assert _rel(r_big.logits, lref).max() <= 1e-5  # FP32 head of the same FP32 rows
        assert r_small.flags.shape == (37,)
        eng.set_layer_csr(0, *layers[0])  # the server is gone: allowed again


def test_full_depth_argmax_on_clear_rows():
    """The 120-layer serving net: FP32 cannot hold the logits to 1e-5 of FP64
    at this depth (the recurrence amplifies rounding), so the argmax is
    compared with the FP64 oracle on every row whose FP64 top-two margin
    exceeds 4x the FP32 port's own logit error on that row -- there the answer
    does not depend on rounding; the count of such rows is reported."""
    N, seed = 1024, 31
    layers, hw, hb = sg.sparse_mlp(seed)
    x = sg.mlp_inputs(seed, 0, 2000)
    with _engine(layers, N) as eng, sg.Server(eng, hw, hb, slots=2, max_rows=4096) as sv:
        r = sv.wait(sv.submit(x))
    Y, alive, _ = orc.infer(layers, N, -0.05, x, precision=64)
    Y32, _, _ = orc.infer(layers, N, -0.05, x, precision=32)
    lref, aref = orc.head(Y, hw, hb)
    l32, _ = orc.head(Y32, hw, hb)
    assert np.array_equal(r.flags, alive.astype(np.int32))
    err32 = np.abs(l32 - lref).max(axis=1)
    top2 = np.sort(lref, axis=1)[:, -2:]
    clear = (top2[:, 1] - top2[:, 0]) > 4.0 * err32
    print(f"120-layer net: {clear.sum()} of {len(x)} rows with a clear FP64 argmax; "
          f"FP32 port logit error up to {err32.max():.3g}")
    assert clear.sum() >= len(x) // 4
    assert np.array_equal(r.argmax[clear], aref[clear])
