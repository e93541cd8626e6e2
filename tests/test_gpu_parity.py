"""GPU parity of the CUDA path against the FP64 oracle (through the C ABI).

Tolerances: the category set is bit-exact.  Final activations agree with the
FP64 oracle within 1e-5 relative, measured per row as
|gpu - ref| / max(1, |ref|) (activations live in [0, 32]) -- except on rows
where FP32 itself cannot: rows still in the non-saturated transient after a
short net, where the recurrence doubles rounding errors every layer.  There
the bound is 4x the error of a plain sequential FP32 evaluation of the same
row (the oracle's FP32 port), i.e. per row
    tol_r = max(1e-5, 4 * err_fp32port_r).
On long nets (the benchmark configurations) rows saturate and the bound is
1e-5 everywhere.  The plain path is also checked bit for bit against a CPU
evaluation in the kernels' own summation order (tests/packed_layout.py).
"""
import os
import tempfile

import numpy as np
import pytest

import snicit_gb300 as sg
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
RTOL = 1e-5


def _layers(N, L, seed, nnz=32, value=0.0625):
    return [sg.generate_layer_csr(N, seed, l, nnz, value) for l in range(L)]


def _rel(Y, Yref):
    return np.abs(Y.astype(np.float64) - Yref) / np.maximum(1.0, np.abs(Yref))


def _check(Y, flags, ids, Yref, alive, label, rtol=RTOL, Y32=None):
    """Y32: the oracle's sequential FP32 evaluation, for the per-row bound."""
    want = np.flatnonzero(alive)
    assert np.array_equal(ids, want), f"{label}: category set differs ({len(ids)} vs {len(want)})"
    assert np.array_equal(flags, alive.astype(np.int32)), f"{label}: flags differ"
    err = _rel(Y, Yref).max(axis=1)
    tol = np.full(err.shape, rtol)
    if Y32 is not None:
        tol = np.maximum(tol, 4.0 * _rel(Y32, Yref).max(axis=1))
    bad = np.flatnonzero(err > tol)
    assert len(bad) == 0, f"{label}: activation error {err[bad].max():.3g} > {tol[bad].min():.3g} on {len(bad)} rows"
    loose = int((tol > rtol).sum())
    print(f"{label}: max error {err.max():.3g}, largest per-row bound {tol.max():.3g} "
          f"({loose} of {len(tol)} rows above {rtol:g})")
    return float(tol.max())


def _ref(layers, N, bias, Y0, **kw):
    """FP64 oracle plus the FP32 port (for the per-row tolerance)."""
    Yref, alive, dead = orc.infer(layers, N, bias, Y0, precision=64, **kw)
    Y32, _, _ = orc.infer(layers, N, bias, Y0, precision=32, **kw)
    return Yref, alive, Y32


def _run(N, L, B, seed, mode, threshold=30, bias=None, centroids=32, tile_rows=0, threads=0,
         batch=None, Y0=None, weights=None):
    bias = sg.load().sdnn_reference_bias(N) if bias is None else bias
    if bias == 0.0:
        bias = -0.3
    Y0 = sg.generate_inputs(N, seed, 0, B) if Y0 is None else Y0
    with sg.Engine(N, L, mode=mode, threshold=threshold, batch=batch or B, bias=bias,
                   num_centroids=centroids, tile_rows=tile_rows, threads=threads) as eng:
        if weights is None:
            eng.generate_weights(seed)
        else:
            for l, (ro, c, v) in enumerate(weights):
                eng.set_layer_csr(l, ro, c, v)
        flags, ids = eng.infer(Y0)
        Y = eng.activations(B) if (batch is None or batch >= B) else None
        st = eng.stats()
    return Y0, flags, ids, Y, st, bias


@pytest.mark.parametrize("mode", ["BF", "SNIG", "XY"])
@pytest.mark.parametrize("N,L,B", [(256, 20, 300), (1024, 24, 200), (4096, 12, 64)])
def test_plain_modes(mode, N, L, B):
    seed = 100 + N + L
    Y0, flags, ids, Y, st, bias = _run(N, L, B, seed, mode, threshold=L // 2)
    Yref, alive, Y32 = _ref(_layers(N, L, seed), N, bias, Y0)
    _check(Y, flags, ids, Yref, alive, f"{mode} N={N}", Y32=Y32)
    assert st["rows_out"] == len(ids)


@pytest.mark.parametrize("N,L,B,T,K", [(1024, 40, 400, 8, 32), (1024, 40, 400, 1, 4),
                                       (4096, 24, 96, 6, 16), (256, 30, 500, 12, 50)])
def test_snicit_matches_oracle(N, L, B, T, K):
    seed = 7 + N + T
    Y0, flags, ids, Y, st, bias = _run(N, L, B, seed, "SNICIT", threshold=T, centroids=K)
    layers = _layers(N, L, seed)
    Yref, alive, Y32 = _ref(layers, N, bias, Y0)
    _check(Y, flags, ids, Yref, alive, f"SNICIT N={N} t={T}", Y32=Y32)
    assert st["threshold"] == T and st["centroids"] >= 1


def test_snicit_residue_form_oracle_agrees():
    """The FP64 residue-form restatement gives the plain categories (exactness)."""
    N, L, B, T, seed = 256, 24, 300, 4, 5
    Y0 = sg.generate_inputs(N, seed, 0, B)
    layers = _layers(N, L, seed)
    Yref, alive, dead = orc.infer(layers, N, -0.3, Y0, precision=64)
    Yt, alive_t, _ = orc.infer(layers[:T], N, -0.3, Y0, precision=64)
    live = np.flatnonzero(alive_t)
    cands = live[orc.ref_candidates(Yt[live].astype(np.float32))]
    Ys, flags, _, nonempty = orc.snicit(layers, N, -0.3, Y0, T, cands)
    assert np.array_equal(flags, alive)
    assert np.abs(Ys - Yref).max() <= 1e-9


@pytest.mark.parametrize("mode", ["SNIG", "SNICIT"])
def test_edge_cases(mode):
    N, L, seed = 1024, 12, 21
    # one row; zero rows; rows not a multiple of the tile; all-dead batch
    for B in (1, 33, 65):
        Y0 = sg.generate_inputs(N, seed, 0, B)
        Y0[0] = 0.0
        _, flags, ids, Y, _, bias = _run(N, L, B, seed, mode, threshold=3, Y0=Y0)
        Yref, alive, Y32 = _ref(_layers(N, L, seed), N, bias, Y0)
        _check(Y, flags, ids, Yref, alive, f"{mode} B={B}", Y32=Y32)
        assert flags[0] == 0
    Y0 = np.zeros((17, N), np.float32)
    _, flags, ids, Y, _, _ = _run(N, L, 17, seed, mode, threshold=3, Y0=Y0)
    assert len(ids) == 0 and not flags.any() and not Y.any()


@pytest.mark.parametrize("T", [0, 1, 11, 12, 50])
def test_snicit_threshold_extremes(T):
    N, L, B, seed = 1024, 12, 150, 33
    Y0, flags, ids, Y, st, bias = _run(N, L, B, seed, "SNICIT", threshold=T)
    Yref, alive, Y32 = _ref(_layers(N, L, seed), N, bias, Y0)
    # t = 0 clusters the raw binary inputs, so the FP32 residue update
    # f(a + d) - f(a) runs through the whole non-saturated transient, where
    # the recurrence doubles rounding errors per layer; the reference's
    # post_minus has the same arithmetic.  Categories stay exact; the
    # activation bound for that case is 1e-4 (1e-5 for every later threshold).
    _check(Y, flags, ids, Yref, alive, f"t={T}", rtol=1e-4 if T == 0 else RTOL, Y32=Y32)
    assert st["threshold"] == min(T, L)


def test_single_layer_and_single_centroid():
    N, B, seed = 1024, 80, 3
    for L, T, K in ((1, 0, 1), (2, 1, 1), (5, 2, 1)):
        Y0, flags, ids, Y, _, bias = _run(N, L, B, seed, "SNICIT", threshold=T, centroids=K)
        Yref, alive, Y32 = _ref(_layers(N, L, seed), N, bias, Y0)
        _check(Y, flags, ids, Yref, alive, f"L={L}", Y32=Y32)


def test_general_weights_per_neuron_bias():
    """beyond-shaped layers: random-valued sparse W, per-neuron bias, clamp 32."""
    N, L, B = 1024, 10, 128
    rng = np.random.default_rng(9)
    layers, biases = [], []
    for _ in range(L):
        mask = rng.random((N, N)) < 0.03
        r, c = np.nonzero(mask)
        v = (rng.standard_normal(len(r)) * 0.3).astype(np.float32)
        layers.append(sg.coo_to_csr(N, r, c, v))
        biases.append(rng.uniform(-0.1, 0.0, N).astype(np.float32))
    Y0 = rng.random((B, N)).astype(np.float32)
    for mode in ("SNIG", "SNICIT"):
        with sg.Engine(N, L, mode=mode, threshold=4, batch=B, bias=-0.05, num_centroids=16) as eng:
            for l, (ro, c, v) in enumerate(layers):
                eng.set_layer_csr(l, ro, c, v)
                eng.set_layer_bias(l, biases[l])
            flags, ids = eng.infer(Y0)
            Y = eng.activations(B)
        Yref, alive, Y32 = _ref(layers, N, -0.05, Y0, bias_vec=np.stack(biases))
        _check(Y, flags, ids, Yref, alive, mode, Y32=Y32)


def test_multi_batch_and_determinism():
    N, L, B, seed = 1024, 16, 500, 44
    Y0 = sg.generate_inputs(N, seed, 0, B)
    _, f1, ids1, _, _, bias = _run(N, L, B, seed, "SNICIT", threshold=4, batch=128, Y0=Y0)
    _, f2, ids2, Y2, _, _ = _run(N, L, B, seed, "SNICIT", threshold=4, Y0=Y0)
    _, f3, ids3, Y3, _, _ = _run(N, L, B, seed, "SNICIT", threshold=4, Y0=Y0)
    Yref, alive, _ = orc.infer(_layers(N, L, seed), N, bias, Y0, precision=64)
    assert np.array_equal(ids1, np.flatnonzero(alive))
    assert np.array_equal(ids1, ids2) and np.array_equal(f1, f2)
    assert np.array_equal(Y2.view(np.uint32), Y3.view(np.uint32)), "runs are not bitwise identical"


@pytest.mark.parametrize("tile_rows,threads", [(8, 256), (12, 512), (16, 512), (24, 256)])
def test_tile_shapes(tile_rows, threads):
    N, L, B, seed = 1024, 10, 257, 8
    Y0, flags, ids, Y, st, bias = _run(N, L, B, seed, "SNICIT", threshold=3, tile_rows=tile_rows,
                                       threads=threads)
    Yref, alive, Y32 = _ref(_layers(N, L, seed), N, bias, Y0)
    _check(Y, flags, ids, Yref, alive, f"T={tile_rows}", Y32=Y32)
    assert st["tile_rows"] == tile_rows and st["threads"] == threads


@pytest.mark.parametrize("N,L,B", [(16384, 4, 24), (512, 10, 100), (2048, 6, 50)])
def test_other_widths(N, L, B):
    seed = 61
    Y0, flags, ids, Y, st, bias = _run(N, L, B, seed, "SNICIT", threshold=2, bias=-0.4)
    Yref, alive, Y32 = _ref(_layers(N, L, seed), N, bias, Y0)
    _check(Y, flags, ids, Yref, alive, f"N={N}", Y32=Y32)


def test_chunked_width_65536():
    N, L, B, seed = 65536, 2, 6, 62
    Y0, flags, ids, Y, st, bias = _run(N, L, B, seed, "SNIG", bias=-0.45)
    Yref, alive, Y32 = _ref(_layers(N, L, seed), N, bias, Y0)
    _check(Y, flags, ids, Yref, alive, "N=65536", Y32=Y32)


def test_tsv_round_trip():
    N, L, B, seed = 1024, 6, 64, 71
    Y0 = sg.generate_inputs(N, seed, 0, B)
    with tempfile.TemporaryDirectory() as d:
        with sg.Engine(N, L, mode="SNIG", batch=B) as a:
            a.generate_weights(seed)
            a.write_weights_tsv(d)
            fa, ia = a.infer(Y0)
        sg.write_inputs_tsv(os.path.join(d, "in.tsv"), Y0)
        Y1 = sg.read_inputs_tsv(os.path.join(d, "in.tsv"), N, 0, B)
        assert np.array_equal(Y0, Y1)
        with sg.Engine(N, L, mode="SNIG", batch=B) as b:
            b.load_weights_tsv(d)
            fb, ib = b.infer(Y1)
        assert np.array_equal(ia, ib) and np.array_equal(fa, fb)
        # the reference class mirror reads the same files
        sg.write_categories_tsv(os.path.join(d, "golden.tsv"), ia)
        ids = sg.SNICIT(d, -0.3, N, L, 2).infer(os.path.join(d, "in.tsv"),
                                                  os.path.join(d, "golden.tsv"), B, B, verbose=False)
        assert np.array_equal(ids, ia)


def test_device_pointer_path():
    torch = pytest.importorskip("torch")
    N, L, B, seed = 1024, 12, 200, 17
    Y0 = sg.generate_inputs(N, seed, 0, B)
    d_in = torch.from_numpy(Y0).cuda()
    d_flags = torch.zeros(B, dtype=torch.int32, device="cuda")
    with sg.Engine(N, L, mode="SNICIT", threshold=3, batch=B) as eng:
        eng.generate_weights(seed)
        s = torch.cuda.current_stream()
        eng.infer_device(d_in.data_ptr(), B, d_flags.data_ptr(), s.cuda_stream)
        torch.cuda.synchronize()
        flags = d_flags.cpu().numpy()
    _, alive, _ = orc.infer(_layers(N, L, seed), N, -0.3, Y0, precision=64, want_y=False)
    assert np.array_equal(flags, alive)


def test_autotune_keeps_categories():
    N, L, B, seed = 1024, 40, 256, 90
    Y0 = sg.generate_inputs(N, seed, 0, B)
    with tempfile.TemporaryDirectory() as d:
        rec = os.path.join(d, "tune.jsonl")
        with sg.Engine(N, L, mode="SNICIT", threshold=30, batch=B) as eng:
            eng.generate_weights(seed)
            eng.autotune(Y0, rec)
            flags, ids = eng.infer(Y0)
        lines = open(rec).read().strip().splitlines()
        assert len(lines) >= 4
        import json
        surv = {json.loads(x)["survivors"] for x in lines if json.loads(x)["status"] == 0}
    _, alive, _ = orc.infer(_layers(N, L, seed), N, -0.3, Y0, precision=64, want_y=False)
    assert surv == {int(alive.sum())}
    assert np.array_equal(ids, np.flatnonzero(alive))


@pytest.mark.parametrize("N,L,B", [(1024, 8, 700), (4096, 5, 300), (16384, 3, 70),
                                   (65536, 2, 100)])
def test_binary_first_layer_is_bitwise_equal(N, L, B):
    """The counting first-layer kernel gives the float kernel's bits exactly;
    tiles with a non-binary value fall back to the float kernel."""
    seed = 5 + N
    Y0 = sg.generate_inputs(N, seed, 0, B)
    Y0[40, 3] = 0.5  # one non-binary value: its 32-row tile takes the fallback
    out = {}
    for fast in (True, False):
        with sg.Engine(N, L, mode="SNIG", batch=B, bias=sg.load().sdnn_reference_bias(N),
                       binary_first_layer=fast) as eng:
            eng.generate_weights(seed)
            flags, ids = eng.infer(Y0)
            out[fast] = (flags, ids, eng.activations(B), eng.stats())
    assert out[True][3]["launches"] > out[False][3]["launches"], "counting kernel not used"
    assert np.array_equal(out[True][1], out[False][1])
    assert np.array_equal(out[True][2].view(np.uint32), out[False][2].view(np.uint32))
    Yref, alive, Y32 = _ref(_layers(N, L, seed), N, sg.load().sdnn_reference_bias(N), Y0)
    _check(out[True][2], out[True][0], out[True][1], Yref, alive, f"bits N={N}", Y32=Y32)


@pytest.mark.parametrize("mode", ["SNIG", "SNICIT"])
def test_placement_gives_same_results(mode):
    """Neuron placement only reorders the layout: categories identical, activations
    within tolerance of each other and of the oracle (summation order differs)."""
    N, L, B, seed = 1024, 14, 300, 77
    Y0 = sg.generate_inputs(N, seed, 0, B)
    res = {}
    for place in (True, False):
        with sg.Engine(N, L, mode=mode, threshold=5, batch=B, bias=-0.3, placement=place) as eng:
            eng.generate_weights(seed)
            flags, ids = eng.infer(Y0)
            res[place] = (flags, ids, eng.activations(B))
    assert np.array_equal(res[True][1], res[False][1])
    Yref, alive, Y32 = _ref(_layers(N, L, seed), N, -0.3, Y0)
    for place in (True, False):
        _check(res[place][2], res[place][0], res[place][1], Yref, alive, f"place={place}", Y32=Y32)


@pytest.mark.parametrize("N,L,B,T,K", [(1024, 60, 600, 30, 50), (4096, 40, 200, 25, 8),
                                       (1024, 30, 300, 2, 4), (4096, 60, 2000, 30, 50),
                                       (16384, 36, 300, 30, 16), (65536, 33, 160, 30, 8)])
def test_chain_path_is_bitwise_equal_to_per_layer_path(N, L, B, T, K):
    """When clustering leaves no residue row, one chain launch carries the
    centroid rows through the remaining layers (cluster kernel with streamed
    weights, cluster kernel reading L2, or the grid-wide kernel); each must give
    the per-layer launches' bits.  (With early thresholds residues remain and
    every run takes the per-layer path.)"""
    seed = 400 + N + T
    bias = sg.load().sdnn_reference_bias(N)
    Y0 = sg.generate_inputs(N, seed, 0, B)
    runs = {"layers": dict(chain=False), "default": dict(),
            "cluster_l2": dict(chain_stream=False, grid_chain=False),
            "grid": dict(chain_stream=False, chain=True),
            "host_choice": dict(device_post_choice=False)}
    out = {}
    for name, kw in runs.items():
        with sg.Engine(N, L, mode="SNICIT", threshold=T, batch=B, bias=bias, num_centroids=K,
                       **kw) as eng:
            eng.generate_weights(seed)
            flags, ids = eng.infer(Y0)
            out[name] = (flags, ids, eng.activations(B), eng.stats(), eng.layer_rows())
    kinds = {k: v[3]["post_kernel"] for k, v in out.items()}
    assert kinds["layers"] == 1
    # the device picks the post-threshold path inside one graph, as the host would
    assert out["default"][3]["device_post_choice"] == 1
    assert out["host_choice"][3]["device_post_choice"] == 0
    assert kinds["host_choice"] == kinds["default"], kinds
    # (the device path adds the one-thread choice kernel)
    assert out["default"][3]["launches"] == out["host_choice"][3]["launches"] + 1
    if out["layers"][3]["residue_rows"] == 0 and out["layers"][3]["centroids"] > 0:
        assert kinds["grid"] in (2, 3, 4), kinds  # a chain kernel of some kind
        assert kinds["cluster_l2"] in (1, 2), kinds
    for k in ("default", "cluster_l2", "grid", "host_choice"):
        assert np.array_equal(out[k][1], out["layers"][1])
        assert np.array_equal(out[k][2].view(np.uint32), out["layers"][2].view(np.uint32)), (k, kinds)
        assert np.array_equal(out[k][4], out["layers"][4])
    Yref, alive, Y32 = _ref(_layers(N, L, seed), N, bias, Y0)
    _check(out["default"][2], out["default"][0], out["default"][1], Yref, alive,
           f"chain N={N}", Y32=Y32)


@pytest.mark.parametrize("mode", ["SNIG", "SNICIT"])
def test_uneven_batches_in_one_schedule(mode):
    """Uneven batches run as one schedule give each batch its own category set
    (the same as running it alone), and graphs are reused across row counts."""
    N, L, seed = 1024, 40, 91
    sizes = [500, 37, 1200, 1, 260]
    batches = [sg.generate_inputs(N, seed, 10000 * i, n) for i, n in enumerate(sizes)]
    layers = _layers(N, L, seed)
    with sg.Engine(N, L, mode=mode, threshold=12, batch=sum(sizes), bias=-0.3) as eng:
        eng.generate_weights(seed)
        flags = eng.infer_batches(batches)
        flags2 = eng.infer_batches(batches[::-1])[::-1]
        alone = [eng.infer(b)[0] for b in batches]
    for f, f2, a, b in zip(flags, flags2, alone, batches):
        _, alive, _ = orc.infer(layers, N, -0.3, b, precision=64, want_y=False)
        assert np.array_equal(f, alive) and np.array_equal(f2, alive) and np.array_equal(a, alive)


@pytest.mark.parametrize("N,L,B,T", [(1024, 60, 3000, 30), (4096, 40, 1500, 30)])
def test_row_merging_is_exact(N, L, B, T):
    """Merging bitwise-identical rows below the threshold keeps the category
    set, keeps activations within the oracle bound, is deterministic, and
    computes fewer row-layers than the same SNICIT run without merging."""
    seed = 23
    Y0 = sg.generate_inputs(N, seed, 0, B)
    out = {}
    for merge in (True, False):
        runs = []
        for _ in range(2):
            with sg.Engine(N, L, mode="SNICIT", threshold=T, batch=B, num_centroids=32,
                           merge=merge, merge_start=2) as eng:
                eng.generate_weights(seed)
                flags, ids = eng.infer(Y0)
                runs.append((flags, ids, eng.activations(B), eng.stats()))
        assert np.array_equal(runs[0][2], runs[1][2]), f"merge={merge}: not deterministic"
        out[merge] = runs[0]
    bias = sg.load().sdnn_reference_bias(N)
    Yref, alive, Y32 = _ref(_layers(N, L, seed), N, bias, Y0)
    for merge, (flags, ids, Y, st) in out.items():
        _check(Y, flags, ids, Yref, alive, f"merge={merge}", Y32=Y32)
    assert out[True][3]["pre_row_layers"] < out[False][3]["pre_row_layers"]


def test_duplicate_input_rows_are_merged_and_recovered():
    """Inputs with repeated rows: the copies end bitwise equal to each other and
    to the oracle bound, with merging on (they merge at the first merge step)."""
    N, L, B, T, seed = 1024, 24, 400, 12, 29
    base = sg.generate_inputs(N, seed, 0, 50)
    idx = np.random.default_rng(3).integers(0, 50, B)
    Y0 = base[idx]
    with sg.Engine(N, L, mode="SNICIT", threshold=T, batch=B, num_centroids=16,
                   merge_start=1) as eng:
        eng.generate_weights(seed)
        flags, ids = eng.infer(Y0)
        Y = eng.activations(B)
        rows = eng.layer_rows()
    for k in range(50):
        grp = np.flatnonzero(idx == k)
        if len(grp) > 1:
            assert np.array_equal(Y[grp], np.repeat(Y[grp[:1]], len(grp), axis=0))
            assert len(set(flags[grp])) == 1
    assert rows[1] <= 50, f"rows after the first merge: {rows[1]}"
    bias = sg.load().sdnn_reference_bias(N)
    Yref, alive, Y32 = _ref(_layers(N, L, seed), N, bias, Y0)
    _check(Y, flags, ids, Yref, alive, "duplicates", Y32=Y32)


@pytest.mark.parametrize("N,off,rows", [(1024, 0, 300), (4096, 12345, 77), (256, 5, 1)])
def test_device_input_generator_matches_host(N, off, rows):
    torch = pytest.importorskip("torch")
    d = torch.empty((rows, N), dtype=torch.float32, device="cuda")
    sg.generate_inputs_device(N, 99, off, rows, d.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(d.cpu().numpy(), sg.generate_inputs(N, 99, off, rows))


def test_set_mode_and_device_autotune():
    """One resident copy of W serves SNICIT and the plain path; the device-side
    autotuner keeps the category set."""
    torch = pytest.importorskip("torch")
    N, L, B, seed = 1024, 64, 2000, 41
    d = torch.empty((B, N), dtype=torch.float32, device="cuda")
    sg.generate_inputs_device(N, seed, 0, B, d.data_ptr())
    f = torch.zeros(B, dtype=torch.int32, device="cuda")
    _, alive, _ = orc.infer(_layers(N, L, seed), N, -0.3, sg.generate_inputs(N, seed, 0, B),
                            precision=64, want_y=False)
    with sg.Engine(N, L, mode="SNICIT", threshold=30, batch=B, bias=-0.3) as eng:
        eng.generate_weights(seed)
        eng.autotune_device(d.data_ptr(), B)
        # the sweep's thresholds, no clustering (L), or the earlier ones tried with merging
        assert eng.stats()["threshold"] in (12, 16, 20, 24, 30, 60, L)
        f.zero_()
        eng.infer_device(d.data_ptr(), B, f.data_ptr())
        torch.cuda.synchronize()
        assert np.array_equal(f.cpu().numpy(), alive), "autotuned"
        for mode, t in (("SNICIT", 30), ("SNIG", L), ("BF", L), ("SNICIT", 60)):
            eng.set_mode(mode, t)
            f.zero_()
            eng.infer_device(d.data_ptr(), B, f.data_ptr())
            torch.cuda.synchronize()
            assert np.array_equal(f.cpu().numpy(), alive), mode


@pytest.mark.parametrize("N,L,B", [(1024, 40, 500), (65536, 3, 64)])
def test_packed_weight_file_gives_the_same_inference(tmp_path, N, L, B):
    seed = 61
    Y0 = sg.generate_inputs(N, seed, 0, B)
    path = tmp_path / "w.sdnnw"
    with sg.Engine(N, L, mode="SNICIT", threshold=min(20, L - 1), batch=B) as eng:
        eng.generate_weights(seed)
        eng.save_packed(path)
        f1, ids1 = eng.infer(Y0)
        y1 = eng.activations(B)
    with sg.Engine(N, L, mode="SNICIT", threshold=min(20, L - 1), batch=B) as eng:
        eng.load_packed(path)
        f2, ids2 = eng.infer(Y0)
        y2 = eng.activations(B)
    assert np.array_equal(ids1, ids2)
    assert np.array_equal(y1.view(np.uint32), y2.view(np.uint32))


@pytest.mark.parametrize("mode", ["SNIG", "SNICIT"])
def test_one_bit_host_inputs_match_float_inputs(mode):
    N, L, B, seed = 1024, 30, 900, 71
    Y0 = sg.generate_inputs(N, seed, 0, B)
    with sg.Engine(N, L, mode=mode, threshold=12, batch=400, bias=-0.3) as eng:
        eng.generate_weights(seed)
        f1, ids1 = eng.infer(Y0)
        f2, ids2 = eng.infer_bits(sg.pack_bits(Y0))
    assert np.array_equal(f1, f2) and np.array_equal(ids1, ids2)


def test_bounded_wait_times_out_and_engine_stays_usable():
    """Failure detection without a fault: a device wait that nothing completes
    runs out (0.2 s), the engine reports the timeout, then infers normally."""
    N, L, B, seed = 1024, 8, 64, 5
    Y0 = sg.generate_inputs(N, seed, 0, B)
    with sg.Engine(N, L, mode="SNIG", batch=B, bias=-0.3) as eng:
        eng.generate_weights(seed)
        rc = sg.load().sdnn_selftest_wait_timeout(eng._h, 200000)
        assert rc == 7, rc  # SDNN_ERR_TIMEOUT
        assert b"timed out" in sg.load().sdnn_last_error(eng._h)
        flags, ids = eng.infer(Y0)
    _, alive, _ = orc.infer(_layers(N, L, seed), N, -0.3, Y0, precision=64, want_y=False)
    assert np.array_equal(flags, alive)


@pytest.mark.parametrize("N,L,T", [(1024, 40, 20), (4096, 40, 20), (65536, 33, 30)])
def test_chain_with_several_centroids(N, L, T):
    """Rows that are copies of a few prototypes: merging leaves one row per
    prototype, the clustering keeps them as centroids without residues, and a
    chain launch carries several rows at once (cluster or grid kernel); the
    result must match the per-layer launches bitwise and the oracle."""
    seed = 13
    protos = sg.generate_inputs(N, seed, 0, 40)
    bias = sg.load().sdnn_reference_bias(N)
    Y0 = protos[np.arange(48) % 40]
    out = {}
    for chain in (True, False):
        with sg.Engine(N, L, mode="SNICIT", threshold=T, batch=48, bias=bias, num_centroids=50,
                       chain=chain, merge_start=1) as eng:
            eng.generate_weights(seed)
            flags, ids = eng.infer(Y0)
            out[chain] = (flags, ids, eng.activations(48), eng.stats())
    st = out[True][3]
    if st["residue_rows"] == 0 and st["centroids"] > 1:
        assert st["post_kernel"] in (2, 3, 4), st
    assert np.array_equal(out[True][1], out[False][1])
    assert np.array_equal(out[True][2].view(np.uint32), out[False][2].view(np.uint32))
    Yref, alive, Y32 = _ref(_layers(N, L, seed), N, bias, Y0)
    _check(out[True][2], out[True][0], out[True][1], Yref, alive, f"K chain N={N}", Y32=Y32)


@pytest.mark.parametrize("N,L,B,mode,T,merge_start,piece,cap,prefix", [
    (1024, 30, 2000, "SNICIT", 20, 4, 256, 2000, 0),   # pieces run layers 0..3, merge at 4
    (1024, 30, 2000, "SNICIT", 3, 0, 300, 2000, 0),    # default merge start past T: to T
    (1024, 16, 1500, "SNIG", 16, 0, 200, 1500, 0),     # every layer per piece
    (4096, 20, 1200, "SNICIT", 12, 3, 250, 1200, 0),   # binary first layer per piece
    (65536, 3, 192, "SNIG", 3, 0, 64, 192, 0),         # chunked binary first layer per piece
    (1024, 30, 2000, "SNICIT", 20, 4, 128, 700, 0),    # three batches per call, each streamed
    (1024, 30, 2000, "SNICIT", 20, 4, 256, 2000, 12),  # merges 4..11 deferred to layer 12
    (4096, 40, 1500, "SNICIT", 30, 6, 300, 1500, 40),  # deferred to the last merge layer (29)
])
def test_streamed_host_input_is_bitwise_equal(N, L, B, mode, T, merge_start, piece, cap, prefix):
    """Host FP32 rows copied in pieces, with the layers before the first
    cross-row step run per piece while later pieces copy, give the bits of the
    one-copy run (categories, activations, per-layer row counts), also with
    non-binary rows that take the float layer-0 kernel."""
    seed = 500 + N + T
    bias = sg.load().sdnn_reference_bias(N)
    Y0 = sg.generate_inputs(N, seed, 0, B)
    Y0[::7] *= 0.5  # some tiles hold other values than 0 and 1
    out = {}
    for streamed in (False, True):
        with sg.Engine(N, L, mode=mode, threshold=T, batch=cap, bias=bias, merge_start=merge_start,
                       streamed_input=streamed, input_piece_rows=piece,
                       input_prefix_layers=prefix) as eng:
            eng.generate_weights(seed)
            flags, ids = eng.infer(Y0)
            st = eng.stats()
            # activations and row counts are those of the last batch of the call
            out[streamed] = (flags, ids, eng.activations(B - (B - 1) // cap * cap),
                             eng.layer_rows(), st)
            flags2, ids2 = eng.infer(Y0)  # graphs and buffers reused
            assert np.array_equal(flags2, flags) and np.array_equal(ids2, ids)
    assert out[False][4]["input_pieces"] == 0
    assert out[True][4]["input_pieces"] == -(-min(B, cap) // piece), out[True][4]
    assert np.array_equal(out[True][1], out[False][1])
    assert np.array_equal(out[True][0], out[False][0])
    assert np.array_equal(out[True][2].view(np.uint32), out[False][2].view(np.uint32))
    rows_t, rows_f = out[True][3], out[False][3]
    if prefix:
        # deferred merges: more rows in the layers between the first merge layer
        # and the one the pieces ran to, the same counts before and after
        m = merge_start
        while m + 1 < T and m + 1 <= prefix:
            m += 1
        assert np.all(rows_t[merge_start:m] >= rows_f[merge_start:m])
        rows_t = np.concatenate([rows_t[:merge_start], rows_t[m:]])
        rows_f = np.concatenate([rows_f[:merge_start], rows_f[m:]])
    assert np.array_equal(rows_t, rows_f)
    if N <= 4096 and cap == B:
        Yref, alive, Y32 = _ref(_layers(N, L, seed), N, bias, Y0)
        _check(out[True][2], out[True][0], out[True][1], Yref, alive, f"streamed N={N}", Y32=Y32)


@pytest.mark.parametrize("N,L", [(4096, 480), (16384, 1920)])
def test_full_size_workload_snicit_equals_plain(N, L):
    """The SDGC-shaped workloads at full size (60000 seeded binary rows, 32
    nonzeros of 0.0625 per row, the reference bias): SNICIT (merging, the
    threshold at 30, chain kernels) gives the plain per-layer path's category
    set exactly, twice over (bitwise repeatable), and -- at N = 4096 -- the
    streamed host ingest gives the device path's flags and the first 32 rows
    match the FP64 oracle."""
    torch = pytest.importorskip("torch")
    B, seed = 60000, 20260101
    bias = sg.load().sdnn_reference_bias(N)
    d_in = torch.empty((B, N), dtype=torch.float32, device="cuda")
    sg.generate_inputs_device(N, seed, 0, B, d_in.data_ptr())
    d_flags = torch.zeros(B, dtype=torch.int32, device="cuda")
    with sg.Engine(N, L, mode="SNICIT", threshold=30, batch=B, bias=bias, num_centroids=50,
                   merge_start=10, merge_every=2) as eng:
        eng.generate_weights(seed, 32, 0.0625)
        runs = []
        for _ in range(2):
            d_flags.zero_()
            eng.infer_device(d_in.data_ptr(), B, d_flags.data_ptr())
            torch.cuda.synchronize()
            runs.append(d_flags.cpu().numpy().copy())
        st = eng.stats()
        assert st["device_post_choice"] == 1
        assert np.array_equal(runs[0], runs[1])
        snicit = runs[0]
        assert 0.01 * B < snicit.sum() < 0.99 * B
        if N == 4096:
            host = d_in.cpu().numpy()
            flags_h, ids_h = eng.infer(host)
            assert eng.stats()["input_pieces"] > 1
            assert np.array_equal(flags_h, snicit)
            assert np.array_equal(ids_h, np.flatnonzero(snicit))
            del host
        eng.set_mode("SNIG", L)
        d_flags.zero_()
        eng.infer_device(d_in.data_ptr(), B, d_flags.data_ptr())
        torch.cuda.synchronize()
        plain = d_flags.cpu().numpy().copy()
    assert np.array_equal(snicit, plain)
    if N == 4096:
        Y0 = sg.generate_inputs(N, seed, 0, 32)
        _, alive, _ = orc.infer(_layers(N, L, seed), N, bias, Y0, precision=64, want_y=False)
        assert np.array_equal(snicit[:32], alive.astype(np.int32))


@pytest.mark.parametrize("N,L,B,mode,flags", [
    (1024, 24, 300, "SNIG", {}),
    (1024, 24, 300, "BF", {"binary_first_layer": False}),
    (4096, 12, 200, "SNIG", {"placement": False}),
    (16384, 6, 64, "SNIG", {}),
    (65536, 3, 32, "SNIG", {}),
])
def test_plain_path_is_bitwise_equal_to_slot_order_evaluation(tmp_path, N, L, B, mode, flags):
    """Bit-exact parity of the plain path: the kernels' activations equal, bit
    for bit, a numpy evaluation of the recurrence in the kernels' summation
    order read from the packed-weight file (exact products with w = 1/16, so
    each fused multiply-add rounds like a float32 add); that evaluation agrees
    with the FP64 oracle within the FP32 bound (checked on the CPU)."""
    import packed_layout as pl
    seed = 900 + N
    bias = sg.load().sdnn_reference_bias(N)
    Y0 = sg.generate_inputs(N, seed, 0, B)
    path = tmp_path / "w.sdnnw"
    with sg.Engine(N, L, mode=mode, batch=B, bias=bias, **flags) as eng:
        eng.generate_weights(seed)
        eng.save_packed(path)
        got_flags, _ = eng.infer(Y0)
        Y = eng.activations(B)
    want = pl.plain_in_slot_order(pl.read_packed(path), Y0, bias)
    alive = (want > 0).any(axis=1)
    assert np.array_equal(got_flags, alive.astype(np.int32))
    assert alive.sum() > 0
    assert np.array_equal(Y[alive].view(np.uint32), want[alive].view(np.uint32))


@pytest.mark.parametrize("N,L,B,T,K", [(1024, 40, 600, 6, 16), (4096, 60, 400, 8, 32),
                                       (256, 40, 500, 4, 8)])
def test_sparse_residue_rows_match_dense_rows_and_oracle(N, L, B, T, K):
    """Residue rows that keep few nonzeros become sparse (position, value)
    lists after the threshold: the sparse update gives the dense update's
    category set and agrees with the FP64 oracle within the FP32 bound; it is
    bitwise repeatable.  Merging is off so that rows stay distinct and
    residues persist past the threshold."""
    seed = 4242 + N
    bias = sg.load().sdnn_reference_bias(N)
    Y0 = sg.generate_inputs(N, seed, 0, B)
    out = {}
    for sparse in (True, False):
        with sg.Engine(N, L, mode="SNICIT", threshold=T, batch=B, bias=bias, num_centroids=K,
                       merge=False, sparse_residue=sparse) as eng:
            eng.generate_weights(seed)
            flags, ids = eng.infer(Y0)
            Y = eng.activations(B)
            st = eng.stats()
            flags2, _ = eng.infer(Y0)
            Y2 = eng.activations(B)
            assert np.array_equal(flags, flags2)
            assert np.array_equal(Y.view(np.uint32), Y2.view(np.uint32))
            out[sparse] = (flags, ids, Y, st)
    st_s, st_d = out[True][3], out[False][3]
    assert st_d["sparse_row_layers"] == 0
    assert st_s["residue_rows"] > 0 and st_s["sparse_row_layers"] > 0, st_s
    print(f"N={N} t={T}: {st_s['residue_rows']} residue rows at the threshold "
          f"({st_s['sparse_residue_rows']} sparse), {st_s['sparse_row_layers']} sparse row-layers")
    assert np.array_equal(out[True][0], out[False][0])
    Yref, alive, Y32 = _ref(_layers(N, L, seed), N, bias, Y0)
    for sparse in (True, False):
        _check(out[sparse][2], out[sparse][0], out[sparse][1], Yref, alive,
               f"sparse={sparse} N={N}", Y32=Y32)
