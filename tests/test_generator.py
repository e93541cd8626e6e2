"""The seeded synthetic data follows its specification (no GPU)."""
import numpy as np

import snicit_gb300 as sg

MASK = (1 << 64) - 1
GOLDEN = 0x9E3779B97F4A7C15


def fin(z):
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK
    return z ^ (z >> 31)


def key(seed, kind, a, b):
    k = fin((seed + GOLDEN) & MASK)
    k = fin(k ^ ((kind * 0xD1B54A32D192ED03 + GOLDEN) & MASK))
    k = fin(k ^ ((a * 0xABC98388FB8FAC03 + GOLDEN) & MASK))
    k = fin(k ^ ((b * 0x8CB92BA72F3D8DD7 + GOLDEN) & MASK))
    return k


def draw(k, i):
    return fin((k + (i + 1) * GOLDEN) & MASK)


def py_row_cols(seed, layer, row, N, nnz):
    k = key(seed, 1, layer, row)
    out, i = [], 0
    while len(out) < nnz:
        c = (draw(k, i) * N) >> 64
        i += 1
        if c not in out:
            out.append(c)
    return out


def py_input_row(seed, row, N):
    k = key(seed, 2, 0, row)
    u = sorted(draw(k, i) >> 11 for i in range(9))
    rho = 0.95 * (u[1] * (1.0 / 9007199254740992.0))
    return np.array([1.0 if (draw(k, 9 + j) >> 11) * (1.0 / 9007199254740992.0) < rho else 0.0
                     for j in range(N)], np.float32)


def test_weight_rows_match_the_restated_stream():
    r, c, v = sg.generate_layer_coo(256, 11, 3, 32, 0.0625)
    c = c.reshape(256, 32)
    for row in (0, 1, 77, 255):
        assert list(c[row]) == py_row_cols(11, 3, row, 256, 32)
    assert np.all(v == 0.0625)
    assert np.array_equal(r, np.repeat(np.arange(256), 32))


def test_weight_rows_are_distinct_uniform():
    N = 1024
    _, c, _ = sg.generate_layer_coo(N, 5, 0, 32)
    c = c.reshape(N, 32)
    assert all(len(set(row)) == 32 for row in c)
    indeg = np.bincount(c.ravel(), minlength=N)
    assert abs(indeg.mean() - 32) < 1e-9
    # binomial in-degree: variance close to 32 * (1 - 32/N)
    assert 20 < indeg.var() < 45


def test_inputs_match_the_restated_stream_and_density():
    N = 512
    Y = sg.generate_inputs(N, 9, 100, 3)
    for i in range(3):
        assert np.array_equal(Y[i], py_input_row(9, 100 + i, N))
    big = sg.generate_inputs(1024, 2026, 0, 4000)
    assert set(np.unique(big)) <= {0.0, 1.0}
    assert abs(big.mean() - 0.19) < 0.01  # marginal entry probability 0.19
    # row windows are independent of how they are requested
    assert np.array_equal(sg.generate_inputs(1024, 2026, 1000, 5), big[1000:1005])
    # per-row densities spread like 0.95 * Beta(2, 8): std ~= 0.95 * 0.1206
    dens = big.mean(1)
    assert 0.09 < dens.std() < 0.14


def test_survival_fraction_is_inside_the_reseed_window():
    """The per-row density model gives 1%..99% survivors where i.i.d. inputs die."""
    from oracle import oracle as orc
    N, L = 1024, 24
    layers = [sg.generate_layer_csr(N, 20260101, l) for l in range(L)]
    Y = sg.generate_inputs(N, 20260101, 0, 1500)
    _, alive, _ = orc.infer(layers, N, -0.3, Y, precision=32, want_y=False)
    assert 0.01 < alive.mean() < 0.99
    rng = np.random.default_rng(0)
    iid = (rng.random((300, N)) < 0.19).astype(np.float32)
    _, alive_iid, dead = orc.infer(layers, N, -0.3, iid, precision=32, want_y=False)
    assert alive_iid.sum() == 0 and dead.max() <= 4


def test_oracle_generator_restates_the_engine_generator():
    """The oracle's C restatement of the synthetic data (used by the CPU
    baseline and the reference arm of the benchmark) gives the engine's bits."""
    from oracle import oracle as orc
    for N in (256, 4096, 65536):
        assert np.array_equal(orc.gen_inputs(N, 2026, 12345, 3), sg.generate_inputs(N, 2026, 12345, 3))
        ro, c, v = orc.gen_layer_csr(N, 20260101, 7)
        r2, c2, v2 = sg.generate_layer_coo(N, 20260101, 7, 32, 0.0625)
        assert np.array_equal(c, c2) and np.array_equal(v, v2)
        assert np.array_equal(ro, np.arange(N + 1, dtype=np.int32) * 32)


def test_streamed_port_equals_the_fp32_port():
    """oracle_port_stream (weights generated per layer, rows in timed groups)
    computes the same bits as oracle_infer's FP32 port."""
    from oracle import oracle as orc
    N, L, seed, bias = 1024, 30, 20260101, -0.3
    Y0 = orc.gen_inputs(N, seed, 0, 300)
    layers = [orc.gen_layer_csr(N, seed, l) for l in range(L)]
    want, alive_w, _ = orc.infer(layers, N, bias, Y0, precision=32, nthreads=4)
    alive, secs, Y = orc.port_stream(N, L, seed, bias, Y0, [100, 150, 50], nthreads=3)
    assert np.array_equal(alive, alive_w)
    assert np.array_equal(Y.view(np.uint32), want.view(np.uint32))
    assert (secs > 0).all() and 0 < alive.sum() < 300


def test_streamed_fp64_oracle_equals_the_fp64_oracle():
    from oracle import oracle as orc
    N, L, seed, bias = 512, 25, 20260101, -0.3
    Y0 = orc.gen_inputs(N, seed, 0, 200)
    layers = [orc.gen_layer_csr(N, seed, l) for l in range(L)]
    want, alive_w, _ = orc.infer(layers, N, bias, Y0, precision=64, nthreads=4)
    Y, alive = orc.infer_stream64(N, L, seed, bias, Y0, nthreads=3)
    assert np.array_equal(alive, alive_w) and 0 < alive.sum() < 200
    assert np.array_equal(Y, want)


# ---- RadiX-Net-structured layers --------------------------------------------

def _hash(v, M, width=16):
    """The reference's HashReorder (src/SDGC/reorder/hash.h:14-22) with M
    buckets of `width`: v -> v / M + (v % M) * width."""
    return v // M + (v % M) * width


def test_radixnet_matches_the_oracle_restatement():
    from oracle import oracle as orc
    for N, block in ((1024, 16), (4096, 16), (256, 8), (64, 32)):
        M = N // block
        for layer in range(0, 2 * int(np.log2(M)) + 1):
            r, c, v = sg.generate_radixnet_layer_coo(N, layer, block)
            ro, oc, ov = orc.gen_radixnet_csr(N, layer, block)
            assert np.array_equal(np.repeat(np.arange(N), np.diff(ro)), r)
            assert np.array_equal(oc, c) and np.array_equal(ov, v)


def test_radixnet_structure_is_the_one_the_reference_kernels_read():
    """Every output has 32 in-edges and every input 32 out-edges; after the
    reference's hash reorder, output node c (16 consecutive outputs) reads the
    16 inputs of node c and the 16 of node c + stride / 16, with the
    reference's strides 16 * 2^l for layers 0 .. log2(M) - 1
    (src/SDGC/SNICIT/SNICIT.hpp:329-342, src/SDGC/XY/kernel.hpp:24-35,71-91),
    and the same cycle again after that."""
    for N in (1024, 4096, 16384):
        M = N // 16
        k = int(np.log2(M))
        for layer in list(range(k + 2)) + [119]:
            r, c, _ = sg.generate_radixnet_layer_coo(N, layer, 16)
            assert np.array_equal(np.bincount(r, minlength=N), np.full(N, 32))
            assert np.array_equal(np.bincount(c, minlength=N), np.full(N, 32))
            hr, hc = _hash(r, M), _hash(c, M)
            stride = 16 * 2 ** (layer % k)
            for node in (0, 1, M // 2, M - 1):
                ins = np.unique(hr[hc // 16 == node])
                want = np.concatenate([node * 16 + np.arange(16),
                                       (node * 16 + stride + np.arange(16)) % N])
                assert np.array_equal(ins, np.sort(want)), (N, layer, node)


def test_radixnet_rejects_shapes_without_a_power_of_two_node_count():
    import ctypes
    n = 48 * 32
    r = np.zeros(n, np.int32)
    c = np.zeros(n, np.int32)
    v = np.zeros(n, np.float32)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    L = sg.load()
    assert L.sdnn_generate_radixnet_layer_coo(48 * 16, 16, 0, 0.0625, P(r), P(c), P(v)) != 0
    assert L.sdnn_generate_radixnet_layer_coo(1024, 0, 0, 0.0625, P(r), P(c), P(v)) != 0
    assert L.sdnn_generate_radixnet_layer_coo(16, 16, 0, 0.0625, P(r), P(c), P(v)) != 0


def test_radixnet_weights_are_emitted_as_sdgc_tsv(tmp_path):
    """An engine with RadiX-Net layers writes them in the SDGC layout
    (dir/n{N}-l{l}.tsv, 1-based "row col value" lines), the same edges as the
    generator's COO."""
    N, L = 256, 5
    with sg.Engine(N, L, mode="SNIG", batch=4) as eng:
        eng.generate_radixnet(16, 0.0625)
        eng.write_weights_tsv(tmp_path)
    for l in range(L):
        t = np.loadtxt(tmp_path / f"n{N}-l{l + 1}.tsv", ndmin=2)
        r, c, v = sg.generate_radixnet_layer_coo(N, l, 16)
        assert np.array_equal(t[:, 0].astype(np.int64) - 1, r)
        assert np.array_equal(t[:, 1].astype(np.int64) - 1, c)
        assert np.allclose(t[:, 2], v)
