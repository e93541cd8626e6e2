"""RadiX-Net-structured nets (GPU, through the C ABI).

The engine's RadiX-Net generator (radix 2, dense blocks of 16 neurons, weights
1/16) builds the structure the reference's SNICIT / XY kernels are written
for.  On those nets:

* 1024 x 120 x 60000 (every row): every mode's category set equals the FP64
  oracle's (weights from the oracle's own restatement of the generator) and
  activations are within 1e-5 relative on every row; the reference's own
  bf_inference / snig_inference kernels (oracle/ref_harness.cpp) give the
  same category set on the same net.
* 4096 x 480 x 60000: SNICIT with row merging equals the plain path's
  category set; a seeded 1000-row subset matches the FP64 oracle.
* 65536 x 120 x 8192 (input chunks): SNICIT == plain; 16 seeded rows (8
  survivors, 8 not) against the FP64 oracle.
"""
import numpy as np
import pytest

import snicit_gb300 as sg
from oracle import oracle as orc
from test_parity_configs_gpu import RTOL, SEED, _ref_harness, _rel_rows

pytestmark = pytest.mark.gpu


def test_radixnet_1024x120_every_row_against_fp64_and_reference_kernels(tmp_path):
    pytest.importorskip("torch")
    N, L, B = 1024, 120, 60000
    bias = sg.load().sdnn_reference_bias(N)
    Y0 = sg.generate_inputs(N, SEED, 0, B)
    layers = [orc.gen_radixnet_csr(N, l) for l in range(L)]
    Yref, alive, _ = orc.infer(layers, N, bias, Y0, precision=64)
    assert 0.01 * B < alive.sum() < 0.99 * B
    want = np.flatnonzero(alive)
    with sg.Engine(N, L, mode="SNICIT", threshold=30, batch=B, bias=bias,
                   num_centroids=50) as eng:
        eng.generate_radixnet(16, 0.0625)
        for mode in ("SNICIT", "SNIG", "BF"):
            eng.set_mode(mode, 30 if mode == "SNICIT" else L)
            flags, ids = eng.infer(Y0)
            Y = eng.activations(B)
            assert np.array_equal(ids, want), f"{mode}: category set"
            assert np.array_equal(flags, alive)
            err = _rel_rows(Y, Yref)
            print(f"RadiX-Net 1024x120 {mode}: {len(want)} survivors of {B}, "
                  f"max error {err.max():.3g}, bound {RTOL:g} on every row")
            assert err.max() <= RTOL, f"{mode}: {err.max():.3g}"
            if mode == "SNIG":
                y_snig = Y
    ref = _ref_harness(tmp_path, N, L, bias, Y0, layers)
    if ref is None:
        pytest.skip("reference kernels not built (oracle/ref_build.sh needs the reference tree)")
    for name, Yr in zip(("bf_inference", "snig_inference"), ref):
        assert np.array_equal((Yr > 0).any(1).astype(np.int32), alive), name
        e_ours = _rel_rows(y_snig, Yr.astype(np.float64)).max()
        print(f"reference {name} on the RadiX-Net net: same category set, engine within "
              f"{e_ours:.3g} of its activations")
        assert e_ours <= 2 * RTOL


def test_radixnet_4096x480_snicit_equals_plain_and_fp64_subset():
    torch = pytest.importorskip("torch")
    N, L, B = 4096, 480, 60000
    bias = sg.load().sdnn_reference_bias(N)
    d_in = torch.empty((B, N), dtype=torch.float32, device="cuda")
    sg.generate_inputs_device(N, SEED, 0, B, d_in.data_ptr())
    d_flags = torch.zeros(B, dtype=torch.int32, device="cuda")
    with sg.Engine(N, L, mode="SNICIT", threshold=30, batch=B, bias=bias, num_centroids=50,
                   merge_start=10, merge_every=2) as eng:
        eng.generate_radixnet(16, 0.0625)
        eng.infer_device(d_in.data_ptr(), B, d_flags.data_ptr())
        torch.cuda.synchronize()
        snicit = d_flags.cpu().numpy().copy()
        Y = eng.activations(B)
        eng.set_mode("SNIG", L)
        d_flags.zero_()
        eng.infer_device(d_in.data_ptr(), B, d_flags.data_ptr())
        torch.cuda.synchronize()
        plain = d_flags.cpu().numpy().copy()
    assert np.array_equal(snicit, plain)
    assert 0.01 * B < snicit.sum() < 0.99 * B
    rows = np.sort(np.random.default_rng([SEED, 1000]).choice(B, 1000, replace=False))
    Y0s = np.concatenate([orc.gen_inputs(N, SEED, int(r), 1) for r in rows])
    layers = [orc.gen_radixnet_csr(N, l) for l in range(L)]
    Yref, alive, _ = orc.infer(layers, N, bias, Y0s, precision=64)
    assert np.array_equal(snicit[rows], alive)
    err = _rel_rows(Y[rows], Yref)
    print(f"RadiX-Net 4096x480: {snicit.sum()} survivors, SNICIT == plain; 1000 rows vs FP64 "
          f"max error {err.max():.3g}")
    assert err.max() <= RTOL


def test_radixnet_65536_input_chunks_snicit_equals_plain_and_fp64_rows():
    """The input-chunked kernels (chunks of 16384) on a RadiX-Net net, whose
    nodes' 16 outputs all read the same 32 inputs."""
    torch = pytest.importorskip("torch")
    N, L, B = 65536, 120, 8192
    bias = sg.load().sdnn_reference_bias(N)
    d_in = torch.empty((B, N), dtype=torch.float32, device="cuda")
    sg.generate_inputs_device(N, SEED, 0, B, d_in.data_ptr())
    d_flags = torch.zeros(B, dtype=torch.int32, device="cuda")
    with sg.Engine(N, L, mode="SNICIT", threshold=30, batch=B, bias=bias,
                   num_centroids=50) as eng:
        eng.generate_radixnet(16, 0.0625)
        eng.infer_device(d_in.data_ptr(), B, d_flags.data_ptr())
        torch.cuda.synchronize()
        snicit = d_flags.cpu().numpy().copy()
        Y = eng.activations(B)
        eng.set_mode("SNIG", L)
        d_flags.zero_()
        eng.infer_device(d_in.data_ptr(), B, d_flags.data_ptr())
        torch.cuda.synchronize()
        plain = d_flags.cpu().numpy().copy()
    assert np.array_equal(snicit, plain)
    assert 0 < snicit.sum() < B
    rng = np.random.default_rng([SEED, 16])
    live, dead = np.flatnonzero(snicit), np.flatnonzero(snicit == 0)
    rows = np.sort(np.concatenate([rng.choice(live, min(8, len(live)), replace=False),
                                   rng.choice(dead, min(8, len(dead)), replace=False)]))
    Y0s = np.concatenate([orc.gen_inputs(N, SEED, int(r), 1) for r in rows])
    layers = [orc.gen_radixnet_csr(N, l) for l in range(L)]
    Yref, alive, _ = orc.infer(layers, N, bias, Y0s, precision=64)
    assert np.array_equal(snicit[rows], alive)
    err = _rel_rows(Y[rows], Yref)
    print(f"RadiX-Net 65536x120: {snicit.sum()} survivors of {B}, SNICIT == plain; "
          f"{len(rows)} rows vs FP64 max error {err.max():.3g}")
    assert err.max() <= RTOL
