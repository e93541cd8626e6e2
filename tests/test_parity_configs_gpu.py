"""Parity at the SDGC-shaped benchmark configurations, at full size, and on
the reference kernels' own fixtures (GPU, through the C ABI).

* 1024 x 120 x 60000 (every row): SNICIT and the plain path against the FP64
  oracle -- category set exact, final activations within 1e-5 relative on
  every row (|gpu - fp64| / max(1, |fp64|), the plain bound: no per-row
  loosening on a 120-layer net) -- and against the reference's own
  bf_inference / snig_inference kernels run by oracle/ref_harness.cpp (same
  category set).
* 4096 x 480 x 60000: SNICIT on all rows; activations of a seeded 2000-row
  subset within 1e-5 of the FP64 oracle, categories of the subset exact.
* 65536 x 1920 x 60000: SNICIT's category set equals the plain per-layer
  path's; 32 seeded rows (16 survivors, 16 others) against the FP64 oracle.
* tests/golden/*.npz (outputs of the reference's kernels): in every mode the
  engine's categories equal the reference kernels' exactly, and its
  activations are within the suite's bound of the FP64 oracle and of the
  reference's activations.
"""
import glob
import os
import struct
import subprocess

import numpy as np
import pytest

import snicit_gb300 as sg
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
RTOL = 1e-5
SEED = 20260101
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "*.npz")))


def _rel_rows(Y, Yref):
    return (np.abs(Y.astype(np.float64) - Yref) / np.maximum(1.0, np.abs(Yref))).max(axis=1)


def _device_inputs(torch, N, B):
    d_in = torch.empty((B, N), dtype=torch.float32, device="cuda")
    sg.generate_inputs_device(N, SEED, 0, B, d_in.data_ptr())
    return d_in


def _run_device(torch, eng, d_in, B):
    d_flags = torch.zeros(B, dtype=torch.int32, device="cuda")
    eng.infer_device(d_in.data_ptr(), B, d_flags.data_ptr())
    torch.cuda.synchronize()
    return d_flags.cpu().numpy().copy()


def _ref_harness(tmp_path, N, L, bias, Y0, layers=None):
    """Runs the reference's bf_inference / snig_inference (built from its
    sources into oracle/_ref/) on the synthetic net (or on `layers`, CSR by
    input row); returns (Y_bf, Y_snig) or None when the reference kernels are
    not built here."""
    module = os.path.join(ROOT, "oracle", "_ref", "sdgc_ref.cubin")
    if not os.path.exists(module):
        return None
    harness = str(tmp_path / "ref_harness")
    subprocess.run(["nvcc", "-O2", "-std=c++17", os.path.join(ROOT, "oracle", "ref_harness.cpp"),
                    "-o", harness, "-lcuda"], check=True)
    B = Y0.shape[0]
    inp, outp = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    with open(inp, "wb") as f:
        f.write(struct.pack("<iiiif", N, L, B, N, bias))  # one section: N fits 48 KB of shared memory
        for l in range(L):
            ro, c, v = layers[l] if layers is not None else orc.gen_layer_csr(N, SEED, l)
            order = np.argsort(c.reshape(N, 32), axis=1, kind="stable")
            c = np.take_along_axis(c.reshape(N, 32), order, 1).ravel()
            f.write(struct.pack("<i", len(c)))
            f.write(ro.astype("<i4").tobytes())
            f.write(c.astype("<i4").tobytes())
            f.write(v.astype("<f4").tobytes())
        f.write(Y0.astype("<f4").tobytes())
    r = subprocess.run([harness, module, inp, outp], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    raw = np.fromfile(outp, dtype="<f4", count=2 * B * N)
    os.remove(inp)
    os.remove(outp)
    return raw[:B * N].reshape(B, N), raw[B * N:].reshape(B, N)


def test_config_1024x120_every_row_against_fp64_and_reference_kernels(tmp_path):
    torch = pytest.importorskip("torch")
    N, L, B = 1024, 120, 60000
    bias = sg.load().sdnn_reference_bias(N)
    Y0 = sg.generate_inputs(N, SEED, 0, B)
    Yref, alive, _ = orc.infer([orc.gen_layer_csr(N, SEED, l) for l in range(L)], N, bias, Y0,
                               precision=64)
    assert 0.01 * B < alive.sum() < 0.99 * B
    want = np.flatnonzero(alive)
    got = {}
    with sg.Engine(N, L, mode="SNICIT", threshold=30, batch=B, bias=bias, num_centroids=50) as eng:
        eng.generate_weights(SEED)
        for mode in ("SNICIT", "SNIG", "BF"):
            eng.set_mode(mode, 30 if mode == "SNICIT" else L)
            flags, ids = eng.infer(Y0)
            Y = eng.activations(B)
            assert np.array_equal(ids, want), f"{mode}: category set"
            assert np.array_equal(flags, alive)
            err = _rel_rows(Y, Yref)
            print(f"1024x120 {mode}: max error {err.max():.3g} over {B} rows "
                  f"({len(want)} survivors), bound {RTOL:g} on every row")
            assert err.max() <= RTOL, f"{mode}: {err.max():.3g} on {(err > RTOL).sum()} rows"
            got[mode] = Y
    ref = _ref_harness(tmp_path, N, L, bias, Y0)
    if ref is None:
        pytest.skip("reference kernels not built (oracle/ref_build.sh needs the reference tree)")
    for name, Yr in zip(("bf_inference", "snig_inference"), ref):
        assert np.array_equal((Yr > 0).any(1).astype(np.int32), alive), name
        e_ref = _rel_rows(Yr, Yref).max()
        e_ours = _rel_rows(got["SNIG"], Yr.astype(np.float64)).max()
        print(f"reference {name}: vs FP64 {e_ref:.3g}, vs the engine {e_ours:.3g}")
        assert e_ref <= RTOL and e_ours <= 2 * RTOL


def test_config_4096x480_subset_activations_against_fp64():
    torch = pytest.importorskip("torch")
    N, L, B = 4096, 480, 60000
    bias = sg.load().sdnn_reference_bias(N)
    d_in = _device_inputs(torch, N, B)
    with sg.Engine(N, L, mode="SNICIT", threshold=30, batch=B, bias=bias, num_centroids=50,
                   merge_start=10, merge_every=2) as eng:
        eng.generate_weights(SEED)
        flags = _run_device(torch, eng, d_in, B)
        Y = eng.activations(B)
    rows = np.sort(np.random.default_rng([SEED, 2000]).choice(B, 2000, replace=False))
    Y0s = np.concatenate([orc.gen_inputs(N, SEED, int(r), 1) for r in rows])
    Yref, alive = orc.infer_stream64(N, L, SEED, bias, Y0s)
    assert np.array_equal(flags[rows], alive)
    assert alive.sum() > 20
    err = _rel_rows(Y[rows], Yref)
    print(f"4096x480 SNICIT: {alive.sum()} survivors in the 2000-row subset, "
          f"max error {err.max():.3g}, bound {RTOL:g} on every row")
    assert err.max() <= RTOL


def test_config_65536x1920_snicit_equals_plain_and_fp64_rows():
    torch = pytest.importorskip("torch")
    N, L, B = 65536, 1920, 60000
    bias = sg.load().sdnn_reference_bias(N)
    d_in = _device_inputs(torch, N, B)
    with sg.Engine(N, L, mode="SNICIT", threshold=30, batch=B, bias=bias, num_centroids=50) as eng:
        eng.generate_weights(SEED)
        snicit = _run_device(torch, eng, d_in, B)
        head = 4096
        Y = eng.activations(head)
        eng.set_mode("SNIG", L)
        plain = _run_device(torch, eng, d_in, B)
    assert np.array_equal(snicit, plain)
    assert 0.01 * B < snicit.sum() < 0.99 * B
    rng = np.random.default_rng([SEED, 32])
    live = np.flatnonzero(snicit[:head])
    dead = np.flatnonzero(snicit[:head] == 0)
    rows = np.sort(np.concatenate([rng.choice(live, 16, replace=False),
                                   rng.choice(dead, 16, replace=False)]))
    Y0s = np.concatenate([orc.gen_inputs(N, SEED, int(r), 1) for r in rows])
    Yref, alive = orc.infer_stream64(N, L, SEED, bias, Y0s)
    assert np.array_equal(snicit[rows], alive)
    err = _rel_rows(Y[rows], Yref)
    print(f"65536x1920: {snicit.sum()} survivors, SNICIT == plain; 32 rows vs FP64 max error "
          f"{err.max():.3g}")
    assert err.max() <= RTOL


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
@pytest.mark.parametrize("mode", ["BF", "SNIG", "SNICIT"])
def test_engine_on_reference_kernel_fixtures(path, mode):
    """The engine on the inputs and weights the reference's kernels ran on:
    its categories are theirs exactly.  Activations: the engine within the
    suite's bound of the FP64 oracle (per row max(1e-5, 4x the FP32 port's
    error), these are short nets still in the transient), and so within that
    bound plus the reference kernel's own FP64 error of the reference's
    activations."""
    d = np.load(path)
    N, L, B = int(d["N"]), int(d["L"]), int(d["B"])
    bias = float(d["bias"])
    layers = [(d["row_off"][l].astype(np.int32), d["cols"][l].astype(np.int32),
               d["vals"][l].astype(np.float32)) for l in range(L)]
    with sg.Engine(N, L, mode=mode, threshold=max(1, L // 3), batch=B, bias=bias,
                   num_centroids=16) as eng:
        for l, (ro, c, v) in enumerate(layers):
            eng.set_layer_csr(l, ro, c, v)
        flags, ids = eng.infer(d["Y0"])
        Y = eng.activations(B)
    Y64, alive64, _ = orc.infer(layers, N, bias, d["Y0"], precision=64)
    Y32, _, _ = orc.infer(layers, N, bias, d["Y0"], precision=32)
    tol = np.maximum(RTOL, 4.0 * _rel_rows(Y32, Y64))
    err = _rel_rows(Y, Y64)
    assert (err <= tol).all(), f"vs FP64: {err.max():.3g}"
    for key in ("Y_bf", "Y_snig"):
        ref = d[key]
        alive = (ref > 0).any(1).astype(np.int32)
        assert np.array_equal(alive, alive64), key
        assert np.array_equal(flags, alive), key
        assert np.array_equal(ids, np.flatnonzero(alive)), key
        err_ref = _rel_rows(ref, Y64)
        err_ours = _rel_rows(Y, ref.astype(np.float64))
        assert (err_ours <= tol + err_ref).all(), f"{key}: {err_ours.max():.3g}"
