"""The slot-order evaluation (tests/packed_layout.py) that the GPU's plain
path is compared with bit for bit must itself be right: on the CPU it agrees
with the FP64 oracle -- categories exactly, activations within the FP32
rounding bound of a sequential evaluation (no GPU)."""
import numpy as np
import pytest

import packed_layout as pl
import snicit_gb300 as sg
from oracle import oracle as orc


@pytest.mark.parametrize("N,L,B,placement", [(1024, 10, 64, True), (1024, 10, 64, False),
                                             (4096, 6, 32, True), (256, 12, 64, False)])
def test_slot_order_evaluation_matches_the_oracle(tmp_path, N, L, B, placement):
    seed = 5
    bias = sg.load().sdnn_reference_bias(N) or -0.3
    path = tmp_path / "w.sdnnw"
    with sg.Engine(N, L, mode="SNIG", batch=8, placement=placement) as e:
        e.generate_weights(seed)
        e.save_packed(path)
    Y0 = sg.generate_inputs(N, seed, 0, B)
    got = pl.plain_in_slot_order(pl.read_packed(path), Y0, bias)
    layers = [sg.generate_layer_csr(N, seed, l, 32, 0.0625) for l in range(L)]
    Y64, alive, _ = orc.infer(layers, N, bias, Y0, precision=64)
    Y32, _, _ = orc.infer(layers, N, bias, Y0, precision=32)
    assert np.array_equal((got > 0).any(axis=1).astype(np.int32), alive)
    rel = lambda Y: (np.abs(Y.astype(np.float64) - Y64) / np.maximum(1.0, np.abs(Y64))).max(axis=1)
    assert np.all(rel(got) <= np.maximum(1e-5, 4.0 * rel(Y32)))
