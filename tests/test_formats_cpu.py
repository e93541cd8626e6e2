"""Binary file formats (no GPU): packed-weight files and binary input files.

Packed weights are written by host packing, so a save -> load -> save round
trip must give the identical file, and a loaded file must be rejected when it
does not fit the engine or is damaged.  Binary inputs must read back exactly
(FP32 and one-bit encodings, any row window).
"""
import os

import numpy as np
import pytest

import snicit_gb300 as sg
from snicit_gb300._lib import SdnnError


@pytest.mark.parametrize("N,L,placement", [(1024, 4, True), (256, 3, False), (4096, 2, True)])
def test_packed_weights_round_trip(tmp_path, N, L, placement):
    a, b = tmp_path / "a.sdnnw", tmp_path / "b.sdnnw"
    with sg.Engine(N, L, mode="SNICIT", batch=16, placement=placement) as e:
        e.generate_weights(7)
        e.save_packed(a)
    with sg.Engine(N, L, mode="SNICIT", batch=16, placement=placement) as e:
        e.load_packed(a)
        e.save_packed(b)
    assert a.read_bytes() == b.read_bytes()
    assert a.stat().st_size > 1024


def test_packed_weights_with_values_and_bias(tmp_path):
    N, L = 256, 2
    rng = np.random.default_rng(3)
    path = tmp_path / "w.sdnnw"
    with sg.Engine(N, L, mode="SNIG", batch=8) as e:
        for l in range(L):
            r, c = np.nonzero(rng.random((N, N)) < 0.05)
            e.set_layer_coo(l, r, c, rng.standard_normal(len(r)).astype(np.float32))
            e.set_layer_bias(l, rng.uniform(-0.1, 0, N).astype(np.float32))
        e.save_packed(path)
    with sg.Engine(N, L, mode="SNIG", batch=8) as e:
        e.load_packed(path)
        with pytest.raises(SdnnError):  # biases travel inside the file
            e.set_layer_bias(0, np.zeros(N, np.float32))
        e.save_packed(tmp_path / "w2.sdnnw")
    assert path.read_bytes() == (tmp_path / "w2.sdnnw").read_bytes()


def test_packed_weights_rejected_when_they_do_not_fit(tmp_path):
    path = tmp_path / "w.sdnnw"
    with sg.Engine(1024, 3, batch=8) as e:
        e.generate_weights(1)
        e.save_packed(path)
    for n, l in ((1024, 4), (2048, 3)):
        with sg.Engine(n, l, batch=8) as e:
            with pytest.raises(SdnnError) as ei:
                e.load_packed(path)
            assert ei.value.code == 5
    bad = tmp_path / "bad.sdnnw"
    bad.write_bytes(path.read_bytes()[: path.stat().st_size // 2])  # truncated
    with sg.Engine(1024, 3, batch=8) as e:
        with pytest.raises(SdnnError) as ei:
            e.load_packed(bad)
        assert ei.value.code == 5
        with pytest.raises(SdnnError) as ei:
            e.load_packed(tmp_path / "missing.sdnnw")
        assert ei.value.code == 4


@pytest.mark.parametrize("bits", [False, True])
def test_binary_inputs_round_trip(tmp_path, bits):
    N = 1000  # not a multiple of 64: the last word of a bit row is partial
    Y = sg.generate_inputs(N, 5, 0, 37)
    path = tmp_path / "in.bin"
    sg.write_inputs_bin(path, Y, bits=bits)
    assert sg.inputs_bin_info(path) == (N, 37, 1 if bits else 0)
    assert np.array_equal(sg.read_inputs_bin(path, N), Y)
    assert np.array_equal(sg.read_inputs_bin(path, N, 10, 5), Y[10:15])
    expect = 32 + 37 * (((N + 63) // 64) * 8 if bits else N * 4)
    assert os.path.getsize(path) == expect


def test_binary_inputs_errors(tmp_path):
    Y = np.full((2, 64), 0.5, np.float32)
    with pytest.raises(SdnnError):
        sg.write_inputs_bin(tmp_path / "x.bin", Y, bits=True)  # not 0/1
    sg.write_inputs_bin(tmp_path / "y.bin", Y)
    with pytest.raises(SdnnError):
        sg.read_inputs_bin(tmp_path / "y.bin", 64, 1, 5)  # past the end
    with pytest.raises(SdnnError):
        sg.read_inputs_bin(tmp_path / "y.bin", 32)  # other width
    (tmp_path / "z.bin").write_bytes(b"not an input file at all, really")
    with pytest.raises(SdnnError):
        sg.inputs_bin_info(tmp_path / "z.bin")


def test_pack_bits_matches_the_file_encoding(tmp_path):
    N = 1000
    Y = sg.generate_inputs(N, 9, 0, 11)
    path = tmp_path / "in.bin"
    sg.write_inputs_bin(path, Y, bits=True)
    words = np.frombuffer(path.read_bytes()[32:], dtype=np.uint64).reshape(11, -1)
    assert np.array_equal(sg.pack_bits(Y), words)
