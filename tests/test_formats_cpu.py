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


def _read_packed(path):
    """Parses a packed-weight file (layout in csrc/packfile.h) into numpy
    arrays, one dict per layer."""
    b = path.read_bytes()
    magic = b[:8]
    N, L, Q, nq, G, placed, scale = np.frombuffer(b, np.int32, 7, 8)
    assert magic == b"SDNNPK01"
    pad = lambda n: (n + 63) // 64 * 64
    off, layers = 64, []
    for _ in range(L):
        constw, = np.frombuffer(b, np.int32, 1, off)
        nnz, nblocks, slots = np.frombuffer(b, np.int64, 3, off + 8)
        has_bias, = np.frombuffer(b, np.int32, 1, off + 40)
        off += 64
        grp = np.frombuffer(b, np.int32, G * nq + 1, off)
        off += pad((G * nq + 1) * 4)
        idx = np.frombuffer(b, np.uint16, nblocks * 128, off).reshape(nblocks, 32, 4)
        off += pad(nblocks * 128 * 2)
        if not constw:
            off += pad(nblocks * 128 * 4)
        if has_bias:
            off += pad(N * 4)
        pos = None
        if placed:
            pos = np.frombuffer(b, np.int32, N, off)
            off += pad(N * 4)
        layers.append(dict(grp=grp, idx=idx, pos=pos, nnz=int(nnz)))
    return dict(N=int(N), Q=int(Q), nq=int(nq), G=int(G), scale=int(scale), layers=layers)


@pytest.mark.parametrize("N,L,placement", [(256, 2, False), (1024, 3, True), (4096, 2, True),
                                           (16384, 2, True), (65536, 1, True)])
def test_packed_layout_is_bank_conflict_free_and_holds_every_edge(tmp_path, N, L, placement):
    """The layout every layer kernel relies on: in each slot the 32 lanes'
    indices (edges and padding alike) fall in 32 distinct shared-memory banks;
    the real slots hold exactly the layer's edges (input position -> output
    position, mapped back to neurons through the placement); and a (group,
    chunk) takes exactly the lower bound max(largest lane degree, largest bank
    degree) of slots, rounded up to a block of 4."""
    seed, path = 11, tmp_path / "w.sdnnw"
    with sg.Engine(N, L, mode="SNICIT", batch=8, placement=placement) as e:
        e.generate_weights(seed)
        e.save_packed(path)
    f = _read_packed(path)
    Q, nq, G, scale = f["Q"], f["nq"], f["G"], f["scale"]
    prev_inv = np.arange(N)  # input position -> neuron (layer 0: the caller's order)
    for l, lay in enumerate(f["layers"]):
        idx, grp = lay["idx"], lay["grp"]
        jl = idx.astype(np.int64) // scale  # chunk-local index per (block, lane, slot)
        banks = jl % 32
        # distinct banks per slot: sort the 32 lanes' banks of every (block, slot)
        per_slot = np.sort(banks.transpose(0, 2, 1), axis=2)
        assert np.array_equal(per_slot, np.broadcast_to(np.arange(32), per_slot.shape))
        real = jl < Q
        inv = np.argsort(lay["pos"]) if lay["pos"] is not None else np.arange(N)
        got_in, got_out = [], []
        for g in range(G):
            for q in range(nq):
                b0, b1 = grp[g * nq + q], grp[g * nq + q + 1]
                if b1 == b0:
                    continue
                m = real[b0:b1]                      # [blocks, lane, slot]
                lanes = np.broadcast_to(np.arange(32)[None, :, None], m.shape)
                got_in.append(q * Q + jl[b0:b1][m])
                got_out.append(32 * g + lanes[m])
                # slot count against the lower bound of this (group, chunk)
                lane_deg = m.sum(axis=(0, 2))
                bank_deg = np.bincount(banks[b0:b1][m], minlength=32)
                bound = max(lane_deg.max(), bank_deg.max())
                # (an edge colouring with exactly that many colours, blocks of 4)
                assert 4 * (b1 - b0) == (bound + 3) // 4 * 4, (l, g, q, b1 - b0, bound)
        got_in = prev_inv[np.concatenate(got_in)]
        got_out = inv[np.concatenate(got_out)]
        r, c, _ = sg.generate_layer_coo(N, seed, l, 32, 0.0625)
        assert len(got_in) == len(r) == lay["nnz"]
        want = np.sort(r.astype(np.int64) * N + c)
        assert np.array_equal(np.sort(got_in * N + got_out), want)
        if placement and l >= 1 and nq == 1:
            # the placement balances this layer's banks (measured 0.86-0.87)
            assert lay["nnz"] / (idx.shape[0] * 128) >= 0.8
        prev_inv = inv
