"""Test helpers: the packed-weight file (layout in csrc/packfile.h) read into
numpy, and a CPU evaluation of the plain recurrence in the layer kernel's own
summation order.

The kernel computes output c of a row as acc = fmaf(w_s, y[j_s], acc) over
its slots s in storage order: chunk by chunk, block by block, the 4 slots of
a block in turn (padding slots read a zero column).  With one power-of-two
weight value w (the SDGC layers: 0.0625) every product w·y is exact, so each
fmaf rounds exactly like a float32 add of w·y -- and this numpy evaluation
gives the kernel's bits, not just values within rounding.
"""
import numpy as np


def read_packed(path):
    """Returns dict(N, Q, nq, G, scale, layers=[dict(grp, idx, pos, nnz, constw, wconst)])."""
    b = open(path, "rb").read()
    assert b[:8] == b"SDNNPK01"
    N, L, Q, nq, G, placed, scale = (int(x) for x in np.frombuffer(b, np.int32, 7, 8))
    pad = lambda n: (n + 63) // 64 * 64
    off, layers = 64, []
    for _ in range(L):
        constw = int(np.frombuffer(b, np.int32, 1, off)[0])
        wconst = float(np.frombuffer(b, np.float32, 1, off + 4)[0])
        nnz, nblocks, _slots = (int(x) for x in np.frombuffer(b, np.int64, 3, off + 8))
        has_bias = int(np.frombuffer(b, np.int32, 1, off + 40)[0])
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
        layers.append(dict(grp=grp, idx=idx, pos=pos, nnz=nnz, constw=constw, wconst=wconst))
    return dict(N=N, Q=Q, nq=nq, G=G, scale=scale, layers=layers)


def slot_order_inputs(f, lay):
    """[N positions, D] input positions of every output position in slot order
    (-1 = padding)."""
    Q, nq, G, scale = f["Q"], f["nq"], f["G"], f["scale"]
    jl = lay["idx"].astype(np.int64) // scale
    grp = lay["grp"]
    cols = []
    for g in range(G):
        seq = []
        for q in range(nq):
            b0, b1 = grp[g * nq + q], grp[g * nq + q + 1]
            blk = jl[b0:b1]                          # [blocks, lane, slot]
            glob = np.where(blk < Q, q * Q + blk, -1)
            seq.append(glob.transpose(1, 0, 2).reshape(32, -1))  # lane, (block, slot)
        cols.append(np.concatenate(seq, axis=1))
    D = max(c.shape[1] for c in cols)
    out = np.full((G * 32, D), -1, np.int64)
    for g, c in enumerate(cols):
        out[g * 32:(g + 1) * 32, : c.shape[1]] = c
    return out


def plain_in_slot_order(f, Y0, bias, clamp=32.0):
    """Final activations (neuron order) of the plain recurrence evaluated in
    the kernel's slot order; layers with one power-of-two weight value only."""
    N = f["N"]
    X = np.ascontiguousarray(Y0, dtype=np.float32)   # layer 0 inputs: the caller's order
    b32, c32 = np.float32(bias), np.float32(clamp)
    for lay in f["layers"]:
        assert lay["constw"], "slot-order evaluation needs one common weight value"
        w = np.float32(lay["wconst"])
        m, e = np.frexp(w)
        assert m == 0.5, "the weight must be a power of two (exact products)"
        order = slot_order_inputs(f, lay)
        acc = np.zeros((X.shape[0], N), np.float32)
        Xz = np.concatenate([X, np.zeros((X.shape[0], 1), np.float32)], axis=1)
        for s in range(order.shape[1]):
            j = np.where(order[:, s] >= 0, order[:, s], N)  # padding reads the zero column
            acc = acc + w * Xz[:, j]
        X = np.minimum(np.maximum(acc + b32, np.float32(0)), c32)  # output positions
        pos = lay["pos"]
    if pos is not None:
        X = X[:, pos]  # position of neuron c -> neuron order
    return X
