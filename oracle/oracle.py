"""ctypes wrapper of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, as the checker or as the timed CPU baseline.  The product never does.

Layers are given as a list of CSR triples (row_off[N+1], cols, vals) by input
row, duplicates already summed (src/SDGC/utility.hpp:85-126 semantics).
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.LIB
        if not os.path.exists(path):
            path = _build.build()
        L = ctypes.CDLL(path)
        P = ctypes.c_void_p
        L.oracle_infer.argtypes = [ctypes.c_int, ctypes.c_int, P, P, P, P, P, ctypes.c_float,
                                   ctypes.c_float, P, ctypes.c_int64, ctypes.c_int, ctypes.c_int,
                                   P, P, P, P]
        L.oracle_infer.restype = ctypes.c_int
        L.oracle_identify.argtypes = [P, ctypes.c_int64, ctypes.c_int, ctypes.c_int, P]
        L.oracle_identify.restype = ctypes.c_int
        L.oracle_snicit.argtypes = [ctypes.c_int, ctypes.c_int, P, P, P, P, P, ctypes.c_float,
                                    ctypes.c_float, P, ctypes.c_int64, ctypes.c_int, P,
                                    ctypes.c_int, P, P, P, P]
        L.oracle_snicit.restype = ctypes.c_int
        L.oracle_ref_candidates.argtypes = [P, ctypes.c_int64, ctypes.c_int, ctypes.c_int, P]
        L.oracle_ref_candidates.restype = ctypes.c_int
        L.oracle_gen_inputs.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.c_int64,
                                        ctypes.c_int64, P]
        L.oracle_gen_inputs.restype = ctypes.c_int
        L.oracle_gen_layer_csr.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.c_int,
                                           ctypes.c_int, ctypes.c_float, P, P, P]
        L.oracle_gen_layer_csr.restype = ctypes.c_int
        L.oracle_gen_radixnet_csr.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                              ctypes.c_float, P, P, P]
        L.oracle_gen_radixnet_csr.restype = ctypes.c_int
        L.oracle_port_stream.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_uint64, ctypes.c_int,
                                         ctypes.c_float, ctypes.c_float, ctypes.c_float, P,
                                         ctypes.c_int64, P, ctypes.c_int, ctypes.c_int, P, P]
        L.oracle_port_stream.restype = ctypes.c_int
        L.oracle_infer_stream64.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_uint64,
                                            ctypes.c_int, ctypes.c_float, ctypes.c_float,
                                            ctypes.c_float, P, ctypes.c_int64, ctypes.c_int, P, P]
        L.oracle_infer_stream64.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def pack_layers(layers, N):
    """Concatenates CSR layers into the oracle's flat arrays."""
    L = len(layers)
    row_off = np.zeros((L, N + 1), dtype=np.int32)
    nnz_off = np.zeros(L + 1, dtype=np.int64)
    for l, (ro, c, v) in enumerate(layers):
        row_off[l] = ro
        nnz_off[l + 1] = nnz_off[l] + len(c)
    cols = np.ascontiguousarray(np.concatenate([c for _, c, _ in layers]).astype(np.int32)) if L else np.zeros(0, np.int32)
    vals = np.ascontiguousarray(np.concatenate([v for _, _, v in layers]).astype(np.float32)) if L else np.zeros(0, np.float32)
    return np.ascontiguousarray(row_off), cols, vals, nnz_off


def _bias_arr(bias_vec, L, N):
    if bias_vec is None:
        return None
    return np.ascontiguousarray(np.asarray(bias_vec, dtype=np.float32).reshape(L, N))


def infer(layers, N, bias, Y0, clamp=32.0, precision=64, nthreads=None, bias_vec=None,
          want_y=True):
    """Plain recurrence (bf_inference semantics).

    Returns (Y, alive, dead_at): Y float64 (precision 64) or float32
    (precision 32) final activations, alive int32 per row, dead_at int32 (first
    empty layer, L if none).
    """
    Y0 = np.ascontiguousarray(Y0, dtype=np.float32)
    rows = Y0.shape[0]
    L = len(layers)
    ro, cols, vals, off = pack_layers(layers, N)
    bv = _bias_arr(bias_vec, L, N)
    if nthreads is None:
        nthreads = os.cpu_count() or 1
    alive = np.zeros(rows, dtype=np.int32)
    dead = np.zeros(rows, dtype=np.int32)
    y64 = np.zeros((rows, N), dtype=np.float64) if (want_y and precision == 64) else None
    y32 = np.zeros((rows, N), dtype=np.float32) if (want_y and precision == 32) else None
    rc = lib().oracle_infer(N, L, _p(ro), _p(cols), _p(vals), _p(off), _p(bv), float(bias),
                            float(clamp), _p(Y0), rows, precision, int(nthreads), _p(y64),
                            _p(y32), _p(alive), _p(dead))
    if rc:
        raise RuntimeError(f"oracle_infer failed ({rc})")
    return (y64 if precision == 64 else y32), alive, dead


def identify(Y, mode=0):
    """mode 0: any activation > 0; mode 1: the reference identify's int-sum rule."""
    Y = np.ascontiguousarray(Y, dtype=np.float64)
    out = np.zeros(Y.shape[0], dtype=np.int32)
    lib().oracle_identify(_p(Y), Y.shape[0], Y.shape[1], int(mode), _p(out))
    return out


def snicit(layers, N, bias, Y0, threshold, centroids, clamp=32.0, bias_vec=None):
    """FP64 SNICIT residue form; returns (Y, flags, assign, nonempty)."""
    Y0 = np.ascontiguousarray(Y0, dtype=np.float32)
    rows = Y0.shape[0]
    L = len(layers)
    ro, cols, vals, off = pack_layers(layers, N)
    bv = _bias_arr(bias_vec, L, N)
    cents = np.ascontiguousarray(np.asarray(centroids, dtype=np.int32))
    Y = np.zeros((rows, N), dtype=np.float64)
    flags = np.zeros(rows, dtype=np.int32)
    assign = np.zeros(rows, dtype=np.int32)
    nonempty = np.zeros(1, dtype=np.int64)
    rc = lib().oracle_snicit(N, L, _p(ro), _p(cols), _p(vals), _p(off), _p(bv), float(bias),
                             float(clamp), _p(Y0), rows, int(threshold), _p(cents), len(cents),
                             _p(Y), _p(flags), _p(assign), _p(nonempty))
    if rc:
        raise RuntimeError(f"oracle_snicit failed ({rc})")
    return Y, flags, assign, int(nonempty[0])


def ref_candidates(Ylive, sample=32):
    """Reference centroid pick on a live-rows-only matrix; returns kept indices."""
    Ylive = np.ascontiguousarray(Ylive, dtype=np.float32)
    out = np.zeros(32, dtype=np.int32)
    n = lib().oracle_ref_candidates(_p(Ylive), Ylive.shape[0], Ylive.shape[1], int(sample),
                                    _p(out))
    return out[:n].copy()


def head(Y, head_w, head_b):
    """Dense output head in FP64: logits = Y . W + b, no activation
    (dense_output, src/beyond/general.hpp:74-102); argmax = first maximum."""
    logits = np.asarray(Y, np.float64) @ np.asarray(head_w, np.float64) + np.asarray(head_b, np.float64)
    return logits, np.argmax(logits, axis=1).astype(np.int32)


def gen_inputs(N, seed, row_offset, rows):
    """Seeded 0/1 input rows of the synthetic SDGC workload (restated generator)."""
    out = np.zeros((rows, N), dtype=np.float32)
    if lib().oracle_gen_inputs(int(N), int(seed), int(row_offset), int(rows), _p(out)):
        raise RuntimeError("oracle_gen_inputs failed")
    return out


def gen_layer_csr(N, seed, layer, nnz=32, value=0.0625):
    """One synthetic layer as CSR by input row (restated generator)."""
    ro = np.zeros(N + 1, dtype=np.int32)
    cols = np.zeros(N * nnz, dtype=np.int32)
    vals = np.zeros(N * nnz, dtype=np.float32)
    if lib().oracle_gen_layer_csr(int(N), int(seed), int(layer), int(nnz), float(value), _p(ro),
                                  _p(cols), _p(vals)):
        raise RuntimeError("oracle_gen_layer_csr failed")
    return ro, cols, vals


def gen_radixnet_csr(N, layer, block=16, value=0.0625):
    """One RadiX-Net layer (radix 2, dense blocks of `block`) as CSR by input
    row, stated output by output (restated generator)."""
    ro = np.zeros(N + 1, dtype=np.int32)
    cols = np.zeros(N * 2 * block, dtype=np.int32)
    vals = np.zeros(N * 2 * block, dtype=np.float32)
    if lib().oracle_gen_radixnet_csr(int(N), int(block), int(layer), float(value), _p(ro),
                                     _p(cols), _p(vals)):
        raise RuntimeError("oracle_gen_radixnet_csr failed")
    return ro, cols, vals


def port_stream(N, L, seed, bias, Y0, group_sizes, nnz=32, value=0.0625, clamp=32.0,
                nthreads=None):
    """FP32 port of bf_inference on the synthetic net, weights generated layer
    by layer; rows split into consecutive groups of the given sizes.  Returns
    (alive, seconds per group of layer arithmetic, final activations)."""
    Y = np.ascontiguousarray(Y0, dtype=np.float32).copy()
    sizes = np.asarray(group_sizes, dtype=np.int64)
    off = np.ascontiguousarray(np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64))
    assert off[-1] == Y.shape[0]
    alive = np.zeros(Y.shape[0], dtype=np.int32)
    secs = np.zeros(len(sizes), dtype=np.float64)
    if nthreads is None:
        nthreads = os.cpu_count() or 1
    rc = lib().oracle_port_stream(int(N), int(L), int(seed), int(nnz), float(value), float(bias),
                                  float(clamp), _p(Y), Y.shape[0], _p(off), len(sizes),
                                  int(nthreads), _p(alive), _p(secs))
    if rc:
        raise RuntimeError(f"oracle_port_stream failed ({rc})")
    return alive, secs, Y


def infer_stream64(N, L, seed, bias, Y0, nnz=32, value=0.0625, clamp=32.0, nthreads=None):
    """FP64 oracle of the synthetic net (weights generated layer by layer);
    returns (Y float64, alive)."""
    Y0 = np.ascontiguousarray(Y0, dtype=np.float32)
    Y = np.zeros(Y0.shape, dtype=np.float64)
    alive = np.zeros(Y0.shape[0], dtype=np.int32)
    if nthreads is None:
        nthreads = os.cpu_count() or 1
    rc = lib().oracle_infer_stream64(int(N), int(L), int(seed), int(nnz), float(value),
                                     float(bias), float(clamp), _p(Y0), Y0.shape[0],
                                     int(nthreads), _p(Y), _p(alive))
    if rc:
        raise RuntimeError(f"oracle_infer_stream64 failed ({rc})")
    return Y, alive
