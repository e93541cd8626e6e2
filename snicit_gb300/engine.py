"""Python face of the engine (thin wrapper over the C ABI)."""
import ctypes

import numpy as np

from . import _lib
from ._lib import Config, Stats, check, load


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


class Engine:
    """One inference engine (one CUDA stream, resident weights).

    Mirrors the reference classes SNICIT_SDGC::{BF,SNIG,XY,SNICIT}: construct
    with (num_neurons, num_layers, mode, threshold, batch), load or generate
    weights, then call infer().
    """

    def __init__(self, num_neurons=1024, num_layers=120, mode="SNICIT", threshold=30,
                 batch=60000, bias=None, clamp=32.0, num_centroids=32, seed=20260101,
                 device=0, tile_rows=0, threads=0, binary_first_layer=True, placement=True,
                 chain=True, merge=True, merge_start=0, merge_every=0, chain_stream=True,
                 grid_chain=True, streamed_input=True, input_piece_rows=0,
                 device_post_choice=True, input_prefix_layers=0, sparse_residue=True):
        lib = load()
        cfg = Config()
        check(lib.sdnn_config_default(ctypes.byref(cfg)))
        cfg.num_neurons = int(num_neurons)
        cfg.num_layers = int(num_layers)
        cfg.mode = _lib.MODES[mode] if isinstance(mode, str) else int(mode)
        cfg.threshold = int(threshold)
        cfg.batch = int(batch)
        cfg.bias = float(lib.sdnn_reference_bias(int(num_neurons)) if bias is None else bias)
        cfg.clamp = float(clamp)
        cfg.num_centroids = int(num_centroids)
        cfg.seed = int(seed)
        cfg.device = int(device)
        cfg.tile_rows = int(tile_rows)
        cfg.threads = int(threads)
        cfg.flags = ((0 if binary_first_layer else _lib.FLAG_NO_BINARY_FIRST_LAYER)
                     | (0 if placement else _lib.FLAG_NO_PLACEMENT)
                     | (0 if chain else _lib.FLAG_NO_CHAIN)
                | (0 if merge else _lib.FLAG_NO_MERGE)
                | (0 if chain_stream else _lib.FLAG_NO_CHAIN_STREAM)
                | (0 if grid_chain else _lib.FLAG_NO_GRID_CHAIN)
                | (0 if streamed_input else _lib.FLAG_NO_STREAMED_INPUT)
                | (0 if device_post_choice else _lib.FLAG_HOST_POST_CHOICE)
                | (0 if sparse_residue else _lib.FLAG_DENSE_RESIDUE))
        cfg.merge_start = int(merge_start)
        cfg.merge_every = int(merge_every)
        cfg.input_piece_rows = int(input_piece_rows)
        cfg.input_prefix_layers = int(input_prefix_layers)
        self.cfg = cfg
        self.N = cfg.num_neurons
        self.L = cfg.num_layers
        self._h = ctypes.c_void_p()
        check(lib.sdnn_create(ctypes.byref(cfg), ctypes.byref(self._h)))

    # ---- lifecycle
    def close(self):
        if self._h:
            load().sdnn_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _ck(self, code):
        check(code, self._h)

    # ---- weights
    def load_weights_tsv(self, directory):
        self._ck(load().sdnn_load_weights_tsv(self._h, str(directory).encode()))

    def set_layer_coo(self, layer, rows, cols, vals):
        rows = np.ascontiguousarray(rows, dtype=np.int32)
        cols = np.ascontiguousarray(cols, dtype=np.int32)
        vals = np.ascontiguousarray(vals, dtype=np.float32)
        self._ck(load().sdnn_set_layer_coo(self._h, int(layer), _ptr(rows), _ptr(cols),
                                           _ptr(vals), len(vals)))

    def set_layer_csr(self, layer, row_off, cols, vals):
        row_off = np.asarray(row_off)
        rows = np.repeat(np.arange(len(row_off) - 1, dtype=np.int32), np.diff(row_off))
        self.set_layer_coo(layer, rows, cols, vals)

    def set_layer_bias(self, layer, bias):
        b = np.ascontiguousarray(bias, dtype=np.float32)
        assert b.shape == (self.N,)
        self._ck(load().sdnn_set_layer_bias(self._h, int(layer), _ptr(b)))

    def generate_weights(self, seed, nnz_per_row=32, value=0.0625):
        self._ck(load().sdnn_generate_weights(self._h, int(seed), int(nnz_per_row), float(value)))

    def generate_radixnet(self, block=16, value=0.0625):
        """RadiX-Net-structured layers (radix 2, dense blocks of `block`
        neurons); see sdnn_generate_radixnet_weights."""
        self._ck(load().sdnn_generate_radixnet_weights(self._h, int(block), float(value)))

    def finalize(self):
        self._ck(load().sdnn_finalize_weights(self._h))

    def write_weights_tsv(self, directory):
        self._ck(load().sdnn_write_weights_tsv(self._h, str(directory).encode()))

    # ---- inference
    def infer(self, Y0, want_flags=True, want_ids=True):
        """Host inference; returns (flags or None, sorted survivor ids or None)."""
        Y0 = np.ascontiguousarray(Y0, dtype=np.float32)
        assert Y0.ndim == 2 and Y0.shape[1] == self.N
        rows = Y0.shape[0]
        flags = np.zeros(rows, dtype=np.int32) if want_flags else None
        ids = np.zeros(rows, dtype=np.int32) if want_ids else None
        count = ctypes.c_int64(0)
        self._ck(load().sdnn_infer_host(self._h, _ptr(Y0), rows, _ptr(flags), _ptr(ids),
                                        ctypes.byref(count)))
        return flags, (ids[: count.value].copy() if ids is not None else None)

    def infer_bits(self, bits, want_flags=True, want_ids=True):
        """Host inference on one-bit rows (uint64 array rows x ceil(N / 64),
        see pack_bits); returns (flags or None, sorted survivor ids or None)."""
        bits = np.ascontiguousarray(bits, dtype=np.uint64)
        assert bits.ndim == 2 and bits.shape[1] == (self.N + 63) // 64
        rows = bits.shape[0]
        flags = np.zeros(rows, dtype=np.int32) if want_flags else None
        ids = np.zeros(rows, dtype=np.int32) if want_ids else None
        count = ctypes.c_int64(0)
        self._ck(load().sdnn_infer_host_bits(self._h, _ptr(bits), rows, _ptr(flags), _ptr(ids),
                                             ctypes.byref(count)))
        return flags, (ids[: count.value].copy() if ids is not None else None)

    def infer_device(self, y0_ptr, rows, flags_ptr, stream_ptr=None):
        """Device inference on raw device pointers (e.g. torch tensor data_ptr())."""
        self._ck(load().sdnn_infer_device(self._h, ctypes.c_void_p(int(y0_ptr)), int(rows),
                                          ctypes.c_void_p(int(flags_ptr)),
                                          ctypes.c_void_p(int(stream_ptr)) if stream_ptr else None))

    def infer_batches(self, batches):
        """Host batches (list of rows x N arrays) in one launch schedule; returns flags per batch."""
        arrs = [np.ascontiguousarray(b, dtype=np.float32) for b in batches]
        nb = len(arrs)
        ptrs = (ctypes.c_void_p * nb)(*[a.ctypes.data for a in arrs])
        rows = (ctypes.c_int64 * nb)(*[a.shape[0] for a in arrs])
        outs = [np.zeros(a.shape[0], dtype=np.int32) for a in arrs]
        fptrs = (ctypes.c_void_p * nb)(*[o.ctypes.data for o in outs])
        self._ck(load().sdnn_infer_batches_host(self._h, ptrs, rows, nb, fptrs))
        return outs

    def infer_batches_device(self, in_ptrs, rows, flag_ptrs, stream_ptr=None):
        nb = len(in_ptrs)
        p = (ctypes.c_void_p * nb)(*[int(x) for x in in_ptrs])
        r = (ctypes.c_int64 * nb)(*[int(x) for x in rows])
        f = (ctypes.c_void_p * nb)(*[int(x) for x in flag_ptrs])
        self._ck(load().sdnn_infer_batches_device(
            self._h, p, r, nb, f, ctypes.c_void_p(int(stream_ptr)) if stream_ptr else None))

    def activations(self, rows):
        out = np.zeros((rows, self.N), dtype=np.float32)
        self._ck(load().sdnn_read_activations(self._h, _ptr(out), int(rows)))
        return out

    def stats(self):
        s = Stats()
        self._ck(load().sdnn_get_stats(self._h, ctypes.byref(s)))
        return {
            "stage_ms": list(s.stage_ms), "total_ms": s.total_ms, "rows_in": s.rows_in,
            "rows_out": s.rows_out, "row_layers": s.row_layers, "centroids": s.centroids,
            "residue_rows": s.residue_rows, "launches": s.launches, "threshold": s.threshold,
            "tile_rows": s.tile_rows, "threads": s.threads,
            "pre_row_layers": s.pre_row_layers, "post_row_layers": s.post_row_layers,
            "weight_nnz": s.weight_nnz, "centroid_candidates": s.centroid_candidates,
            "merge_start": s.merge_start, "merge_every": s.merge_every,
            "post_kernel": s.post_kernel, "input_pieces": s.input_pieces,
            "device_post_choice": s.device_post_choice,
            "sparse_residue_rows": s.sparse_residue_rows,
            "sparse_row_layers": s.sparse_row_layers,
        }

    def layer_rows(self):
        out = np.zeros(self.L, dtype=np.int64)
        self._ck(load().sdnn_get_layer_rows(self._h, _ptr(out), self.L))
        return out

    def save_packed(self, path):
        """Writes the packed weights (host packing; no GPU needed)."""
        self._ck(load().sdnn_save_packed_weights(self._h, str(path).encode()))

    def load_packed(self, path):
        """Takes the weights from a packed-weight file (mmap)."""
        self._ck(load().sdnn_load_packed_weights(self._h, str(path).encode()))

    def set_mode(self, mode, threshold=None):
        """Switches mode (and threshold) keeping the packed weights."""
        m = _lib.MODES[mode] if isinstance(mode, str) else int(mode)
        t = self.cfg.threshold if threshold is None else int(threshold)
        self._ck(load().sdnn_set_mode(self._h, m, t))
        self.cfg.mode = m
        self.cfg.threshold = t

    def set_input_streaming(self, piece_rows):
        """Host FP32 inputs: copy in pieces of piece_rows rows overlapped with
        the first layers (0 = automatic size), or one whole copy (< 0)."""
        self._ck(load().sdnn_set_input_streaming(self._h, int(piece_rows)))

    def autotune_device(self, d_ptr, rows, record_path=None):
        """Autotuner on device-resident sample rows (applies the fastest setting)."""
        self._ck(load().sdnn_autotune_device(self._h, ctypes.c_void_p(int(d_ptr)), int(rows),
                                             str(record_path).encode() if record_path else None))

    def autotune(self, Y0, record_path=None):
        Y0 = np.ascontiguousarray(Y0, dtype=np.float32)
        self._ck(load().sdnn_autotune(self._h, _ptr(Y0), Y0.shape[0],
                                      str(record_path).encode() if record_path else None))
        return self.stats()


# ---- synthetic data and file formats (host-only; no GPU needed)

def generate_inputs(num_neurons, seed, row_offset, rows):
    out = np.zeros((rows, num_neurons), dtype=np.float32)
    check(load().sdnn_generate_inputs(int(num_neurons), int(seed), int(row_offset), int(rows),
                                      _ptr(out)))
    return out


def generate_inputs_device(num_neurons, seed, row_offset, rows, d_ptr, stream_ptr=None):
    """Same rows as generate_inputs, written on the current device at d_ptr."""
    check(load().sdnn_generate_inputs_device(int(num_neurons), int(seed), int(row_offset), int(rows),
                                             ctypes.c_void_p(int(d_ptr)),
                                             ctypes.c_void_p(int(stream_ptr)) if stream_ptr else None))


def generate_layer_coo(num_neurons, seed, layer, nnz_per_row=32, value=0.0625):
    n = num_neurons * nnz_per_row
    r = np.zeros(n, dtype=np.int32)
    c = np.zeros(n, dtype=np.int32)
    v = np.zeros(n, dtype=np.float32)
    check(load().sdnn_generate_layer_coo(int(num_neurons), int(seed), int(layer), int(nnz_per_row),
                                         float(value), _ptr(r), _ptr(c), _ptr(v)))
    return r, c, v


def generate_radixnet_layer_coo(num_neurons, layer, block=16, value=0.0625):
    n = num_neurons * 2 * block
    r = np.zeros(n, dtype=np.int32)
    c = np.zeros(n, dtype=np.int32)
    v = np.zeros(n, dtype=np.float32)
    check(load().sdnn_generate_radixnet_layer_coo(int(num_neurons), int(block), int(layer),
                                                  float(value), _ptr(r), _ptr(c), _ptr(v)))
    return r, c, v


def coo_to_csr(N, rows, cols, vals):
    """CSR by input row with duplicates summed in input order (Eigen semantics)."""
    rows = np.asarray(rows, dtype=np.int64)
    cols = np.asarray(cols, dtype=np.int64)
    vals = np.asarray(vals, dtype=np.float32)
    order = np.lexsort((cols, rows))
    r, c, v = rows[order], cols[order], vals[order]
    key = r * N + c
    uniq, start = np.unique(key, return_index=True)
    summed = np.add.reduceat(v, start) if len(v) else v
    ur = (uniq // N).astype(np.int64)
    row_off = np.zeros(N + 1, dtype=np.int32)
    np.add.at(row_off, ur + 1, 1)
    row_off = np.cumsum(row_off).astype(np.int32)
    return row_off, (uniq % N).astype(np.int32), summed.astype(np.float32)


def generate_layer_csr(num_neurons, seed, layer, nnz_per_row=32, value=0.0625):
    r, c, v = generate_layer_coo(num_neurons, seed, layer, nnz_per_row, value)
    return coo_to_csr(num_neurons, r, c, v)


def read_inputs_tsv(path, num_neurons, row_offset, rows):
    out = np.zeros((rows, num_neurons), dtype=np.float32)
    check(load().sdnn_read_inputs_tsv(str(path).encode(), int(num_neurons), int(row_offset),
                                      int(rows), _ptr(out)))
    return out


def write_inputs_tsv(path, Y0):
    Y0 = np.ascontiguousarray(Y0, dtype=np.float32)
    check(load().sdnn_write_inputs_tsv(str(path).encode(), _ptr(Y0), Y0.shape[0], Y0.shape[1]))


def write_categories_tsv(path, ids):
    ids = np.ascontiguousarray(ids, dtype=np.int32)
    check(load().sdnn_write_categories_tsv(str(path).encode(), _ptr(ids), len(ids)))


def write_inputs_bin(path, Y0, bits=False):
    """Binary input file: FP32 rows, or one bit per entry (0/1 inputs)."""
    Y0 = np.ascontiguousarray(Y0, dtype=np.float32)
    check(load().sdnn_write_inputs_bin(str(path).encode(), _ptr(Y0), Y0.shape[0], Y0.shape[1],
                                       1 if bits else 0))


def inputs_bin_info(path):
    n, r, enc = ctypes.c_int32(0), ctypes.c_int64(0), ctypes.c_int32(0)
    check(load().sdnn_inputs_bin_info(str(path).encode(), ctypes.byref(n), ctypes.byref(r),
                                      ctypes.byref(enc)))
    return n.value, r.value, enc.value


def read_inputs_bin(path, num_neurons, row_offset=0, rows=None):
    if rows is None:
        rows = inputs_bin_info(path)[1] - row_offset
    out = np.zeros((rows, num_neurons), dtype=np.float32)
    check(load().sdnn_read_inputs_bin(str(path).encode(), int(num_neurons), int(row_offset),
                                      int(rows), _ptr(out)))
    return out


def pack_bits(Y0):
    """0/1 rows to the one-bit layout (uint64 words, entry j in bit j % 64 of word j / 64)."""
    Y0 = np.asarray(Y0)
    rows, N = Y0.shape
    W = (N + 63) // 64
    padded = np.zeros((rows, W * 64), dtype=np.uint8)
    padded[:, :N] = Y0 != 0
    return np.packbits(padded.reshape(rows, W, 64)[:, :, ::-1], axis=2).reshape(rows, W, 8)[:, :, ::-1] \
        .copy().view(np.uint64).reshape(rows, W)
