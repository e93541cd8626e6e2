"""ctypes binding of the C ABI in include/snicit_gb300.h.

The shared library is built in-tree by snicit_gb300.build.build().  Loading
fails loudly when it is missing: there is no CPU fallback for any call.
"""
import ctypes
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libsnicit_gb300.so")

MODES = {"BF": 0, "SNIG": 1, "XY": 2, "SNICIT": 3}
FLAG_NO_BINARY_FIRST_LAYER = 1
FLAG_NO_PLACEMENT = 2
FLAG_NO_CHAIN = 4
FLAG_NO_MERGE = 8
FLAG_NO_CHAIN_STREAM = 16
FLAG_NO_GRID_CHAIN = 32
FLAG_NO_STREAMED_INPUT = 64
FLAG_HOST_POST_CHOICE = 128
FLAG_DENSE_RESIDUE = 256

STATUS = {
    0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "out of memory", 4: "I/O error",
    5: "malformed input", 6: "call out of order", 7: "device wait timed out",
    8: "unsupported", 9: "busy",
}


class SdnnError(RuntimeError):
    def __init__(self, code, msg=""):
        self.code = code
        super().__init__(f"sdnn status {code} ({STATUS.get(code, '?')}){': ' + msg if msg else ''}")


class Config(ctypes.Structure):
    _fields_ = [
        ("num_neurons", ctypes.c_int32), ("num_layers", ctypes.c_int32),
        ("mode", ctypes.c_int32), ("threshold", ctypes.c_int32), ("batch", ctypes.c_int64),
        ("bias", ctypes.c_float), ("clamp", ctypes.c_float), ("num_centroids", ctypes.c_int32),
        ("autotune", ctypes.c_int32), ("seed", ctypes.c_uint64), ("device", ctypes.c_int32),
        ("tile_rows", ctypes.c_int32), ("threads", ctypes.c_int32),
        ("flags", ctypes.c_int32), ("merge_start", ctypes.c_int32),
        ("merge_every", ctypes.c_int32), ("input_piece_rows", ctypes.c_int32),
        ("input_prefix_layers", ctypes.c_int32),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("stage_ms", ctypes.c_float * 4), ("total_ms", ctypes.c_float),
        ("rows_in", ctypes.c_int64), ("rows_out", ctypes.c_int64),
        ("row_layers", ctypes.c_int64), ("centroids", ctypes.c_int32),
        ("residue_rows", ctypes.c_int32), ("launches", ctypes.c_int32),
        ("threshold", ctypes.c_int32), ("tile_rows", ctypes.c_int32),
        ("threads", ctypes.c_int32), ("input_pieces", ctypes.c_int32),
        ("pre_row_layers", ctypes.c_int64), ("post_row_layers", ctypes.c_int64),
        ("weight_nnz", ctypes.c_int64), ("centroid_candidates", ctypes.c_int32),
        ("merge_start", ctypes.c_int32), ("merge_every", ctypes.c_int32),
        ("post_kernel", ctypes.c_int32), ("device_post_choice", ctypes.c_int32),
        ("sparse_residue_rows", ctypes.c_int32), ("sparse_row_layers", ctypes.c_int64),
    ]


class ServerConfig(ctypes.Structure):
    _fields_ = [
        ("slots", ctypes.c_int32), ("head_outputs", ctypes.c_int32),
        ("max_rows", ctypes.c_int64), ("memory_fraction", ctypes.c_double),
        ("max_pending", ctypes.c_int64), ("max_delay_us", ctypes.c_int64),
        ("max_requests_per_pass", ctypes.c_int32), ("reserved", ctypes.c_int32 * 5),
    ]


class ServerStats(ctypes.Structure):
    _fields_ = [
        ("passes", ctypes.c_int64), ("rows", ctypes.c_int64), ("requests", ctypes.c_int64),
        ("max_rows_in_pass", ctypes.c_int64), ("queued", ctypes.c_int64),
        ("slot_rows", ctypes.c_int64), ("slots", ctypes.c_int32),
        ("reserved", ctypes.c_int32 * 7),
    ]


# (name, restype, argtypes) of every exported entry point
P, I32, I64, U64, F32 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_uint64, ctypes.c_float
SIGNATURES = [
    ("sdnn_config_default", ctypes.c_int, [P]),
    ("sdnn_reference_bias", ctypes.c_float, [I32]),
    ("sdnn_create", ctypes.c_int, [P, P]),
    ("sdnn_destroy", ctypes.c_int, [P]),
    ("sdnn_last_error", ctypes.c_char_p, [P]),
    ("sdnn_status_string", ctypes.c_char_p, [ctypes.c_int]),
    ("sdnn_abi_version", ctypes.c_int, []),
    ("sdnn_abi_sizes", ctypes.c_int, [P, I32]),
    ("sdnn_load_weights_tsv", ctypes.c_int, [P, ctypes.c_char_p]),
    ("sdnn_set_layer_coo", ctypes.c_int, [P, I32, P, P, P, I64]),
    ("sdnn_set_layer_bias", ctypes.c_int, [P, I32, P]),
    ("sdnn_generate_weights", ctypes.c_int, [P, U64, I32, F32]),
    ("sdnn_generate_radixnet_weights", ctypes.c_int, [P, I32, F32]),
    ("sdnn_finalize_weights", ctypes.c_int, [P]),
    ("sdnn_infer_host", ctypes.c_int, [P, P, I64, P, P, P]),
    ("sdnn_infer_device", ctypes.c_int, [P, P, I64, P, P]),
    ("sdnn_infer_host_bits", ctypes.c_int, [P, P, I64, P, P, P]),
    ("sdnn_infer_batches_host", ctypes.c_int, [P, P, P, I32, P]),
    ("sdnn_infer_batches_device", ctypes.c_int, [P, P, P, I32, P, P]),
    ("sdnn_read_inputs_tsv", ctypes.c_int, [ctypes.c_char_p, I32, I64, I64, P]),
    ("sdnn_read_activations", ctypes.c_int, [P, P, I64]),
    ("sdnn_get_stats", ctypes.c_int, [P, P]),
    ("sdnn_get_layer_rows", ctypes.c_int, [P, P, I32]),
    ("sdnn_autotune", ctypes.c_int, [P, P, I64, ctypes.c_char_p]),
    ("sdnn_autotune_device", ctypes.c_int, [P, P, I64, ctypes.c_char_p]),
    ("sdnn_set_mode", ctypes.c_int, [P, I32, I32]),
    ("sdnn_set_input_streaming", ctypes.c_int, [P, I32]),
    ("sdnn_selftest_wait_timeout", ctypes.c_int, [P, I64]),
    ("sdnn_save_packed_weights", ctypes.c_int, [P, ctypes.c_char_p]),
    ("sdnn_load_packed_weights", ctypes.c_int, [P, ctypes.c_char_p]),
    ("sdnn_layer_noalloc", ctypes.c_int, [P, I32, P, P, I64, P, P]),
    ("sdnn_selftest_noalloc_timeout", ctypes.c_int, [P, P, I64, I64, P]),
    ("sdnn_server_config_default", ctypes.c_int, [P]),
    ("sdnn_server_create", ctypes.c_int, [P, P, P, P, P]),
    ("sdnn_server_destroy", ctypes.c_int, [P]),
    ("sdnn_server_capacity", I64, [P]),
    ("sdnn_submit", ctypes.c_int, [P, P, I64, P]),
    ("sdnn_poll", ctypes.c_int, [P, U64, P, P, P, P, P]),
    ("sdnn_wait", ctypes.c_int, [P, U64, P, P, P, P]),
    ("sdnn_server_get_stats", ctypes.c_int, [P, P]),
    ("sdnn_generate_inputs", ctypes.c_int, [I32, U64, I64, I64, P]),
    ("sdnn_generate_inputs_device", ctypes.c_int, [I32, U64, I64, I64, P, P]),
    ("sdnn_generate_layer_coo", ctypes.c_int, [I32, U64, I32, I32, F32, P, P, P]),
    ("sdnn_generate_radixnet_layer_coo", ctypes.c_int, [I32, I32, I32, F32, P, P, P]),
    ("sdnn_write_weights_tsv", ctypes.c_int, [P, ctypes.c_char_p]),
    ("sdnn_write_inputs_tsv", ctypes.c_int, [ctypes.c_char_p, P, I64, I32]),
    ("sdnn_write_categories_tsv", ctypes.c_int, [ctypes.c_char_p, P, I64]),
    ("sdnn_write_inputs_bin", ctypes.c_int, [ctypes.c_char_p, P, I64, I32, I32]),
    ("sdnn_inputs_bin_info", ctypes.c_int, [ctypes.c_char_p, P, P, P]),
    ("sdnn_read_inputs_bin", ctypes.c_int, [ctypes.c_char_p, I32, I64, I64, P]),
]

_lib = None


def load(path: str = LIB_PATH):
    """Loads the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build the CUDA extension first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = ctypes.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(code, engine_ptr=None):
    if code != 0:
        msg = ""
        if engine_ptr:
            msg = (load().sdnn_last_error(engine_ptr) or b"").decode(errors="replace")
        raise SdnnError(code, msg)
