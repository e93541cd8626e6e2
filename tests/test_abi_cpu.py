"""C ABI checks that need no GPU: exports, defaults, argument validation,
host-side weight handling and the reference file formats."""
import ctypes
import os
import re
import tempfile

import numpy as np
import pytest

import snicit_gb300 as sg
from snicit_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", f)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(sdnn_[a-z0-9_]+)\s*\(", txt))
    return names


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(_lib.LIB_PATH)
    declared = header_functions()
    assert len(declared) >= 20
    for name in declared:
        assert hasattr(lib, name), f"{name} declared in include/ but not exported"
    bound = {n for n, _, _ in _lib.SIGNATURES}
    assert declared <= bound | {"sdnn_no_alloc_entry_placeholder"}, declared - bound


def test_defaults_and_reference_bias():
    lib = sg.load()
    cfg = _lib.Config()
    assert lib.sdnn_config_default(ctypes.byref(cfg)) == 0
    assert (cfg.num_neurons, cfg.num_layers, cfg.threshold, cfg.batch) == (1024, 120, 30, 60000)
    assert cfg.mode == _lib.MODES["SNICIT"] and cfg.clamp == 32.0
    # main/SDGC.cu:49-54
    for n, b in ((65536, -0.45), (16384, -0.4), (4096, -0.35), (1024, -0.3), (77, 0.0)):
        assert lib.sdnn_reference_bias(n) == pytest.approx(b)
    assert lib.sdnn_abi_version() == 3


def test_struct_layouts_match_the_c_abi():
    """The ctypes mirrors of the public structs have the C sizes (a field
    added on one side only would shift every later field)."""
    lib = _lib.load()
    sizes = (ctypes.c_int32 * 4)()
    assert lib.sdnn_abi_sizes(sizes, 4) == 0
    want = [ctypes.sizeof(c) for c in (_lib.Config, _lib.Stats, _lib.ServerConfig, _lib.ServerStats)]
    assert list(sizes) == want
    assert lib.sdnn_status_string(7) == b"device wait timed out"


@pytest.mark.parametrize("field,value", [("num_neurons", 100), ("num_neurons", 0),
                                         ("num_layers", 0), ("mode", 9), ("num_centroids", 0),
                                         ("num_centroids", 1000), ("batch", 0), ("clamp", 0.0),
                                         ("tile_rows", 64)])
def test_create_rejects_bad_config(field, value):
    lib = sg.load()
    cfg = _lib.Config()
    lib.sdnn_config_default(ctypes.byref(cfg))
    setattr(cfg, field, value)
    h = ctypes.c_void_p()
    assert lib.sdnn_create(ctypes.byref(cfg), ctypes.byref(h)) == 1
    assert not h


def test_null_arguments_return_status():
    lib = sg.load()
    assert lib.sdnn_create(None, None) == 1
    assert lib.sdnn_destroy(None) == 0
    assert lib.sdnn_infer_host(None, None, 0, None, None, None) == 1
    assert lib.sdnn_get_stats(None, None) == 1
    assert lib.sdnn_generate_inputs(0, 1, 0, 1, None) == 1


def test_engine_without_gpu_handles_weights_on_host():
    """Creation, weight generation and TSV writing need no device."""
    with tempfile.TemporaryDirectory() as d:
        e = sg.Engine(64, 3, mode="SNIG", batch=4)
        e.generate_weights(5, 8, 0.5)
        e.write_weights_tsv(d)
        files = sorted(os.listdir(d))
        assert files == ["n64-l1.tsv", "n64-l2.tsv", "n64-l3.tsv"]
        lines = open(os.path.join(d, "n64-l2.tsv")).read().split("\n")
        lines = [l for l in lines if l]
        assert len(lines) == 64 * 8
        r, c, v = zip(*[l.split("\t") for l in lines])
        assert {float(x) for x in v} == {0.5}
        r = np.array(r, int) - 1
        c = np.array(c, int) - 1
        # same content as the generator's COO for layer 1
        gr, gc, gv = sg.generate_layer_coo(64, 5, 1, 8, 0.5)
        assert set(zip(r, c)) == set(zip(gr, gc))
        # reload and rewrite: identical files
        e2 = sg.Engine(64, 3, mode="SNIG", batch=4)
        e2.load_weights_tsv(d)
        with tempfile.TemporaryDirectory() as d2:
            e2.write_weights_tsv(d2)
            for f in files:
                assert open(os.path.join(d, f)).read() == open(os.path.join(d2, f)).read()
        e.close()
        e2.close()


def test_weight_tsv_duplicates_are_summed_and_errors_reported():
    with tempfile.TemporaryDirectory() as d:
        with open(os.path.join(d, "n32-l1.tsv"), "w") as f:
            f.write("1\t2\t0.25\n1\t2\t0.5\n3\t4\t1\n")
        e = sg.Engine(32, 1, mode="SNIG", batch=2)
        e.load_weights_tsv(d)
        with tempfile.TemporaryDirectory() as d2:
            e.write_weights_tsv(d2)
            txt = open(os.path.join(d2, "n32-l1.tsv")).read()
        assert txt == "1\t2\t0.75\n3\t4\t1\n"
        with open(os.path.join(d, "n32-l1.tsv"), "w") as f:
            f.write("1\t99\t0.25\n")
        with pytest.raises(sg.SdnnError) as ei:
            e.load_weights_tsv(d)
        assert ei.value.code == 5
        with open(os.path.join(d, "n32-l1.tsv"), "w") as f:
            f.write("1\tx\t0.25\n")
        with pytest.raises(sg.SdnnError) as ei:
            e.load_weights_tsv(d)
        assert ei.value.code == 5
        with pytest.raises(sg.SdnnError) as ei:
            e.load_weights_tsv(os.path.join(d, "missing"))
        assert ei.value.code == 4
        e.close()


def test_input_and_category_formats():
    Y0 = sg.generate_inputs(128, 3, 0, 20)
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "sparse-images-128.tsv")
        sg.write_inputs_tsv(p, Y0)
        first = open(p).readline().split("\t")
        assert int(first[0]) == 1 and float(first[2]) == 1.0
        assert np.array_equal(sg.read_inputs_tsv(p, 128, 0, 20), Y0)
        # offset window like read_input_xy (src/SDGC/utility.hpp:268-293)
        assert np.array_equal(sg.read_inputs_tsv(p, 128, 5, 10), Y0[5:15])
        q = os.path.join(d, "cat.tsv")
        sg.write_categories_tsv(q, np.array([0, 4, 9], np.int32))
        assert open(q).read() == "1\n5\n10\n"


def test_infer_needs_device_and_reports_cuda_error():
    pytest.importorskip("torch")
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    e = sg.Engine(64, 2, mode="SNIG", batch=4)
    e.generate_weights(1)
    with pytest.raises(sg.SdnnError) as ei:
        e.infer(np.zeros((4, 64), np.float32))
    assert ei.value.code == 2
    e.close()
