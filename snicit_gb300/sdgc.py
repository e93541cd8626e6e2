"""The reference's engine classes, same constructor and infer() signatures.

SNICIT_SDGC::BF / SNIG / XY / SNICIT (src/SDGC/{BF,SNIG,XY,SNICIT}/*.hpp):
    ctor(weight_path, bias, num_neurons, num_layers[, threshold])
    infer(input_path, golden_path, num_inputs[, batch])
Each prints the reference's machine-parsed line ("<MODE> info: runtime X ms
[avgpost Y ms]") and the golden verdict, and returns the sorted 0-based
survivor ids.  All work runs in the CUDA library.
"""
import os

import numpy as np

from .engine import Engine, read_inputs_tsv


def _read_golden(path, num_inputs):
    g = np.zeros(num_inputs, dtype=np.int32)
    with open(path) as f:
        for line in f:
            line = line.strip()
            if line:
                g[int(line) - 1] = 1
    return g


class _Base:
    MODE = "SNICIT"

    def __init__(self, weight_path, bias=-0.3, num_neurons=1024, num_layers=120, threshold=30,
                 **engine_kw):
        self.weight_path = weight_path
        self.N = int(num_neurons)
        self.L = int(num_layers)
        self.bias = float(bias)
        self.threshold = int(threshold)
        self.engine_kw = engine_kw

    def infer(self, input_path, golden_path, num_inputs=60000, batch=None, verbose=True):
        batch = int(batch or num_inputs)
        eng = Engine(self.N, self.L, mode=self.MODE, threshold=self.threshold, batch=batch,
                     bias=self.bias, **self.engine_kw)
        try:
            eng.load_weights_tsv(self.weight_path)
            Y0 = read_inputs_tsv(input_path, self.N, 0, num_inputs)
            flags, ids = eng.infer(Y0)
            st = eng.stats()
        finally:
            eng.close()
        self.stats = st
        total = st["total_ms"]
        if verbose:
            if self.MODE == "SNICIT":
                print(f"pre-conv Time [SNICIT] = {st['stage_ms'][0]}ms")
                print(f"cluster-based conversion Time [overhead] = {st['stage_ms'][1]}ms")
                print(f"post-conv Time [SNICIT] = {st['stage_ms'][2]}ms")
                print(f"recover Time [SNICIT] = {st['stage_ms'][3]}ms")
            post_layers = max(1, self.L - min(self.threshold, self.L))
            if self.MODE in ("SNICIT", "XY"):
                print(f"{self.MODE} info: runtime {total}ms avgpost {st['stage_ms'][2] / post_layers}ms")
            else:
                print(f"{self.MODE} info: runtime {total} ms")
        if golden_path and os.path.exists(golden_path):
            golden = _read_golden(golden_path, num_inputs)
            diff = int(np.sum(golden != flags))
            if verbose:
                print(f"\nNumber of different categories: {diff}")
                print("CHALLENGE PASSED" if diff == 0 else "CHALLENGE FAILED")
        return ids


class BF(_Base):
    MODE = "BF"


class SNIG(_Base):
    MODE = "SNIG"


class XY(_Base):
    MODE = "XY"


class SNICIT(_Base):
    MODE = "SNICIT"
