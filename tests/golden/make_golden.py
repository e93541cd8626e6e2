"""Generates the golden fixtures of tests/golden/ from the reference's own kernels.

Runs on a machine with a GPU and with oracle/_ref/ built by
oracle/ref_build.sh (the reference's bf_inference / snig_inference /
identify compiled from its sources).  For each case it draws seeded inputs
and weights with numpy, runs oracle/ref_harness.cpp, and stores inputs,
weights and the reference kernels' final activations and categories as
<case>.npz.  The CPU tests then check the oracle against these files.

    python tests/golden/make_golden.py [OUT_DIR]      (default: tests/golden/)
"""
import os
import struct
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
REF = os.path.join(ROOT, "oracle", "_ref")

# name: (N, L, B, sec_size, bias, nnz_per_row, weight kind, input kind, seed)
CASES = {
    "sdgc_n128_l12": (128, 12, 192, 128, -0.3, 32, "const", "binary", 11),
    "sdgc_n64_l30_slab2": (64, 30, 256, 32, -0.3, 16, "const", "binary", 12),
    "beyond_n256_l6": (256, 6, 128, 256, -0.05, 8, "normal", "uniform", 13),
    "sdgc_n256_l9_odd": (256, 9, 96, 128, -0.35, 32, "const", "binary", 14),
}


def make_case(N, L, B, nnz, wkind, ikind, seed):
    rng = np.random.default_rng(seed)
    layers = []
    for _ in range(L):
        cols = np.stack([rng.choice(N, nnz, replace=False) for _ in range(N)]).astype(np.int32)
        cols.sort(axis=1)
        if wkind == "const":
            vals = np.full(cols.shape, 0.0625, np.float32)
        else:
            vals = (rng.standard_normal(cols.shape) * 0.3).astype(np.float32)
        row_off = (np.arange(N + 1) * nnz).astype(np.int32)
        layers.append((row_off, cols.ravel(), vals.ravel()))
    if ikind == "binary":
        rho = 0.95 * np.sort(rng.random((B, 9)), axis=1)[:, 1]
        Y0 = (rng.random((B, N)) < rho[:, None]).astype(np.float32)
    else:
        Y0 = rng.random((B, N)).astype(np.float32)
    return layers, Y0


def main(out_dir):
    os.makedirs(out_dir, exist_ok=True)
    harness = os.path.join(REF, "ref_harness")
    subprocess.run(["nvcc", "-O2", "-std=c++17", os.path.join(ROOT, "oracle", "ref_harness.cpp"),
                    "-o", harness, "-lcuda"], check=True)
    module = os.path.join(REF, "sdgc_ref.cubin")
    for name, (N, L, B, sec, bias, nnz, wkind, ikind, seed) in CASES.items():
        layers, Y0 = make_case(N, L, B, nnz, wkind, ikind, seed)
        inp = os.path.join(out_dir, name + ".in.bin")
        outp = os.path.join(out_dir, name + ".out.bin")
        with open(inp, "wb") as f:
            f.write(struct.pack("<iiiif", N, L, B, sec, bias))
            for ro, c, v in layers:
                f.write(struct.pack("<i", len(c)))
                f.write(ro.astype("<i4").tobytes())
                f.write(c.astype("<i4").tobytes())
                f.write(v.astype("<f4").tobytes())
            f.write(Y0.astype("<f4").tobytes())
        r = subprocess.run([harness, module, inp, outp], capture_output=True, text=True)
        print(name, r.stdout.strip(), r.stderr.strip())
        r.check_returncode()
        raw = np.fromfile(outp, dtype=np.uint8)
        o = 0
        def take(dtype, n):
            nonlocal o
            a = raw[o:o + n * 4].view(dtype).copy()
            o += n * 4
            return a
        ybf = take("<f4", B * N).reshape(B, N)
        ysn = take("<f4", B * N).reshape(B, N)
        id_bf = take("<i4", B)
        id_sn = take("<i4", B)
        alive_bf = take("<i4", L)
        np.savez_compressed(
            os.path.join(out_dir, name + ".npz"),
            N=N, L=L, B=B, sec_size=sec, bias=np.float32(bias), nnz_per_row=nnz,
            row_off=np.stack([ro for ro, _, _ in layers]),
            cols=np.stack([c for _, c, _ in layers]).astype(np.int16 if N <= 32767 else np.int32),
            vals=np.stack([v for _, _, v in layers]),
            Y0=Y0, Y_bf=ybf, Y_snig=ysn, identify_bf=id_bf, identify_snig=id_sn,
            alive_bf=alive_bf)
        os.remove(inp)
        os.remove(outp)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.dirname(os.path.abspath(__file__)))
