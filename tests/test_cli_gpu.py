"""The SDGC command-line driver keeps the reference's flags, paths and output
grammar (main/SDGC.cu; the lines bin/*.sh grep for)."""
import os
import re
import subprocess
import tempfile

import pytest

from snicit_gb300 import build

pytestmark = pytest.mark.gpu


def sdgc(args, cwd):
    r = subprocess.run([build.CLI_BIN, *args], cwd=cwd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def test_modes_and_golden_check():
    with tempfile.TemporaryDirectory() as d:
        data = os.path.join(d, "dataset", "SDGC")
        run = os.path.join(d, "bin")
        os.makedirs(run)
        common = ["-n", "1024", "-l", "24", "--num-inputs", "600"]
        # write a synthetic set in the reference layout plus its category file
        out = sdgc(["-m", "BF", *common, "--synthetic", "5", "--write-data", "--write-golden",
                    "--data", data], run)
        assert "Current mode: BF" in out
        assert re.search(r"BF info: runtime [0-9.e+-]+ ms", out)
        for f in ("tsv_weights/neuron1024/n1024-l24.tsv", "MNIST/sparse-images-1024.tsv",
                  "MNIST/neuron1024-l24-categories.tsv"):
            assert os.path.exists(os.path.join(data, f)), f
        # every mode reads the TSV files from ../dataset/SDGC like the reference
        os.makedirs(os.path.join(d, "dataset"), exist_ok=True)
        for mode, pat in (("BF", r"BF info: runtime [0-9.e+-]+ ms"),
                          ("SNIG", r"SNIG info: runtime [0-9.e+-]+ ms"),
                          ("XY", r"XY info: runtime [0-9.e+-]+ms avgpost [0-9.e+-]+ms"),
                          ("SNICIT", r"SNICIT info: runtime [0-9.e+-]+ms avgpost [0-9.e+-]+ms")):
            out = sdgc(["-m", mode, *common, "-t", "6", "-b", "200"], run)
            assert re.search(pat, out), out
            assert "CHALLENGE PASSED" in out, out
            assert "Number of different categories: 0" in out
        out = sdgc(["-m", "SNICIT", *common, "-t", "6"], run)
        for line in ("pre-conv Time [SNICIT] = ", "cluster-based conversion Time [overhead] = ",
                     "post-conv Time [SNICIT] = ", "recover Time [SNICIT] = "):
            assert line in out


def test_unknown_mode_is_an_error():
    r = subprocess.run([build.CLI_BIN, "-m", "FOO"], capture_output=True, text=True)
    assert r.returncode != 0
    assert "Error mode" in r.stderr
