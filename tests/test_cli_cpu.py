"""The SDGC command line's argument handling (no GPU: every case below ends
before the first CUDA call).  The reference's CLI (main/SDGC.cu:13-48,
107-110) takes -m/-n/-l/-t/-b and rejects an unknown mode; errors here are
exit statuses with a message, never a crash."""
import os
import subprocess

import pytest

from snicit_gb300 import build


def run(args, cwd):
    assert os.path.exists(build.CLI_BIN), "build the CLI first (__graft_entry__.build())"
    return subprocess.run([build.CLI_BIN, *args], cwd=cwd, capture_output=True, text=True,
                          timeout=60)


def test_help_lists_the_reference_flags(tmp_path):
    r = run(["--help"], tmp_path)
    assert r.returncode == 0
    for flag in ("-m,--mode SNICIT|BF|SNIG|XY", "-n,--num_neurons", "-l,--num_layers",
                 "-t,--threshold", "-b,--input_batch_size"):
        assert flag in r.stdout


@pytest.mark.parametrize("args,code,message", [
    (["-m", "FOO"], 1, "Error mode"),
    (["--bogus"], 2, "unknown option --bogus"),
    (["-n"], 2, "-n needs a value"),
])
def test_bad_arguments_exit_with_a_status(tmp_path, args, code, message):
    r = run(args, tmp_path)
    assert r.returncode == code
    assert message in r.stdout + r.stderr


def test_missing_weight_file_is_reported(tmp_path):
    """The reference layout ../dataset/SDGC/tsv_weights/neuronN/nN-lK.tsv is
    read on the host before any device work; a missing file is an I/O error
    naming the path."""
    r = run(["-m", "BF", "-n", "1024", "-l", "2", "--data", str(tmp_path / "none")], tmp_path)
    assert r.returncode == 1
    assert "Current mode: BF" in r.stdout
    assert "I/O error" in r.stderr and "n1024-l1.tsv" in r.stderr
