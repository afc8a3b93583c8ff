"""Command line front-end: option parsing, error reporting and the streamed JSON format
(CPU; the GPU run through the CLI is in test_gpu_end_to_end.py)."""
import io
import json
import subprocess
import sys

import numpy as np
import pytest

from bqa_gb300 import cli


def test_parse_defaults_and_paths(tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    ctx = cli.parse_args(["prog"])
    assert ctx == {"input": None, "output": None, "log-level": "INFO"}
    ctx = cli.parse_args(["prog", "-i", "a.json", "--output", "b.json", "-l", "DEBUG"])
    assert ctx["input"].name == "a.json" and ctx["output"].name == "b.json" and ctx["log-level"] == "DEBUG"


@pytest.mark.parametrize("argv,msg", [(["prog", "-i", "a.txt"], "must have .json suffix"),
                                      (["prog", "-l", "LOUD"], "cannot be interpeted"),
                                      (["prog", "-o"], "is not provided after")])
def test_parse_errors(argv, msg):
    with pytest.raises(cli.CliError, match=msg):
        cli.parse_args(argv)


def test_unknown_option_exits_1():
    with pytest.raises(SystemExit) as e:
        cli.parse_args(["prog", "--bogus"])
    assert e.value.code == 1


def test_streamed_results_are_the_reference_json():
    bloch = np.array([[0.1, -0.2, 0.3], [1.0 / 3.0, 0.0, -1.0]])
    outcomes = np.array([1, -1])
    buf = io.StringIO()
    cli.write_results([["bloch_vectors", bloch], ["measurement_outcomes", outcomes]], buf)
    assert json.loads(buf.getvalue()) == [["bloch_vectors", bloch.tolist()], ["measurement_outcomes", [1, -1]]]


def test_bad_config_reports_cause_chain(tmp_path):
    p = tmp_path / "job.json"
    p.write_text(json.dumps({"edges": [[[0, 0], 1.0]]}))
    r = subprocess.run([sys.executable, "-m", "bqa_gb300.cli", "-i", str(p)], capture_output=True, text=True,
                       cwd=str(tmp_path), env={**__import__("os").environ,
                                               "PYTHONPATH": str(__import__("pathlib").Path(__file__).parents[1])})
    assert r.returncode == 1
    assert "Invalid config" in r.stderr and "caused by" in r.stderr and "must not be equal" in r.stderr
