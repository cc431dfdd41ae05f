"""The `abm` driver's command line (no GPU: every case here stops before the device is touched)."""
import subprocess

import pytest

from paragraph_gb300.build import DRIVER


def _run(*args):
    return subprocess.run([str(DRIVER), *args], capture_output=True, text=True, timeout=60)


def test_help_and_required_options(built):
    r = _run("--help")
    assert r.returncode == 0 and "--edgelist" in r.stderr
    r = _run("--edgelist", "e.csv")
    assert r.returncode == 1 and "--nodelist is required" in r.stderr


@pytest.mark.parametrize("args,msg", [
    (["--bogus", "1"], "unknown option --bogus"),
    (["--edgelist"], "missing value for --edgelist"),
    (["--edgelist", "e", "--nodelist", "n", "--growth-rate", "0.1", "--num-cycles", "2",
      "--output-file", "o", "--auxiliary-information-file", "a", "--log-file", "l"],
     "--same-year-proportion is required"),
    (["--edgelist", "e", "--nodelist", "n", "--growth-rate", "0.1", "--num-cycles", "2",
      "--same-year-proportion", "0", "--output-file", "o", "--auxiliary-information-file", "a",
      "--log-file", "l"], "--out-degree-bag and --recency-probabilities are required"),
])
def test_bad_command_lines(built, args, msg):
    r = _run(*args)
    assert r.returncode == 1 and msg in r.stderr


def test_missing_input_file_is_an_error(built, tmp_path):
    r = _run("--edgelist", str(tmp_path / "none.csv"), "--nodelist", str(tmp_path / "none2.csv"),
             "--growth-rate", "0.1", "--num-cycles", "1", "--same-year-proportion", "0",
             "--weight-model", "baseline", "--output-file", str(tmp_path / "o"),
             "--auxiliary-information-file", str(tmp_path / "a"), "--log-file", str(tmp_path / "l"))
    assert r.returncode == 1 and "cannot open" in r.stderr
    assert "[ERROR]" in (tmp_path / "l").read_text()


def test_malformed_number_is_an_error(built, tmp_path):
    r = _run("--edgelist", "e", "--nodelist", "n", "--growth-rate", "fast", "--num-cycles", "1",
             "--same-year-proportion", "0", "--weight-model", "baseline", "--output-file", "o",
             "--auxiliary-information-file", "a", "--log-file", str(tmp_path / "l"))
    assert r.returncode == 1 and "malformed number" in r.stderr
