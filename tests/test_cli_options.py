"""Options of the `brr` CLI: the reference's parser semantics (CPU only).

Cases of test/optionstest.cpp:5-184 (variance components from the command
line and from a file, input type from the extension, analysis type), plus the
additions of this CLI: --bfile and per-group mixture sizes.
"""
import json
import subprocess
from pathlib import Path

import pytest

from bayesrrcmd_gb300.build import build_cli


@pytest.fixture(scope="module")
def brr():
    return str(build_cli())


def opts(brr, *args):
    r = subprocess.run([brr, *args, "--print-options"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_default_variance_components(brr):
    assert opts(brr)["S"] == [[0.01, 0.001, 0.0001]]


def test_variance_components_from_command_line(brr):
    assert opts(brr, "--S", "0.1,0.1")["S"] == [[0.1, 0.1]]
    assert opts(brr, "--S", "0.01,0.001,0.0001;0.02,0.002,0.0002")["S"] == \
        [[0.01, 0.001, 0.0001], [0.02, 0.002, 0.0002]]


def test_variance_components_from_file(brr, tmp_path):
    f = tmp_path / "test.cva"
    f.write_text("0.001,0.01;0.001,0.01")   # the reference's test.groups/test.cva
    assert opts(brr, "--S", str(f))["S"] == [[0.001, 0.01], [0.001, 0.01]]


def test_unparsable_variance_components_give_empty(brr, tmp_path):
    assert opts(brr, "--S", str(tmp_path / "non-existant.cva"))["S"] == []


def test_groups_may_have_their_own_mixture_size(brr):
    assert opts(brr, "--S", "0.01,0.001,0.0001;0.1,0.01")["S"] == [[0.01, 0.001, 0.0001], [0.1, 0.01]]


def test_input_type_from_extension(brr):
    assert opts(brr, "--data-file", "foo.bed")["input"] == 1
    assert opts(brr, "--data-file", "foo.csv")["input"] == 2
    assert opts(brr, "--data-file", "foo")["input"] == 0
    o = opts(brr, "--bfile", "dir/foo")
    assert o["input"] == 1 and o["data"] == "dir/foo.bed"


def test_analysis_type(brr):
    assert opts(brr, "--preprocess")["analysis"] == 1
    assert opts(brr, "--analysis-type", "preprocess")["analysis"] == 1
    assert opts(brr, "--analysis-type", "ppbayes")["analysis"] == 2
    # test/optionstest.cpp:133-154: the reference's other analysis types parse to
    # their own values (src/common.h:8-15) ...
    assert opts(brr, "--analysis-type", "asyncppbayes")["analysis"] == 3
    assert opts(brr, "--analysis-type", "gauss")["analysis"] == 4
    assert opts(brr, "--analysis-type", "asyncgauss")["analysis"] == 5
    assert opts(brr, "--analysis-type", "other")["analysis"] == 0
    assert opts(brr)["analysis"] == 0


@pytest.mark.parametrize("kind", ["gauss", "asyncgauss"])
def test_analyses_off_this_path_are_refused(brr, kind):
    """... and the BayesW analyses are refused with a message naming what runs here."""
    r = subprocess.run([brr, "--analysis-type", kind, "--S", "0.01"], capture_output=True, text=True)
    assert r.returncode == 1 and "ppbayes" in r.stderr and "not supported" in r.stderr


def test_asyncppbayes_takes_the_analysis_tokens(brr):
    """asyncppbayes runs with --analysis-tokens markers in flight (the
    reference's default 20, src/options.hpp:33); the GPU batch holds 1..64."""
    assert opts(brr, "--analysis-type", "asyncppbayes")["tokens"] == 20
    assert opts(brr, "--analysis-type", "asyncppbayes", "--analysis-tokens", "7")["tokens"] == 7


def test_sparse_data_and_chain_flags(brr):
    o = opts(brr, "--sparse-data", "ragged", "--chain-length", "10", "--burn-in", "2", "--thin", "3",
             "--seed", "5", "--mcmc-samples", "x.csv", "--form", "fp32c")
    assert (o["sparse"], o["chain"], o["burnin"], o["thin"], o["seed"], o["samples"], o["form"]) == \
        (3, 10, 2, 3, 5, "x.csv", "fp32c")
    assert opts(brr, "--sparse-data", "other")["sparse"] == 0


def test_unknown_option_is_an_error(brr):
    r = subprocess.run([brr, "--bogus"], capture_output=True, text=True)
    assert r.returncode == 1 and "invalid option" in r.stderr


def test_option_file(brr, tmp_path):
    """--inp-file reads key/value pairs and ignores the arguments after it
    (src/options.cpp:98-101), so --print-options must come first."""
    f = tmp_path / "run.inp"
    # a comment key consumes exactly one value token, as in the reference
    f.write_text("# note\nchainLength 7\n// x\nthin 2\nS 0.5,0.05\n")
    r = subprocess.run([brr, "--print-options", "--inp-file", str(f), "--bogus"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    o = json.loads(r.stdout.strip().splitlines()[-1])
    assert (o["chain"], o["thin"], o["S"]) == (7, 2, [[0.5, 0.05]])


def test_logs_fixed_effects_and_failure_options(brr):
    """--colLog, --fixedEffectNumber and --failure are parsed as the reference
    does (src/options.cpp:167-174, :230-233)."""
    o = opts(brr, "--colLog", "cols.csv", "--fixedEffectNumber", "0", "--failure", "fail.txt")
    assert (o["colLog"], o["fixed"], o["failure"]) == ("cols.csv", 0, "fail.txt")
    assert (opts(brr)["colLog"], opts(brr)["fixed"]) == ("", 0)


def test_fixed_effects_are_refused_before_any_work(brr):
    r = subprocess.run([brr, "--analysis-type", "ppbayes", "--fixedEffectNumber", "2", "--bfile", "missing"],
                       capture_output=True, text=True)
    assert r.returncode == 1 and "fixed effects are not supported" in r.stderr
