"""The benchmark driver lmm_bench (cli/lmm_bench.cpp), which replaces the
reference's main.cpp + MPTest/runbatch.sh + getresults.sh: argument handling
without a GPU; on the GPU, its per-call results equal the library call's and
its throughput line follows LiborMarketModel/README.txt:113-114."""
import os
import re
import subprocess

import pytest

from conftest import pkg


def cli():
    P = pkg()
    exe = os.path.join(os.path.dirname(P.LIB_PATH), "lmm_bench")
    if not os.path.exists(exe):
        P.build()
    return exe


def run(*args, timeout=600):
    return subprocess.run([cli(), *map(str, args)], capture_output=True, text=True, timeout=timeout)


def test_help_and_argument_errors():
    r = run("--help")
    assert r.returncode == 0 and "usage:" in r.stdout and "--processes" in r.stdout
    for bad in (["--loops", "0"], ["0"], ["--processes", "0"], ["--rng", "mt19937"], ["--bogus"],
                ["--loops"]):
        r = run(*bad)
        assert r.returncode == 2, (bad, r.stdout, r.stderr)


def _field(text, name):
    return float(re.search(name + r"[=:]\s*([-+0-9.eE]+)", text).group(1))


@pytest.mark.gpu
@pytest.mark.parametrize("precision,rng", [("f64", "philox"), ("f32", "mrg32k3a")])
def test_results_match_the_library_call(precision, rng):
    P = pkg()
    n = 4096
    args = [n, "--loops", 2, "--processes", 2, "--rng", rng] + (["--f32"] if precision == "f32" else [])
    r = run(*args)
    assert r.returncode == 0, r.stderr
    fn = P.swaption_greeks_f32 if precision == "f32" else P.swaption_greeks
    _, v, lb = fn(n, rng=rng)
    assert _field(r.stdout, r"Result: value") == pytest.approx(v, rel=1e-9)
    assert _field(r.stdout, r"lambda") == pytest.approx(lb, rel=1e-9, abs=1e-12)
    # every process and loop prints main.cpp's lines
    assert len(re.findall(r"Total time: [0-9.]+ ms", r.stdout)) == 4
    avg = _field(r.stdout, "Average total time per call")
    thr = _field(r.stdout, "LiborMarketModel throughput")
    assert thr == pytest.approx(n * 2 / (avg * 1e-3), rel=1e-5)
