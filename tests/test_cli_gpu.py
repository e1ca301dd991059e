"""The command-line benchmark programs, run with the reference's argument
lists on synthetic .smtx matrices: each must report its own host
verification as PASS and print the runtime / TOP/s lines."""
import re
import subprocess

import pytest

from magicube_gb300 import build, smtx, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bins(cuda):
    build.build_cli()
    return build.BIN


@pytest.mark.parametrize("preA,preB", [(4, 4), (8, 4), (12, 4), (16, 4), (8, 8), (12, 8), (16, 8), (16, 16)])
@pytest.mark.parametrize("V", [2, 8])
@pytest.mark.parametrize("sort", [0, 1])
def test_spmm_benchmark_cli(bins, tmp_path, preA, preB, V, sort):
    m = synth.normal_mask(64, 512, V, 0.8, seed=preA + preB + V)
    path = tmp_path / "m.smtx"
    smtx.write(path, m)
    res = subprocess.run([str(bins / "spmm_benchmark"), str(path), "256", str(V), "0", str(sort), "1", "1",
                          str(preA), str(preB)], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr
    assert "Results verification: PASS" in res.stdout, res.stdout
    assert re.search(r"Magicube SpMM runtime [0-9.e+-]+ ms", res.stdout)
    assert re.search(r"performance TOP/s: [0-9.e+-]+", res.stdout)


@pytest.mark.parametrize("preA,preB", [(4, 4), (8, 8), (16, 16), (16, 8)])
@pytest.mark.parametrize("V", [2, 8])
def test_sddmm_benchmark_cli(bins, tmp_path, preA, preB, V):
    m = synth.normal_mask(64, 1024, V, 0.9, seed=preA + V)
    path = tmp_path / "m.smtx"
    smtx.write(path, m)
    res = subprocess.run([str(bins / "sddmm_benchmark"), str(path), "128", str(V), "1", "1", "1", str(preA),
                          str(preB)], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr
    assert "SDDMM results verification: PASS" in res.stdout, res.stdout
    assert re.search(r"Magicube SDDMM runtime [0-9.e+-]+ ms", res.stdout)


def test_cli_usage(bins):
    res = subprocess.run([str(bins / "spmm_benchmark"), "-h"], capture_output=True, text=True)
    assert "usage" in res.stdout
