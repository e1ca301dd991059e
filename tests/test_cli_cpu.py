"""The benchmark programs refuse an inconsistent .smtx file while reading it,
before any packing or GPU work (CPU only), and name the reason."""
import subprocess

import pytest

from magicube_gb300 import build

BAD = {
    "header": ("x, 64, 2\n0 1 2\n0 1\n", "malformed header"),
    "negative rows": ("-1, 64, 0\n0\n\n", "header out of range"),
    "short": ("2, 64, 3\n0 1 3\n0 1\n", "fewer offsets or columns"),
    "end": ("2, 64, 3\n0 1 2\n0 1 2\n", "end at the nonzero count"),
    "start": ("2, 64, 2\n1 1 2\n0 1\n", "start at 0"),
    "decrease": ("2, 64, 2\n0 3 2\n0 1\n", "row offsets decrease"),
    "column": ("2, 64, 2\n0 1 2\n0 64\n", "outside [0, columns)"),
}
ARGS = {
    "spmm_benchmark": ["128", "8", "0", "1", "0", "1", "8", "8"],
    "sddmm_benchmark": ["64", "8", "1", "0", "1", "8", "8"],
}


@pytest.fixture(scope="module")
def bins():
    build.build_cli()
    return build.BIN


@pytest.mark.parametrize("prog", sorted(ARGS))
@pytest.mark.parametrize("case", sorted(BAD))
def test_inconsistent_smtx_is_refused(bins, tmp_path, prog, case):
    text, reason = BAD[case]
    path = tmp_path / "bad.smtx"
    path.write_text(text)
    res = subprocess.run([str(bins / prog), str(path)] + ARGS[prog], capture_output=True, text=True, timeout=60)
    assert res.returncode == 1, res.stdout + res.stderr
    assert reason in res.stderr
    assert "runtime" not in res.stdout


@pytest.mark.parametrize("prog", sorted(ARGS))
def test_consistent_smtx_is_read_and_packed(bins, tmp_path, prog):
    """A consistent file passes the reader and the host packer (the programs
    print the aligned count before their first GPU call)."""
    from magicube_gb300 import smtx, synth
    path = tmp_path / "ok.smtx"
    smtx.write(str(path), synth.uniform_mask(16, 64, 8, 0.5, seed=1))
    res = subprocess.run([str(bins / prog), str(path)] + ARGS[prog], capture_output=True, text=True, timeout=120)
    assert " nonzero_vec: 512 aligned_ nonzero_vec: 512" in res.stdout, res.stdout + res.stderr
    assert not any(reason in res.stderr for _, reason in BAD.values())
