"""`psr search` on the reference's own input files, on the GPU, against the
reports the reference saved for them (output_confirm_synth/report.json and
output_confirm_gbt/report.json, summarised in tests/golden/).

Integers, lists, windows, decisions, refined DMs and every measurement must
match; spectral scores within 2e-6 relative (the reference's FFT is rustfft,
whose rounding is not reproduced), frequencies within 1e-9.  The files are
found through PSR_REFERENCE_DIR or the copies tests/golden/stage_inputs.py
stages; the tests skip without them."""
import json
import os

import pytest

from conftest import GOLDEN, reference_file
from test_cli import psr, run  # noqa: F401  (the psr fixture)
from test_oracle_golden import compare_report

pytestmark = pytest.mark.gpu


def golden(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def search_file(psr, fil, tmp_path, *args):
    out = tmp_path / "out"
    r = run(psr, "search", fil, "--out", out, *args)
    assert r.returncode == 0, r.stderr
    return json.loads((out / "report.json").read_text())


def check_settings(rep, g):
    for k, v in g["settings"].items():
        assert rep[k] == v, k
    assert rep["input_sha256"] == g["input_sha256"]
    assert rep["rfi"] == g["rfi"]


def test_synthetic_fil_report_matches_reference(gpu, psr, tmp_path):  # noqa: F811
    """synthetic.fil (32 ch f32): the reference's schema-2 search settings."""
    g = golden("synth_report_summary.json")
    fil = reference_file("synthetic.fil")
    rep = search_file(psr, fil, tmp_path, "--dm-max", 120, "--dm-step", 2, "--min-hz", 10,
                      "--max-hz", 2000, "--threshold", 8, "--top", 5, "--bins", 64)
    check_settings(rep, g)
    compare_report(rep, g, score_rtol=2e-6)


def test_gbt_fil_report_matches_reference(gpu, psr, tmp_path):  # noqa: F811
    """GBT_Lband_PSR.fil (96 ch 4-bit): the full 2000-trial default search."""
    g = golden("gbt_report_summary.json")
    fil = reference_file("GBT_Lband_PSR.fil")
    rep = search_file(psr, fil, tmp_path, "--dm-max", 500, "--min-hz", 15, "--max-hz", 2000,
                      "--threshold", 8, "--top", 5, "--bins", 64)
    check_settings(rep, g)
    compare_report(rep, g, score_rtol=2e-6)
