"""The psr command line (crates/cli/src/main.rs) built on libpsr."""
import hashlib
import json
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, reference_file


@pytest.fixture(scope="module")
def psr():
    from pulsarsr_gb300 import build
    build.build()
    exe = os.path.join(os.path.dirname(build.LIB), "psr")
    assert os.path.exists(exe)
    return exe


def run(exe, *args, cwd=None):
    return subprocess.run([exe, *map(str, args)], capture_output=True, text=True, cwd=cwd)


def test_header_matches_reference_header_json(psr):
    """psr header prints the reference's output_confirm_gbt/header.json."""
    fil = reference_file("GBT_Lband_PSR.fil")
    want = open(os.path.join(GOLDEN, "gbt_header.json")).read()
    r = run(psr, "header", fil)
    assert r.returncode == 0, r.stderr
    assert r.stdout == want + "\n"


def test_header_of_synthetic_file(psr, tmp_path):
    from pulsarsr_gb300 import synth
    p = tmp_path / "x.fil"
    p.write_bytes(synth.header_bytes(96, 4, 7.2e-5, 1447.5, -1.0) + bytes(48 * 8))
    r = run(psr, "header", p)
    assert r.returncode == 0, r.stderr
    h = json.loads(r.stdout)
    assert (h["nchans"], h["nbits"], h["tsamp"], h["fch1"], h["foff"]) == \
        (96, 4, 7.2e-5, 1447.5, -1.0)
    assert list(h["fields"]) == sorted(h["fields"])
    assert list(h)[1:] == ["nchans", "nbits", "tsamp", "fch1", "foff", "data_offset"]


def test_errors_exit_nonzero(psr, tmp_path):
    from pulsarsr_gb300 import synth
    p = tmp_path / "bad.fil"
    p.write_bytes(synth._s("HEADER_START") + synth._s("surprise"))
    r = run(psr, "header", p)
    assert r.returncode != 0
    assert "unknown keyword surprise" in r.stderr
    r = run(psr, "search", p, "--min-hz", "-1")
    assert r.returncode != 0 and "invalid search settings" in r.stderr
    r = run(psr, "search", p, "--birdie", "12")
    assert r.returncode != 0 and "expected HZ:HALF_WIDTH_HZ" in r.stderr


@pytest.mark.gpu
def test_search_report_schema2_matches_oracle(gpu, oracle, psr, tmp_path):
    from pulsarsr_gb300 import synth
    obs = synth.config_c1(1)
    raw = obs.to_bytes()
    fil = tmp_path / "c1.fil"
    fil.write_bytes(raw)
    out = tmp_path / "out"
    r = run(psr, "search", fil.name, "--dm-max", 120, "--dm-step", 2, "--out", out, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    rep = json.loads((out / "report.json").read_text())
    assert list(rep) == ["schema_version", "input_sha256", "code_revision", "confirmation",
                         "input", "version", "sample_count", "tsamp", "dm_min", "dm_max",
                         "dm_step", "trial_count", "common_samples", "threads",
                         "elapsed_seconds", "min_hz", "max_hz", "threshold", "birdies",
                         "score_definition", "rfi", "candidates", "folded"]
    assert rep["schema_version"] == 2
    assert rep["input_sha256"] == hashlib.sha256(raw).hexdigest()
    assert rep["input"] == "c1.fil"
    ref = oracle.psr_search(raw, dm_max=120.0, dm_step=2.0, threads=4)
    from test_analyze import compare
    compare(rep["confirmation"], ref["confirmation"])
    assert rep["rfi"] == ref["rfi"]
    for k in ("sample_count", "trial_count", "common_samples"):
        assert rep[k] == ref[k]
    assert rep["candidates"] == [c["candidate"] for c in rep["confirmation"]["candidates"]]
    for f, c in zip(rep["folded"], rep["confirmation"]["candidates"]):
        assert f["confirmation"] == c and f["profile"] == c["profile"]
        assert f["dm_curve"] == [[p["dm"], p["discovery_profile_response"]]
                                 for p in c["dm_response"]]
    lines = r.stdout.splitlines()
    assert lines[0].startswith(f"{obs.nsamples} samples, 64 channels, 61 DM trials (step 2.000000)")
    assert sum(1 for x in lines if x.startswith("#")) == len(rep["candidates"])
    assert json.loads((out / "header.json").read_text())["nchans"] == 64


@pytest.mark.gpu
def test_fold_and_dedisperse_outputs(gpu, oracle, psr, tmp_path):
    from pulsarsr_gb300 import synth
    obs = synth.config_c1(1)
    raw = obs.to_bytes()
    fil = tmp_path / "c1.fil"
    fil.write_bytes(raw)
    r = run(psr, "dedisperse", fil, "--dm", 62, "--out", tmp_path / "dd")
    assert r.returncode == 0, r.stderr
    meta = json.loads((tmp_path / "dd" / "series.json").read_text())
    assert list(meta) == ["delays", "dm", "dtype", "normalization", "samples", "tsamp"]
    x = np.fromfile(tmp_path / "dd" / "series.f32", dtype="<f4")
    _, d = oracle.decode(raw)
    dl = oracle.delays(obs.frequencies(), obs.tsamp, 62.0)
    assert meta["delays"] == [int(v) for v in dl]
    want = oracle.apply(d, dl)
    assert meta["samples"] == want.size and x.tobytes() == want.tobytes()
    r = run(psr, "fold", fil, "--period", 0.032, "--dm", 62, "--out", tmp_path / "f")
    assert r.returncode == 0, r.stderr
    fold = json.loads((tmp_path / "f" / "fold.json").read_text())
    assert list(fold) == ["dm", "input", "profile", "searched"]
    assert list(fold["profile"]) == ["bins", "counts", "period_s", "reduced_chi_square", "snr"]
    p = oracle.profile_at(want, obs.tsamp, 0.032, 64)
    assert fold["profile"]["counts"] == [int(c) for c in p["counts"]]
    assert np.array_equal(np.array(fold["profile"]["bins"], dtype=np.float32), p["bins"])
    assert fold["searched"] is False


@pytest.mark.gpu
def test_synth_writes_reference_layout_and_searchable_file(gpu, psr, tmp_path):
    """psr synth (main.rs:341-367): the reference's header keywords, 32-bit
    time-major samples and FILE.truth.json; the injected pulsar is found."""
    from pulsarsr_gb300 import fbank
    fil = tmp_path / "s.fil"
    r = run(psr, "synth", fil, "--samples", 65536, "--channels", 32, "--seed", 5)
    assert r.returncode == 0, r.stderr
    truth = json.loads((tmp_path / "s.truth.json").read_text())
    assert list(truth) == ["nsamples", "nchans", "tsamp", "fch1", "foff", "period_s", "dm",
                           "duty_cycle", "amplitude", "seed"]
    raw = fil.read_bytes()
    h = json.loads(run(psr, "header", fil).stdout)
    assert list(h["fields"]) == ["data_type", "fch1", "foff", "nbits", "nchans", "nifs",
                                 "signed", "source_name", "tsamp"]
    assert h["nbits"] == 32 and h["nchans"] == 32
    assert len(raw) == h["data_offset"] + 65536 * 32 * 4
    x = fbank.decode(raw).data
    assert abs(float(x.mean()) - 100.0) < 0.05
    out = tmp_path / "out"
    r = run(psr, "search", fil, "--dm-max", 120, "--dm-step", 2, "--out", out)
    assert r.returncode == 0, r.stderr
    rep = json.loads((out / "report.json").read_text())
    f = [c["candidate"]["frequency_hz"] for c in rep["confirmation"]["candidates"]]
    assert any(abs(v * k - 31.25) < 0.05 for v in f for k in (1, 2, 4))
