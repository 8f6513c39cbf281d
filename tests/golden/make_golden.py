"""Extract the reference's saved outputs into small golden fixtures.

Run once in a checkout where the PulsarSr reference tree is available:

    python tests/golden/make_golden.py /path/to/PulsarSr

It reads only the reference's own saved run outputs (schema-2 reports, the
DM-62 series metadata, the fold record and the GBT header text) and writes
compact JSON files beside this script.  The input filterbanks themselves
are staged separately by stage_inputs.py (git-ignored copies).
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def member(m: dict) -> list:
    return [m["frequency_hz"], m["dm"], m["harmonics"], m["score"]]


def family_summary(c: dict) -> dict:
    return {
        "candidate": member(c["candidate"]),
        "refined_dm": c["refined_dm"],
        "profile": {k: c["profile"][k] for k in ("period_s", "snr", "reduced_chi_square",
                                                  "bins", "counts")},
        "window": c["window"],
        "validation": c["validation"],
        "zero_dm_validation": c["zero_dm_validation"],
        "zero_dm_period_s": c["zero_dm_period_s"],
        "zero_dm_window": c["zero_dm_window"],
        "dm_contrast": c["dm_contrast"],
        "dispersion_widths": c["dispersion_widths"],
        "zero_dm_related_spectral_ratio": c["zero_dm_related_spectral_ratio"],
        "time_parts": c["time_parts"],
        "subbands": c["subbands"],
        "time_profiles": c["time_profiles"],
        "subband_profiles": c["subband_profiles"],
        "dm_response": [[p["dm"], p["spectral_score"], p["discovery_profile_response"]]
                        for p in c["dm_response"]],
        "harmonic_members": [member(m) for m in c["harmonic_members"]],
        "accepted": c["accepted"],
        "rejection_reasons": c["rejection_reasons"],
    }


def report_summary(path: str) -> dict:
    r = json.load(open(path))
    conf = r["confirmation"]
    return {
        "source": os.path.relpath(path, REF),
        "settings": {k: r[k] for k in ("sample_count", "tsamp", "dm_min", "dm_max", "dm_step",
                                        "trial_count", "common_samples", "min_hz", "max_hz",
                                        "threshold", "birdies")},
        "input_sha256": r["input_sha256"],
        "rfi": r["rfi"],
        "confirmation": {k: conf[k] for k in ("discovery_samples", "validation_start_sample",
                                               "validation_samples", "common_samples",
                                               "trial_count")},
        "families": [family_summary(c) for c in conf["candidates"]],
    }


def main(ref: str) -> None:
    global REF
    REF = ref
    out = {}
    s = json.load(open(os.path.join(ref, "output_dm62", "series.json")))
    out["gbt_dm62_series.json"] = {"source": "output_dm62/series.json", **s}
    f = json.load(open(os.path.join(ref, "output_fold", "fold.json")))
    out["gbt_fold.json"] = {"source": "output_fold/fold.json", **f}
    out["gbt_report_summary.json"] = report_summary(
        os.path.join(ref, "output_confirm_gbt", "report.json"))
    out["synth_report_summary.json"] = report_summary(
        os.path.join(ref, "output_confirm_synth", "report.json"))
    hashes = {}
    for name in ("GBT_Lband_PSR.fil", "synthetic.fil"):
        with open(os.path.join(ref, name), "rb") as fh:
            hashes[name] = hashlib.sha256(fh.read()).hexdigest()
    out["inputs.json"] = {"sha256": hashes}
    for name, obj in out.items():
        with open(os.path.join(HERE, name), "w") as fh:
            json.dump(obj, fh, separators=(",", ":"))
        print(name, os.path.getsize(os.path.join(HERE, name)))
    # `psr header` output of the GBT file, byte for byte (pretty JSON text)
    with open(os.path.join(ref, "output_confirm_gbt", "header.json"), "rb") as fh:
        text = fh.read()
    with open(os.path.join(HERE, "gbt_header.json"), "wb") as fh:
        fh.write(text)
    print("gbt_header.json", len(text))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PSR_REFERENCE_DIR", ""))
