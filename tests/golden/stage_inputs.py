"""Stage the reference's two shipped filterbanks for the tests.

    python tests/golden/stage_inputs.py [REFERENCE_TREE]

Copies `synthetic.fil` (32 ch f32, 65,536 samples) and `GBT_Lband_PSR.fil`
(the GBT L-band tutorial observation, 96 ch 4-bit) from a PulsarSr checkout
into tests/golden/_ref_data/ after checking their SHA-256 against
inputs.json.  That folder is git-ignored (the files are the reference's
data, 33 MB), but it travels with the working tree, so tests on machines
without the reference tree still find them.  REFERENCE_TREE defaults to
$PSR_REFERENCE_DIR, then /root/reference.  Missing inputs are skipped.
"""
from __future__ import annotations

import hashlib
import json
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
DEST = os.path.join(HERE, "_ref_data")
NAMES = ("synthetic.fil", "GBT_Lband_PSR.fil")


def sha256(path: str) -> str:
    h = hashlib.sha256()
    with open(path, "rb") as f:
        for block in iter(lambda: f.read(1 << 22), b""):
            h.update(block)
    return h.hexdigest()


def main(ref: str | None = None) -> list[str]:
    ref = ref or os.environ.get("PSR_REFERENCE_DIR") or "/root/reference"
    want = json.load(open(os.path.join(HERE, "inputs.json")))["sha256"]
    staged = []
    for name in NAMES:
        dst = os.path.join(DEST, name)
        if os.path.exists(dst) and sha256(dst) == want[name]:
            staged.append(dst)
            continue
        src = os.path.join(ref, name)
        if not os.path.exists(src):
            continue
        if sha256(src) != want[name]:
            raise RuntimeError(f"{src}: SHA-256 differs from inputs.json")
        os.makedirs(DEST, exist_ok=True)
        shutil.copyfile(src, dst)
        staged.append(dst)
    return staged


if __name__ == "__main__":
    for p in main(sys.argv[1] if len(sys.argv) > 1 else None):
        print(p)
