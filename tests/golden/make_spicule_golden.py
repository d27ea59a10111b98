"""Freeze the reference's own spicule-run output as a fixture.

Run from the repository root, where the reference tree is present:

    python tests/golden/make_spicule_golden.py <root of the reference tree>

The reference ships the output of one run of its spicule model
(cans_beta_one/cans1d/md_spicule/hdmlw/: params.txt, out.txt and the DAC
files x, bx, bxm, sc, scm, gx, gxm, rr, rrm, t, ro, pr, vx, vy, by).  This
script reads them with utrip_gb300.dac (which checks their framing and
header) and stores, for every file, its arrays and the SHA-256 of its bytes,
plus the two text files, in spicule_reference.npz.  The tests then check the
DAC writer byte for byte and the spicule set-up value for value against the
reference's output without needing the reference tree.
"""
import hashlib
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from utrip_gb300 import dac  # noqa: E402

OUT = Path(__file__).resolve().parent / "spicule_reference.npz"
RUN = Path("cans_beta_one/cans1d/md_spicule/hdmlw")
FILES = ["x", "bx", "bxm", "sc", "scm", "gx", "gxm", "rr", "rrm", "t", "ro", "pr", "vx", "vy",
         "by"]


def main(ref_root: str) -> None:
    d = Path(ref_root) / RUN
    out = {}
    for name in FILES:
        raw = (d / f"{name}.dac").read_bytes()
        f = dac.DacFile(d / f"{name}.dac")
        out[f"{name}_records"] = f.records
        out[f"{name}_sha256"] = np.array(hashlib.sha256(raw).hexdigest())
        out[f"{name}_unlimited"] = np.array(f.unlimited)
        out[f"{name}_mtype"] = np.array(f.mtype)
    out["params_txt"] = np.array((d / "params.txt").read_text())
    out["out_txt"] = np.array((d / "out.txt").read_text())
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes)")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: make_spicule_golden.py <root of the reference tree>")
    main(sys.argv[1])
