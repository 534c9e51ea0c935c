"""Regenerate tests/golden/input_files.json from the reference's own config-1
input files (input_file/input_{SPH,BND,DEM,DEMBND}.txt of hojin9908/Warp_SPH_GPT).

Run from the repository root with the reference checked out:
    python tests/golden/make_golden.py /path/to/Warp_SPH_GPT
Records, per file, its SHA-256, row count and the first data row, so the tests
can check that this project's generator writes the same bytes without the
reference being present.
"""
import hashlib
import json
import sys
from pathlib import Path


def main(ref_root: str) -> None:
    out = {}
    for kind in ("SPH", "BND", "DEM", "DEMBND"):
        path = Path(ref_root) / "input_file" / f"input_{kind}.txt"
        data = path.read_bytes()
        lines = data.decode("utf-8").splitlines()
        out[kind] = {"sha256": hashlib.sha256(data).hexdigest(), "rows": len(lines) - 1, "header": lines[0],
                     "first_row": lines[1] if len(lines) > 1 else ""}
    Path(__file__).with_name("input_files.json").write_text(json.dumps(out, indent=1) + "\n")


if __name__ == "__main__":
    main(sys.argv[1])
