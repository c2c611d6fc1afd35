"""Writes tests/golden/materials.json: the absorption tables of the
reference's built-in materials (core/wavey-materials/src/library.json, read
through core/wavey-materials/src/library.rs:7-13), which its FDTD tests and
its impedance-fit unit tests (impedance_fit.rs:242-283) use.

Usage: python tests/golden/make_materials.py <reference checkout>

Run where a checkout of the reference is available; the JSON is committed so
the tests never read the reference at run time.
"""
import json
import sys
from pathlib import Path

if len(sys.argv) != 2:
    sys.exit("usage: make_materials.py <reference checkout>")
REF = Path(sys.argv[1]) / "core/wavey-materials/src/library.json"
lib = {m["id"]: m for m in json.loads(REF.read_text())}
out = {}
for mid in lib:
    a = lib[mid]["absorption"]
    out[mid] = a if isinstance(a, (int, float)) else {"freqs_hz": a["freqs_hz"], "values": a["values"]}
Path(__file__).with_name("materials.json").write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")
print(f"wrote {len(out)} materials")
