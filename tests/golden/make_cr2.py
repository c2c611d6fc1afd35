"""Writes tests/golden/cr2.json: the BRAS seminar room CR2 as the reference
ships it (rooms/bras/cr2: the simplified OBJ, cr2.json's material groups,
speakers S1-S2 and microphones R1-R5, the fitted absorption tables
mat_CR2_*.csv, and the air temperature of the comparison from
rooms/bras/README.md), read through this package's own reader of that format
(wavey_gb300.mesh.load_room_spec), and the reference's published results of
its wave solver alone on that room (docs/validation/plot_li2022.py: the
"Wavey wave solver" entry, bras_wave with a 700 Hz grid, means over both
sources and the five microphones at 63, 125 and 250 Hz).

Usage: python tests/golden/make_cr2.py <reference checkout>

The room data come from the Benchmark for Room Acoustical Simulation (BRAS),
L. Aspoeck et al., TU Berlin, CC BY 4.0, as redistributed by the reference.
The JSON is committed so that the tests never read the reference at run time.
"""
import ast
import json
import re
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from wavey_gb300.mesh import load_room_spec  # noqa: E402

if len(sys.argv) != 2:
    sys.exit("usage: make_cr2.py <reference checkout>")
ref = Path(sys.argv[1])
spec = load_room_spec(ref / "rooms/bras/cr2/cr2.json")
room = spec.room

# The air the CR2 comparison used (its README: "medium 19.5 °C / 41.7 % RH (CR2)").
readme = (ref / "rooms/bras/README.md").read_text()
temperature_c = float(re.search(r"medium\s+([0-9.]+)\s*°C", readme).group(1))

# The published numbers: the dict literal after "Wavey wave solver": in the plot script.
text = (ref / "docs/validation/plot_li2022.py").read_text()
bands = ast.literal_eval(re.search(r"^BANDS\s*=\s*(\[[^\]]*\])", text, re.M).group(1))
m = re.search(r'"Wavey wave solver":\s*dict\(([^)]*)\)', text)
published = {k: ast.literal_eval(v) for k, v in re.findall(r"(\w+)=(\[[^\]]*\])", m.group(1))}

out = {
    "source": "BRAS CR2 (L. Aspoeck et al., TU Berlin, CC BY 4.0), as shipped in the reference's rooms/bras/cr2",
    "vertices": room.vertices.tolist(),
    "faces": [[f, g] for f, g in room.faces],
    "groups": room.groups,
    "materials": {g: {"id": mat.id, "freqs_hz": list(mat.absorption.freqs_hz), "abs": list(mat.absorption.values)}
                  for g, mat in spec.group_materials.items()},
    "medium_temperature_c": temperature_c,
    "speakers": [[n, list(p)] for n, p in spec.speakers],
    "mics": [[n, list(p)] for n, p in spec.mics],
    "published_wave_solver": {
        "what": "bras_wave: FDTD grid f_max 700 Hz, ppw 10, 2.5 s, both sources x R1-R5, mean per octave band",
        "bands_hz": bands,
        **published,
    },
}
dst = Path(__file__).with_name("cr2.json")
dst.write_text(json.dumps(out, indent=1) + "\n")
print(f"wrote {dst}: {len(room.vertices)} vertices, {len(room.faces)} faces, {room.n_surfaces} surfaces")
