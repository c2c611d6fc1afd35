"""The BRAS room CR2 as the tests use it: tests/golden/cr2.json (made by
tests/golden/make_cr2.py from the reference's rooms/bras/cr2) turned into a
RoomSpec, with the reference's published wave-solver results and the air
temperature of that comparison."""
from __future__ import annotations

import json
from pathlib import Path

from wavey_gb300.materials import Material, Spectrum
from wavey_gb300.mesh import MeshRoom, RoomSpec

FIXTURE = Path(__file__).with_name("golden") / "cr2.json"


def cr2_spec() -> tuple[RoomSpec, dict, float]:
    """(room spec, published wave-solver results, air temperature in C)."""
    d = json.loads(FIXTURE.read_text())
    room = MeshRoom(d["vertices"], [(f, g) for f, g in d["faces"]], d["groups"])
    mats = {g: Material(id=m["id"], absorption=Spectrum.bands(m["freqs_hz"], m["abs"]))
            for g, m in d["materials"].items()}
    spec = RoomSpec(room, room.materials_for(mats), [(n, tuple(p)) for n, p in d["speakers"]],
                    [(n, tuple(p)) for n, p in d["mics"]], mats)
    return spec, d["published_wave_solver"], d["medium_temperature_c"]
