"""Regenerate the committed MIR fixtures of the bundled device models.

The Verilog-A sources live in the reference tree (``vajax/devices/models``);
this script compiles them with the project's Verilog-A front end and writes
one JSON file per model next to this script.  The JSON files are what the
build and the tests consume, so machines without the reference tree (the GPU
hosts) never need the sources.

Usage: ``python -m vajax_gb300.devices.generate <reference-root>``
"""

import json
import sys
from pathlib import Path

from vajax_gb300.va.frontend import compile_va_file

# fixture name -> path of the Verilog-A source inside the reference tree
SOURCES = {
    "resistor": "vajax/devices/models/resistor.va",
    "capacitor": "vajax/devices/models/capacitor.va",
    "ekv_longchannel": "vajax/devices/models/ekv_longchannel/ekv_longchannel.va",
    "ekv": "vajax/devices/models/ekv/ekv.va",
}


def main(ref_root: str) -> None:
    out_dir = Path(__file__).resolve().parent
    for key, rel in SOURCES.items():
        model = compile_va_file(Path(ref_root) / rel)
        model["source"] = rel
        (out_dir / f"{key}.json").write_text(json.dumps(model, separators=(",", ":"), sort_keys=True))
        print(f"{key}: {len(model['mir']['instructions'])} instructions, "
              f"{len(model['dae']['jacobian'])} Jacobian entries")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python -m vajax_gb300.devices.generate <reference-root>")
    main(sys.argv[1])
