"""Writes reference_fields.json: the field names of the reference's input types (Config,
Layer, PlaneGeometry, SphereGeometry, RayleighScatterer, MieScatterer), read from the
reference's Julia sources. The Julia binding reads these fields by name, so the fixture
lets a CPU test check every field access of the binding without Julia.

Run from the repository root with the reference checked out (default /root/reference):
    python tests/golden/make_reference_fields.py [reference_dir]
"""
import json
import os
import re
import sys

FILES = ["src/config.jl", "src/geometries/plane.jl", "src/geometries/sphere.jl", "src/scatterers/rayleigh.jl",
         "src/scatterers/mie.jl"]
TYPES = ["Config", "Layer", "PlaneGeometry", "SphereGeometry", "RayleighScatterer", "MieScatterer"]


def fields(path):
    """{type name: [field names]} for the top-level structs of one Julia file."""
    out, name = {}, None
    for line in open(path, encoding="utf-8"):
        m = re.match(r"^(?:Base\.@kwdef\s+)?(?:mutable\s+)?struct\s+(\w+)", line)
        if m:
            name = m.group(1)
            out[name] = []
            continue
        if name is not None:
            if re.match(r"^end\b", line):
                name = None
                continue
            f = re.match(r"^\s+([^\s:\"#]+)::", line)
            if f:
                out[name].append(f.group(1))
    return out


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    found = {}
    for f in FILES:
        found.update(fields(os.path.join(ref, f)))
    table = {t: found[t] for t in TYPES}
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "reference_fields.json"), "w", encoding="utf-8") as fh:
        json.dump({"source": FILES, "fields": table}, fh, ensure_ascii=False, indent=1)
        fh.write("\n")


if __name__ == "__main__":
    main()
