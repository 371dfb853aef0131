"""Writes reference_fields.json from the reference's Julia sources:
- the field names of its input types (Config, Layer, PlaneGeometry, SphereGeometry,
  RayleighScatterer, MieScatterer), which the Julia binding reads by name;
- Config's literal defaults (numbers and booleans) and the DEFAULT_THEB angles in
  degrees, which the Python mirrors of Config restate;
- the ArgumentError messages of the geometries' validate methods, which the C ABI and
  the Python mirrors return.
So CPU tests can check the binding and the mirrors against the reference's own text.

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


def config_defaults(path):
    """Config's fields whose default is a number or a boolean literal."""
    out = {}
    for line in open(path, encoding="utf-8"):
        m = re.match(r"^\s+([^\s:\"#]+)::\w+\s*=\s*(\S+)\s*$", line)
        if not m:
            continue
        v = m.group(2)
        if v in ("true", "false"):
            out[m.group(1)] = v == "true"
        elif re.fullmatch(r"[-+]?\d+", v):
            out[m.group(1)] = int(v)
        elif re.fullmatch(r"[-+]?(\d+\.\d*|\d*\.\d+|\d+)([eE][-+]?\d+)?", v):
            out[m.group(1)] = float(v)
    return out


def default_theb_degrees(path):
    """The numbers of `const DEFAULT_THEB = pi / 180.0 * Float64[...]`."""
    text = open(path, encoding="utf-8").read()
    body = re.search(r"DEFAULT_THEB\s*=\s*\S+\s*/\s*180\.0\s*\*\s*Float64\[(.*?)\]", text, re.S).group(1)
    return [float(x) for x in body.replace("\n", " ").split(",") if x.strip()]


def argument_errors(path):
    return re.findall(r'ArgumentError\("([^"]*)"\)', open(path, encoding="utf-8").read())


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    found = {}
    for f in FILES:
        found.update(fields(os.path.join(ref, f)))
    table = {t: found[t] for t in TYPES}
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "reference_fields.json"), "w", encoding="utf-8") as fh:
        json.dump({"source": FILES, "fields": table,
                   "config_defaults": config_defaults(os.path.join(ref, FILES[0])),
                   "default_theb_degrees": default_theb_degrees(os.path.join(ref, FILES[0])),
                   "validate_messages": {"PlaneGeometry": argument_errors(os.path.join(ref, FILES[1])),
                                         "SphereGeometry": argument_errors(os.path.join(ref, FILES[2]))}},
                  fh, ensure_ascii=False, indent=1)
        fh.write("\n")


if __name__ == "__main__":
    main()
