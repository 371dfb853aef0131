"""The C ABI's structs as the bindings see them: the ctypes structures of the Python host
package and the Julia binding's structs (julia/MCRTGB300.jl, the drop-in for
MonteCarloRadiativeTransfer.jl's `simulate`/`run_rt`) must mirror include/mcrt.h field by
field, with the same offsets and sizes; and every function the Julia binding `ccall`s
must be declared there. No GPU and no Julia are needed: the header and the binding are
parsed as text, and C layouts follow the LP64 natural alignment of x86_64 and aarch64."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "mcrt.h")
JULIA = os.path.join(ROOT, "montecarloradiativetransfer.jl_gb300", "julia", "MCRTGB300.jl")

# size in bytes of the C scalar kinds (also their alignment on LP64), and the Julia names
C_SCALARS = {"int": 4, "double": 8, "int64_t": 8, "uint64_t": 8, "uint32_t": 4, "float": 4}
JL_SCALARS = {"Cint": "int", "Float64": "double", "Cdouble": "double", "Int64": "int64_t", "UInt64": "uint64_t",
              "UInt32": "uint32_t", "Cfloat": "float"}


def _strip_comments(s):
    s = re.sub(r"/\*.*?\*/", " ", s, flags=re.S)
    return re.sub(r"//[^\n]*", " ", s)


def header_structs():
    """{name: [(field, kind, count)]} for every `typedef struct {...} name;` of mcrt.h,
    kind being a scalar type name or "ptr"."""
    text = _strip_comments(open(HEADER, encoding="utf-8").read())
    out = {}
    for body, name in re.findall(r"typedef\s+struct\s*\{(.*?)\}\s*(\w+)\s*;", text, flags=re.S):
        fields = []
        for decl in body.split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            m = re.match(r"(?:const\s+)?(\w+)\s*(.*)$", decl)
            base, rest = m.group(1), m.group(2)
            for d in rest.split(","):
                d = d.strip()
                dm = re.match(r"(\**)\s*(?:const\s+)?(\w+)\s*(?:\[(\d+)\])?$", d)
                assert dm, (name, decl)
                ptr, fname, count = dm.group(1), dm.group(2), int(dm.group(3) or 1)
                if ptr:
                    fields.append((fname, "ptr", count))
                else:
                    assert base in C_SCALARS, (name, decl)
                    fields.append((fname, base, count))
        out[name] = fields
    return out


def layout(fields):
    """[(offset, size)] per field and the struct size, LP64 natural alignment."""
    off, align_max, res = 0, 1, []
    for _, kind, count in fields:
        sz = 8 if kind == "ptr" else C_SCALARS[kind]
        off = (off + sz - 1) // sz * sz
        res.append((off, sz * count))
        off += sz * count
        align_max = max(align_max, sz)
    return res, (off + align_max - 1) // align_max * align_max


def julia_structs():
    """{c_name: [(field, kind, count)]} for every `struct X  # c_name` of the binding."""
    text = open(JULIA, encoding="utf-8").read()
    out = {}
    for name, cname, body in re.findall(r"^struct\s+(\w+)\s*#\s*(\w+)\s*\n(.*?)^end", text, flags=re.S | re.M):
        fields = []
        for line in body.splitlines():
            line = line.split("#")[0].strip()
            if not line:
                continue
            fname, typ = [x.strip() for x in line.split("::")]
            if typ.startswith("Ptr{"):
                fields.append((fname, "ptr", 1))
            elif typ.startswith("NTuple{"):
                n, t = re.match(r"NTuple\{(\d+),\s*(\w+)\}", typ).groups()
                fields.append((fname, JL_SCALARS[t], int(n)))
            else:
                fields.append((fname, JL_SCALARS[typ], 1))
        out[cname] = (name, fields)
    return out


def test_header_parses():
    hs = header_structs()
    for name in ("mcrt_scatterer_desc", "mcrt_config", "mcrt_layer", "mcrt_geometry", "mcrt_run_opts",
                 "mcrt_stats", "mcrt_instance", "mcrt_server_opts", "mcrt_request", "mcrt_ticket_info"):
        assert name in hs and hs[name], name


CTYPES_FOR = {"ScattererDesc": "mcrt_scatterer_desc", "ConfigC": "mcrt_config", "LayerC": "mcrt_layer",
              "GeometryC": "mcrt_geometry", "RunOpts": "mcrt_run_opts", "Stats": "mcrt_stats",
              "ServerOpts": "mcrt_server_opts", "RequestC": "mcrt_request", "TicketInfo": "mcrt_ticket_info",
              "InstanceC": "mcrt_instance"}


@pytest.mark.parametrize("cls", sorted(CTYPES_FOR))
def test_ctypes_structures_mirror_the_header(M, cls):
    from mcrt_gb300 import _lib

    S = getattr(_lib, cls)
    fields = header_structs()[CTYPES_FOR[cls]]
    offs, size = layout(fields)
    assert [f[0] for f in S._fields_] == [f[0] for f in fields]
    assert C.sizeof(S) == size
    for (fname, _, _), (off, sz) in zip(fields, offs):
        d = getattr(S, fname)
        assert (d.offset, d.size) == (off, sz), (cls, fname)


def test_julia_structs_mirror_the_header():
    hs = header_structs()
    js = julia_structs()
    assert set(js) >= {"mcrt_scatterer_desc", "mcrt_config", "mcrt_layer", "mcrt_geometry", "mcrt_run_opts"}
    for cname, (jname, jfields) in js.items():
        cfields = hs[cname]
        assert [(k, n) for _, k, n in jfields] == [(k, n) for _, k, n in cfields], (jname, cname)
        assert layout(jfields) == layout(cfields)


def _call_args(text, name):
    """The argument lists of every positional call `name(...)` in ``text`` (keyword calls
    and definitions are skipped), split at top-level commas."""
    out = []
    for m in re.finditer(r"(?<![\w.])" + name + r"\(", text):
        depth, k, args, cur = 1, m.end(), [], ""
        while depth:
            ch = text[k]
            depth += ch in "({["
            depth -= ch in ")}]"
            if depth == 1 and ch == ",":
                args.append(cur)
                cur = ""
            elif depth:
                cur += ch
            k += 1
        args.append(cur)
        keyword = args[0].lstrip().startswith(";") or any("=" in a for a in args)
        if any(a.strip() for a in args) and not keyword:
            out.append([a.strip() for a in args])
    return out


def test_julia_positional_constructors_fill_every_field():
    text = open(JULIA, encoding="utf-8").read()
    js = {jname: fields for jname, fields in julia_structs().values()}
    for jname, n_calls in (("RunOpts", 1), ("ScattererDesc", 2)):
        calls = _call_args(text, jname)
        assert len(calls) == n_calls, (jname, calls)
        for args in calls:
            assert len(args) == len(js[jname]), (jname, args)


def test_julia_ccalls_are_declared_in_the_header():
    declared = set(re.findall(r"\b(mcrt_\w+)\s*\(", _strip_comments(open(HEADER, encoding="utf-8").read())))
    called = set(re.findall(r"ccall\(\(:(\w+),\s*libmcrt\)", open(JULIA, encoding="utf-8").read()))
    assert called and called <= declared, called - declared


def test_julia_binding_reads_only_fields_the_reference_defines():
    """Every field the binding reads from the reference's objects (cfg::Config, g a
    geometry, l a Layer, s a scatterer) is a field of the reference's type, by the names
    in tests/golden/reference_fields.json (extracted from the reference's sources by
    make_reference_fields.py beside it): a misspelt or missing field would only fail
    when Julia runs the binding."""
    import json

    ref = json.load(open(os.path.join(ROOT, "tests", "golden", "reference_fields.json"), encoding="utf-8"))["fields"]
    allowed = {
        "cfg": set(ref["Config"]),
        "g": set(ref["PlaneGeometry"]) | set(ref["SphereGeometry"]),
        "l": set(ref["Layer"]),
        "s": set(ref["RayleighScatterer"]) | set(ref["MieScatterer"]),
    }
    src = open(JULIA, encoding="utf-8").read()
    seen = {}
    for obj, field in re.findall(r"(?<![\w.])(cfg|g|l|s)\.([^\W\d]\w*)", src):
        seen.setdefault(obj, set()).add(field)
    assert {"cfg", "g", "l", "s"} <= set(seen)
    for obj, names in seen.items():
        assert names <= allowed[obj], (obj, sorted(names - allowed[obj]))
    assert len(seen["cfg"]) >= 15  # the binding marshals the whole Config


def test_julia_parity_script_uses_the_reference_constructors():
    """julia/test_binding.jl builds the reference's types with keyword constructors
    (the types are Base.@kwdef structs): every keyword is a field of that type (for
    MieScatterer, the keywords of its outer constructor, Nθ and random_points, are fields
    too), and every field it reads from them exists (names from
    tests/golden/reference_fields.json)."""
    import json

    ref = json.load(open(os.path.join(ROOT, "tests", "golden", "reference_fields.json"), encoding="utf-8"))["fields"]
    src = open(os.path.join(os.path.dirname(JULIA), "test_binding.jl"), encoding="utf-8").read()
    checked = 0
    # innermost calls only, so that a nested constructor's keywords stay its own
    for name, args in re.findall(r"MCRT\.(\w+)\(([^()]*)\)", src):
        if name not in ref:  # a function (simulate), not one of the types
            continue
        for kw in re.findall(r"(?:^|[,;]\s*)([^\W\d]\w*)\s*=(?!=)", args):
            assert kw in ref[name], (name, kw)
            checked += 1
    assert checked >= 8
    assert "kl" in ref["MieScatterer"] and "layers" in ref["PlaneGeometry"]  # mie.kl, plane.layers
