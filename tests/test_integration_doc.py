"""The C# binding of the repository's integration guide against include/sst.h: every entry point
the header declares has exactly one LibraryImport, with the same name, the same number of arguments
and matching types (the C# side cannot be compiled here; this is the check that it binds what the
library exports)."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GUIDE = os.path.join(ROOT, "INTEGRATION.md")

# C# parameter type -> canonical type
CS = {
    "nint": "handle", "out nint": "handle*", "int": "i32", "uint": "u32", "float": "f32", "nuint": "usize",
    "int*": "i32*", "out int": "i32*", "uint*": "u32*", "float*": "f32*", "float**": "f32**", "double*": "f64*", "long*": "i64*",
    "byte*": "char*",
    "GenericMaterial*": "SstGenericMaterial*", "Ray*": "SstRay*", "Hit*": "SstHit*", "PathTracerParams*": "SstPathTracerParams*",
    "RenderStats*": "SstRenderStats*", "Tuning*": "SstTuning*", "FilmLayers*": "SstFilmLayers*", "RenderJob*": "SstRenderJob*",
    "Gradients*": "SstGradients*", "PathVertex*": "SstPathVertex*",
}


def c_canonical(param):
    p = " ".join(param.replace("const", " ").split())
    p = re.sub(r"\*\s+\*", "**", p)  # "float* * x" (from "float* const* x") -> "float** x"
    array = re.search(r"\[\d+\]$", p) is not None
    p = re.sub(r"\[\d+\]$", "", p)
    m = re.match(r"^(\w+)\s*(\**)\s*(\w+)$", p)
    assert m, param
    base, stars = m.group(1), m.group(2) + ("*" if array else "")
    base = {"int32_t": "i32", "uint32_t": "u32", "int64_t": "i64", "float": "f32", "double": "f64", "size_t": "usize", "char": "char"}.get(base, base)
    if base in ("sst_ctx", "sst_scene"):
        return "handle" + stars[1:]
    return base + stars


def header_signatures():
    text = re.sub(r"/\*.*?\*/", "", open(os.path.join(ROOT, "include", "sst.h")).read(), flags=re.S)
    out = {}
    for m in re.finditer(r"^int\s+(sst_\w+)\s*\((.*?)\);", text, flags=re.M | re.S):
        out[m.group(1)] = [c_canonical(a) for a in " ".join(m.group(2).split()).split(",")]
    return out


def csharp_signatures():
    text = open(GUIDE).read()
    out = {}
    for m in re.finditer(r"\[LibraryImport\(Lib\)\] public static partial int (sst_\w+)\((.*?)\);", text):
        name = m.group(1)
        assert name not in out, f"{name} is imported twice"
        args = []
        for a in m.group(2).split(","):
            words = a.split()
            t = " ".join(words[:-1])  # drop the parameter name
            assert t in CS, (name, a)
            args.append(CS[t])
        out[name] = args
    return out


def test_every_entry_point_has_one_library_import():
    assert set(csharp_signatures()) == set(header_signatures())


def test_library_import_signatures_match_the_header():
    cs, c = csharp_signatures(), header_signatures()
    for name, args in c.items():
        assert cs[name] == args, (name, cs[name], args)


def test_binding_uses_no_setter_the_reference_lacks():
    """FrameBuffer.Image has a private setter and no SetImage in the reference
    (Images/FrameBuffer.cs:25); the binding writes pixels through the image's indexer."""
    text = open(GUIDE).read()
    assert "SetImage(" not in text and "AddMaterial(" not in text
