"""The C# P/Invoke binding (csharp/DDLA.BLAS.Cuda/*.cs) agrees with the C ABI.

No .NET runtime exists here, so the C# sources are checked as text: every
[DllImport(Lib, EntryPoint = "...")] names a function declared in
include/ddla_gb300.h, has the same number of parameters, and each parameter's
C# type marshals to the C parameter's kind (int64 dims / strides, int32 flags
or enums, double by value, pointers to double / int32 / int64, the option and
report structs, strings, pointer arrays); the return types agree too.  The
struct layouts the binding declares (Opts, SolveReport) match the C structs
field by field.
"""
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CS_DIR = os.path.join(ROOT, "csharp", "DDLA.BLAS.Cuda")
ENUMS = {"TransType", "UpLo", "DiagType", "SideType", "ConjType"}


def _split_params(text):
    text = " ".join(text.split())
    if text.strip() in ("", "void"):
        return []
    return [p.strip() for p in text.split(",")]


def c_prototypes():
    src = open(os.path.join(ROOT, "include", "ddla_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    out = {}
    for m in re.finditer(r"^\s*((?:const\s+)?[\w]+\s*\*?)\s*(ddla_\w+)\s*\(([^;]*?)\)\s*;", src, flags=re.M):
        out[m.group(2)] = (" ".join(m.group(1).split()), _split_params(m.group(3)))
    return out


def c_kind(p):
    t = " ".join(p.replace("*", " * ").split()[:-1]) if not p.endswith("*") else p
    stars = p.count("*")
    base = re.sub(r"\bconst\b", "", p.split("*")[0]).split()
    base = base[0] if base else ""
    if stars == 0:
        if base in ("ddla_dim_t", "ddla_inc_t", "int64_t"):
            return "i64"
        if base in ("int32_t", "int"):
            return "i32"
        if base == "double":
            return "f64"
        if base == "float":
            return "f32"
        if base == "ddla_handle":
            return "ptr"
        raise AssertionError(f"unmapped C parameter {p!r} ({t})")
    if stars >= 2:
        return "pptr"
    return {"double": "pdouble", "int32_t": "pint32", "int64_t": "pint64", "char": "str" if "const" in p else "buf",
            "ddla_opts": "opts", "ddla_solve_report": "report", "ddla_contract_desc": "desc",
            "void": "ptr", "float": "pfloat", "ddla_handle": "pptr"}.get(base, "ptr")


def cs_kind(p):
    words = p.split()
    mod = words[0] if words[0] in ("in", "ref", "out") else ""
    typ = words[1] if mod else words[0]
    if typ == "IntPtr":
        return "ptr"
    if typ == "IntPtr[]":
        return "pptr"
    if mod:
        return {"double": "pdouble", "int": "pint32", "long": "pint64", "Opts": "opts", "SolveReport": "report",
                "ContractDesc": "desc"}[typ]
    return {"dim_t": "i64", "inc_t": "i64", "long": "i64", "int": "i32", "double": "f64", "float": "f32",
            "string": "str", "byte[]": "buf", "long[]": "pint64", "int[]": "pint32", "double[]": "pdouble"}.get(
        typ, "i32" if typ in ENUMS else f"?{typ}")


def cs_imports():
    out = []
    for path in glob.glob(os.path.join(CS_DIR, "*.cs")):
        src = open(path).read()
        for m in re.finditer(r'\[DllImport\(Lib, EntryPoint = "(\w+)"\)\]\s*(?:public\s+)?static\s+extern\s+'
                             r'(\w+)\s+(\w+)\(([^)]*)\);', src):
            out.append((m.group(1), m.group(2), m.group(3), _split_params(m.group(4)), os.path.basename(path)))
    return out


def test_every_dllimport_matches_a_c_prototype():
    protos = c_prototypes()
    imports = cs_imports()
    assert len(imports) >= 30
    for entry, ret, name, params, path in imports:
        assert entry in protos, f"{path}: {name} binds {entry}, which include/ddla_gb300.h does not declare"
        cret, cparams = protos[entry]
        assert len(params) == len(cparams), f"{entry}: C# has {len(params)} parameters, C has {len(cparams)}"
        want_ret = {"int": "int", "int64_t": "long", "const char *": "IntPtr", "const char*": "IntPtr"}[cret]
        assert ret == want_ret, f"{entry}: returns {ret}, C returns {cret}"
        for i, (cs, c) in enumerate(zip(params, cparams)):
            k_cs, k_c = cs_kind(cs), c_kind(c)
            ok = k_cs == k_c or (k_cs == "ptr" and k_c in ("ptr", "pdouble", "pint32", "pint64", "pfloat"))
            assert ok, f"{entry} parameter {i + 1}: C# '{cs}' ({k_cs}) vs C '{c}' ({k_c})"


def test_binding_covers_every_host_entry_point():
    # every host-pointer call of the header (no handle, no device pointers) has a binding
    protos = c_prototypes()
    bound = {e for e, *_ in cs_imports()}
    host = {n for n in protos if not n.startswith(("ddla_dev_", "ddla_handle", "ddla_batched", "ddla_timing",
                                                    "ddla_measure"))}
    missing = sorted(host - bound)
    assert not missing, f"host entry points without a C# binding: {missing}"


def _c_struct(name):
    src = open(os.path.join(ROOT, "include", "ddla_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    body = re.search(r"typedef struct " + name + r"\s*\{(.*?)\}", src, flags=re.S).group(1)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        typ, rest = decl.split(None, 1)
        fields += [(typ, f.strip()) for f in rest.split(",")]
    return fields


def _cs_struct(name):
    src = open(os.path.join(CS_DIR, "Source.cs")).read()
    body = re.search(r"public struct " + name + r"\s*\{(.*?)\n    \}", src, flags=re.S).group(1)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl or decl.startswith("//"):
            continue
        m = re.match(r"public\s+(\w+)\s+(.*)", decl)
        fields += [(m.group(1), f.strip()) for f in m.group(2).split(",")]
    return fields


def test_struct_layouts_match():
    size = {"int32_t": 4, "double": 8, "int": 4}
    for c_name, cs_name in (("ddla_opts", "Opts"), ("ddla_solve_report", "SolveReport")):
        cf, csf = _c_struct(c_name), _cs_struct(cs_name)
        assert [size[t] for t, _ in cf] == [size[t] for t, _ in csf], (c_name, cf, csf)
        # same field order: the C# names are the C names in Pascal case
        for (_, a), (_, b) in zip(cf, csf):
            assert a.replace("_", "").lower() == b.lower(), (c_name, a, b)
