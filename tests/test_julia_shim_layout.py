"""The Julia ccall shim mirrors include/gpdhg.h's structs by hand; this text-level test
parses both and checks that every mirrored struct has the same fields, in the same order,
with types of the same width (Julia cannot run here, so the layouts are compared as text)."""
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "gpdhg.h")
SHIM = os.path.join(REPO, "cupdlp.jl_gb300", "julia", "GpdhgShim.jl")

# Julia struct name -> C typedef name
PAIRS = {
    "GpdhgParams": "gpdhg_params",
    "GpdhgConvergenceInformation": "gpdhg_convergence_information",
    "GpdhgInfeasibilityInformation": "gpdhg_infeasibility_information",
    "GpdhgIterationStats": "gpdhg_iteration_stats",
    "GpdhgResult": "gpdhg_result",
    "GpdhgLpDesc": "gpdhg_lp_desc",
    "GpdhgTwoSidedDesc": "gpdhg_two_sided_desc",
}

C_TYPES = {"int32_t": "i32", "int": "i32", "int64_t": "i64", "double": "f64", "float": "f32"}
JL_TYPES = {"Int32": "i32", "Int64": "i64", "Float64": "f64", "Float32": "f32", "Cint": "i32",
            "Clonglong": "i64", "Cdouble": "f64"}


def c_structs():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    out = {}
    for m in re.finditer(r"typedef struct (\w+) \{(.*?)\}\s*(\w+);", text, flags=re.S):
        fields = []
        for decl in m.group(2).split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            dm = re.fullmatch(r"(?:const )?(\w+)\s*(\**)\s*(?:const )?(\w+)(?:\[(\d+)\])?", decl)
            assert dm, f"unparsed C declaration in {m.group(3)}: {decl!r}"
            base, stars, name, count = dm.groups()
            t = "ptr" if stars else C_TYPES.get(base, base)
            if count:
                t = f"{t}[{count}]"
            fields.append((name, t))
        out[m.group(3)] = fields
    return out


def julia_structs():
    text = open(SHIM).read()
    out = {}
    for m in re.finditer(r"^struct (\w+)\n(.*?)^end", text, flags=re.S | re.M):
        fields = []
        for line in m.group(2).splitlines():
            line = line.split("#")[0].strip()
            if not line:
                continue
            fm = re.fullmatch(r"(\w+)::(.+)", line)
            assert fm, f"unparsed Julia field in {m.group(1)}: {line!r}"
            name, jt = fm.groups()
            tm = re.fullmatch(r"NTuple\{(\d+),\s*(\w+)\}", jt)
            if jt.startswith("Ptr{"):
                t = "ptr"
            elif tm:
                t = f"{JL_TYPES[tm.group(2)]}[{tm.group(1)}]"
            else:
                t = JL_TYPES.get(jt, jt)
            fields.append((name, t))
        out[m.group(1)] = fields
    return out


def test_every_mirrored_struct_matches_the_header():
    cs, js = c_structs(), julia_structs()
    for jname, cname in PAIRS.items():
        assert jname in js, f"{jname} missing from the shim"
        assert cname in cs, f"{cname} missing from the header"
        jf = [(n, PAIRS.get(t, t)) for n, t in js[jname]]
        assert jf == cs[cname], f"{jname} differs from {cname}"


def test_shim_mirrors_every_plain_header_struct():
    cs = c_structs()
    mirrored = set(PAIRS.values())
    # the server configuration is the only struct the shim does not need
    for name in sorted(set(cs) - mirrored):
        assert name.startswith("gpdhg_server"), f"{name} has no Julia mirror"


@pytest.mark.parametrize("planted", ["rename", "retype", "drop"])
def test_the_comparison_catches_a_planted_mismatch(planted):
    cs, js = c_structs(), julia_structs()
    fields = [(n, PAIRS.get(t, t)) for n, t in js["GpdhgResult"]]
    assert fields == cs["gpdhg_result"]
    if planted == "rename":
        fields[1] = ("iterations", fields[1][1])
    elif planted == "retype":
        fields[2] = (fields[2][0], "i32")
    else:
        del fields[3]
    assert fields != cs["gpdhg_result"]
