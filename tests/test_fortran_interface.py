"""The Fortran ISO_C_BINDING module (fortran/oakg.F90) against the C header (include/oakg.h).

No Fortran compiler is available to build the module, so its interfaces are checked as text:
every function the header declares has a bind(C) interface of the same C name, with the same
number of arguments, the same argument names (Fortran is case-blind), the interoperable kind
of each C type, `value` exactly where C passes by value, and the matching result type; the
bind(C) derived types have the members of the C structures, in order, with matching kinds.
"""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# C scalar type -> Fortran interoperable type spelling
C2F = {"double": "real(c_double)", "float": "real(c_float)",
       "int32_t": "integer(c_int32_t)", "int64_t": "integer(c_int64_t)",
       "int": "integer(c_int)", "size_t": "integer(c_size_t)", "uint8_t": "integer(c_int8_t)",
       "char": "character(kind=c_char)", "oakg_dims": "type(oakg_dims)",
       "oakg_loc": "type(oakg_loc)", "oakg_obsoper": "type(oakg_obsoper)"}


def c_declarations():
    src = open(os.path.join(ROOT, "include", "oakg.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    out = {}
    for ret, name, params in re.findall(
            r"^\s*(int|void|size_t|int64_t)\s+((?:oak|oakg)_\w+)\s*\(([^)]*)\)\s*;", src,
            flags=re.M):
        plist = []
        p = " ".join(params.split())
        if p not in ("", "void"):
            for item in p.split(","):
                item = item.strip().replace("const ", "")
                m = re.match(r"([\w]+)\s*(\**)\s*(\w+)$", item)
                assert m, item
                plist.append((m.group(1), len(m.group(2)), m.group(3)))
        out[name] = (ret, plist)
    return out


def c_structs():
    src = open(os.path.join(ROOT, "include", "oakg.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    out = {}
    for body, name in re.findall(r"typedef struct\s*\w*\s*\{(.*?)\}\s*(\w+)\s*;", src, flags=re.S):
        members = []
        for decl in body.split(";"):
            decl = " ".join(decl.split()).replace("const ", "")
            if not decl:
                continue
            m = re.match(r"(\w+)\s*(\**)\s*(.+)$", decl)
            for nm in m.group(3).split(","):
                members.append((m.group(1), len(m.group(2)) + nm.count("*")))
        out[name] = members
    return out


def fortran_source():
    src = open(os.path.join(ROOT, "fortran", "oakg.F90")).read()
    src = "\n".join(ln.split("!")[0] if '"' not in ln and "'" not in ln else ln
                    for ln in src.splitlines())
    return re.sub(r"&\s*\n\s*&?", " ", src)


def fortran_interfaces():
    src = fortran_source()
    body = src[src.index("\n  interface"):src.index("end interface")]
    out = {}
    for blk in re.finditer(
            r"(?:(integer\(c_\w+\))\s+)?(function|subroutine)\s+(\w+)\s*\(([^)]*)\)\s*"
            r"bind\(C,\s*name=\"(\w+)\"\)(.*?)end (?:function|subroutine)", body, flags=re.S):
        ftype, kind, _, args, cname, decls = blk.groups()
        names = [a.strip().lower() for a in args.split(",") if a.strip()]
        info = {}
        for ln in decls.splitlines():
            if "::" not in ln:
                continue
            spec, vars_ = ln.split("::")
            parts = [s.strip().lower() for s in re.split(r",(?![^()]*\))", spec)]
            typ, attrs = parts[0].replace(" ", ""), parts[1:]
            for v in re.split(r",(?![^()]*\))", vars_):
                v = v.strip().lower()
                nm = re.match(r"(\w+)", v).group(1)
                info[nm] = (typ, "value" in attrs, "(" in v)
        out[cname] = (ftype, kind, names, info)
    return out


def fortran_types():
    src = fortran_source()
    out = {}
    for name, body in re.findall(r"type, bind\(C\) :: (\w+)(.*?)end type", src, flags=re.S):
        members = []
        for ln in body.splitlines():
            if "::" in ln:
                typ = ln.split("::")[0].strip().lower().replace(" ", "")
                for _ in ln.split("::")[1].split("=")[0].split(","):
                    members.append(typ)
        out[name] = members
    return out


def expected_fortran(ctype, stars):
    """(type, value?) the Fortran dummy must have for a C parameter."""
    if ctype == "void":
        return "type(c_ptr)", True
    if ctype == "oakg_plan":
        return "type(c_ptr)", stars == 1
    return C2F[ctype], stars == 0


def test_every_header_function_has_an_interface():
    c = c_declarations()
    f = fortran_interfaces()
    assert len(c) >= 35
    missing = sorted(set(c) - set(f))
    assert not missing, f"no bind(C) interface for {missing}"
    extra = sorted(set(f) - set(c))
    assert not extra, f"interfaces without a header declaration: {extra}"


def test_arguments_kinds_and_passing():
    c = c_declarations()
    f = fortran_interfaces()
    bad = []
    for name, (ret, params) in c.items():
        ftype, kind, fnames, info = f[name]
        if [p[2].lower() for p in params] != fnames:
            bad.append((name, "names/arity", [p[2] for p in params], fnames))
            continue
        for (ctype, stars, pname) in params:
            typ, value, _ = info[pname.lower()]
            exp_t, exp_v = expected_fortran(ctype, stars)
            if typ != exp_t or value != exp_v:
                bad.append((name, pname, (typ, value), (exp_t, exp_v)))
        if ret == "void":
            ok = kind == "subroutine"
        else:
            ok = kind == "function" and ftype == C2F[ret]
        if not ok:
            bad.append((name, "result", ret, (ftype, kind)))
    assert not bad, bad


def test_struct_layouts():
    cs = c_structs()
    ft = fortran_types()
    for name in ("oakg_dims", "oakg_loc", "oakg_obsoper"):
        cm = cs[name]
        fm = ft[name]
        assert len(cm) == len(fm), name
        for (ctype, stars), ftyp in zip(cm, fm):
            exp = "type(c_ptr)" if stars else C2F[ctype]
            assert ftyp == exp, (name, ctype, ftyp)


def test_wrappers_keep_the_reference_argument_lists():
    """gpu_analysis / gpu_locAnalysis take the arguments of analysis (rrsqrt.F90:196) and
    locAnalysis (rrsqrt.F90:433-434) in the same order, selectObservations replaced by the
    geometry."""
    src = fortran_source()
    a = re.search(r"subroutine gpu_analysis\(([^)]*)\)", src).group(1)
    assert [x.strip() for x in a.split(",")] == ["xf", "Hxf", "yo", "Sf", "HSf", "R", "xa", "Sa",
                                                 "amplitudes"]
    la = re.search(r"subroutine gpu_locAnalysis\(([^)]*)\)", src).group(1)
    assert [x.strip() for x in la.split(",")] == ["zoneSize", "geometry", "xf", "Hxf", "yo",
                                                  "Sf", "HSf", "R", "xa", "Sa", "amplitudes",
                                                  "localise_obs"]
    la4 = re.search(r"subroutine gpu_locAnalysis_r4\(([^)]*)\)", src).group(1)
    assert la4.split() == la.split()
    assert "subroutine gpu_locAnalysis_adjoint" in src
