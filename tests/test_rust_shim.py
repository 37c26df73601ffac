"""The Rust binding (fock-gb300-sys/) against the C header, by parsing both:
every C struct has a #[repr(C)] struct with the same fields in the same order
and the same C types; every function has an extern "C" declaration with the
same argument types and return type; every #define constant has a pub const of
the same value.  (No Rust toolchain exists on the build machines, so the crate
is checked this way instead of being compiled.)  No GPU needed."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "fock_gb300.h")
RUST = os.path.join(ROOT, "fock-gb300-sys", "src", "lib.rs")

C2R = {"double": "c_double", "int": "c_int", "long long": "c_longlong", "float": "c_float", "char": "c_char",
       "void": "c_void"}


def _strip_c(text):
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    return re.sub(r"//[^\n]*", " ", text)


def _c_type(t):
    """'const double*' -> '*const c_double', 'fock_ctx**' -> '*mut *mut fock_ctx'."""
    t = " ".join(t.replace("*", " * ").split())
    stars = t.count("*")
    base = t.replace("*", "").strip()
    const = base.startswith("const ")
    base = base.replace("const ", "").strip()
    r = C2R.get(base, base)
    for k in range(stars):
        # the const qualifies the pointee (outermost pointer in Rust's order)
        r = ("*const " if (const and k == 0) else "*mut ") + r
    return r


def _split_decl(decl):
    """'double x, y, z' -> [('double', 'x'), ...]; 'const double* exps' -> [('const double*', 'exps')]."""
    decl = " ".join(decl.split())
    first = re.match(r"^(.+?[\s*])(\w+)\s*((?:,\s*\w+\s*)*)$", decl)
    assert first, decl
    typ, name, rest = first.group(1).strip(), first.group(2), first.group(3)
    names = [name] + [n.strip() for n in rest.split(",") if n.strip()]
    return [(typ, n) for n in names]


def header_structs():
    text = _strip_c(open(HEADER).read())
    out = {}
    for body, name in re.findall(r"typedef struct\s*\{(.*?)\}\s*(\w+)\s*;", text, flags=re.S):
        fields = []
        for decl in body.split(";"):
            if decl.strip():
                fields += [(n, _c_type(t)) for t, n in _split_decl(decl)]
        out[name] = fields
    return out


def header_functions():
    text = " ".join(_strip_c(open(HEADER).read()).split())
    out = {}
    for ret, name, args in re.findall(r"((?:const\s+)?(?:long long|int|void|char)\s*\**)\s*(fock_\w+)\s*\(([^)]*)\)\s*;",
                                      text):
        params = []
        for a in args.split(","):
            a = a.strip()
            if not a or a == "void":
                continue
            m = re.match(r"^(.*?)(\w+)$", a)
            params.append(_c_type(m.group(1)))
        r = _c_type(ret)
        out[name] = (None if r == "c_void" else r, params)
    return out


def header_constants():
    text = open(HEADER).read()
    return {k: int(v) for k, v in re.findall(r"#define\s+(FOCK_\w+)\s+\(?(-?\d+)\)?", text)}


def rust_text():
    return re.sub(r"//[^\n]*", " ", open(RUST).read())


def rust_structs():
    out = {}
    for name, body in re.findall(r"#\[repr\(C\)\][^{]*?pub struct (\w+)\s*\{(.*?)\}", rust_text(), flags=re.S):
        fields = [(n, " ".join(t.split())) for n, t in re.findall(r"pub (\w+):\s*([^,]+),", body)]
        out[name] = fields
    return out


def rust_functions():
    block = re.search(r'extern "C"\s*\{(.*)\}', rust_text(), flags=re.S).group(1)
    out = {}
    for name, args, ret in re.findall(r"pub fn (\w+)\((.*?)\)\s*(?:->\s*([^;]+))?;", block, flags=re.S):
        params = [" ".join(t.split()) for _, t in re.findall(r"(\w+):\s*([^,]+)", args)]
        out[name] = (" ".join(ret.split()) if ret else None, params)
    return out


def rust_constants():
    return {k: int(v) for k, v in re.findall(r"pub const (FOCK_\w+): c_int = (-?\d+);", rust_text())}


def test_structs_match_header():
    h, r = header_structs(), rust_structs()
    assert set(h) <= set(r), set(h) - set(r)
    for name, fields in h.items():
        assert r[name] == fields, (name, fields, r[name])


def test_functions_match_header():
    h, r = header_functions(), rust_functions()
    assert len(h) > 30
    assert set(h) == set(r), (set(h) ^ set(r))
    for name, sig in h.items():
        assert r[name] == sig, (name, sig, r[name])


def test_constants_match_header():
    h, r = header_constants(), rust_constants()
    assert h == r, set(h.items()) ^ set(r.items())
