"""The Rust binding crate (bindings/rust) against the C header, on the CPU.

No Rust toolchain is available to build the crate, so these tests check
what can be checked from its source: every entry point of
include/bendy2d.h is declared in src/ffi.rs with the same parameter and
return types, the #[repr(C)] structs have the C structs' fields in the same
order, the status and flag constants agree, and the crate root declares the
reference crate's six modules (src/lib.rs:1-6)."""
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "bendy2d.h"
CRATE = ROOT / "bindings" / "rust"

C_SCALARS = {
    "float": "f32", "double": "c_double", "int": "c_int", "char": "c_char", "void": "c_void",
    "uint32_t": "u32", "uint64_t": "u64", "size_t": "usize",
}


def c_header():
    text = HEADER.read_text()
    return re.sub(r"/\*.*?\*/", "", text, flags=re.S)


def c_type_to_rust(t: str) -> str:
    """'const b2d_circle*' -> '*const b2d_circle', 'b2d_solver**' -> '*mut *mut b2d_solver'."""
    t = t.strip()
    const = t.startswith("const ")
    if const:
        t = t[len("const "):].strip()
    stars = t.count("*")
    base = t.replace("*", "").strip()
    r = C_SCALARS.get(base, base)
    for k in range(stars):
        # the outermost pointer carries the const of the pointee only at depth 1
        r = ("*const " if (const and k == 0) else "*mut ") + r
    return r


def c_functions():
    out = {}
    for m in re.finditer(r"^\s*(const char\*|int)\s+(b2d_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", c_header(),
                         flags=re.M | re.S):
        ret, name, params = m.group(1), m.group(2), " ".join(m.group(3).split())
        types = []
        if params and params != "void":
            for p in params.split(","):
                p = p.strip()
                mm = re.match(r"(.*?)([A-Za-z_][A-Za-z0-9_]*)$", p)
                types.append(c_type_to_rust(mm.group(1)))
        out[name] = (c_type_to_rust(ret), types)
    return out


def rust_functions():
    text = (CRATE / "src" / "ffi.rs").read_text()
    block = text[text.index('extern "C" {'):]
    out = {}
    for m in re.finditer(r"pub fn (b2d_[a-z0-9_]+)\s*\(([^)]*)\)\s*->\s*([^;]+);", block, flags=re.S):
        name, params, ret = m.group(1), " ".join(m.group(2).split()), m.group(3).strip()
        types = []
        for p in [x for x in params.split(",") if x.strip()]:
            types.append(p.split(":", 1)[1].strip())
        out[name] = (ret, types)
    return out


def test_ffi_declares_every_entry_point_with_c_types():
    c, r = c_functions(), rust_functions()
    assert len(c) > 70
    assert sorted(c) == sorted(r), (sorted(set(c) - set(r)), sorted(set(r) - set(c)))
    bad = {k: (c[k], r[k]) for k in c if c[k] != r[k]}
    assert not bad, bad


def c_structs():
    out = {}
    for m in re.finditer(r"typedef struct\s*\{(.*?)\}\s*(b2d_[a-z0-9_]+)\s*;", c_header(), flags=re.S):
        fields = []
        for decl in m.group(1).split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            mm = re.match(r"((?:const )?[A-Za-z_0-9]+\*?)\s+(.*)$", decl)
            fields += [f.strip() for f in mm.group(2).split(",")]
        out[m.group(2)] = fields
    return out


def rust_structs():
    text = (CRATE / "src" / "ffi.rs").read_text()
    out = {}
    for m in re.finditer(r"#\[repr\(C\)\][^{]*?pub struct (b2d_[a-z0-9_]+)\s*\{(.*?)\}", text, flags=re.S):
        fields = re.findall(r"pub ([a-z_0-9]+)\s*:", m.group(2))
        if fields:
            out[m.group(1)] = fields
    return out


def test_repr_c_structs_match_the_header():
    c, r = c_structs(), rust_structs()
    assert set(c) == set(r), (set(c) ^ set(r))
    for k in c:
        assert c[k] == r[k], (k, c[k], r[k])


def test_constants_match_the_header():
    text = HEADER.read_text()
    c = {m.group(1): int(m.group(2)) for m in
         re.finditer(r"#define (B2D_[A-Z_]+)\s+(\d+)u?\b", text)}
    rs = (CRATE / "src" / "ffi.rs").read_text()
    r = {m.group(1): int(m.group(2)) for m in
         re.finditer(r"pub const (B2D_[A-Z_]+):\s*[a-z_0-9]+\s*=\s*(\d+);", rs)}
    assert len(c) >= 20
    assert c == r


def test_crate_mirrors_the_reference_modules():
    lib = (CRATE / "src" / "lib.rs").read_text()
    mods = re.findall(r"^pub mod ([a-z_]+);", lib, flags=re.M)
    for m in ("circle", "common", "link", "particle", "polygon", "solver"):
        assert m in mods
        assert (CRATE / "src" / f"{m}.rs").is_file()
    cargo = (CRATE / "Cargo.toml").read_text()
    assert 'name = "bendy2d"' in cargo and "nalgebra" in cargo


def test_solver_methods_of_the_reference_are_bound():
    """Solver's public methods, src/solver.rs:34-116."""
    src = (CRATE / "src" / "solver.rs").read_text()
    for f in ("new", "add_particle", "add_circle", "add_polygon", "add_particle_link",
              "add_circle_link", "get_particle_len", "get_circles_len", "get_polygons_len",
              "get_particle_links", "get_circle_links", "get_particles", "get_circles",
              "get_polygons", "get_particle", "get_circle", "get_polygon", "update"):
        assert re.search(rf"pub fn {f}\(", src), f
    for field in ("gravity", "bounds", "bounds_active"):
        assert re.search(rf"pub {field}:", src), field


def test_value_type_methods_of_the_reference_are_bound():
    """The public methods of the reference's value types and its free
    functions: src/particle.rs:11-59, src/circle.rs:10-45, src/link.rs:17-48,
    src/polygon.rs:16-229, src/common.rs:3-26."""
    expect = {
        "particle.rs": ["new", "update", "solve_bounds", "add_force", "add_force_v2",
                        "add_force_towards"],
        "circle.rs": ["solve_bounds", "solve_circle"],
        "link.rs": ["solve"],
        "polygon.rs": ["circle", "new", "update", "solve_bounds", "solve_polygon",
                       "solve_polygon_single", "solve_links", "add_force_v2"],
        "common.rs": ["line_intersection"],
    }
    for f, names in expect.items():
        src = (CRATE / "src" / f).read_text()
        for n in names:
            assert re.search(rf"pub fn {n}\(", src), (f, n)
    link = (CRATE / "src" / "link.rs").read_text()
    assert link.count("pub fn solve(") == 2  # ParticleLink and CircleLink
    for ty, fields in (("particle.rs", ["pos", "prev_pos"]), ("circle.rs", ["point", "radius"]),
                       ("link.rs", ["particle_a", "particle_b", "target_distance", "link"]),
                       ("polygon.rs", ["particles", "particle_links", "is_static", "center",
                                       "scale"])):
        src = (CRATE / "src" / ty).read_text()
        for fl in fields:
            assert re.search(rf"pub {fl}:", src), (ty, fl)
