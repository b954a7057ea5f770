"""The C-ABI library: loads, exports exactly what include/sr.h declares, and
its host-side argument checking (no GPU work is launched here)."""
import ctypes as C
import os
import re

import pytest

import softrender._lib as L
from softrender import _abi as A

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if not f.endswith(".h"):
            continue
        txt = open(os.path.join(ROOT, "include", f)).read()
        names |= set(re.findall(r"SR_API\s+[\w\s\*]+?\b(sr_\w+)\s*\(", txt))
    return names


def test_header_declares_entry_points():
    names = declared_symbols()
    for must in ("sr_pipeline_create", "sr_render", "sr_sync", "sr_mesh_upload", "sr_shader_lookup",
                 "sr_framebuffer_read", "sr_texture_upload"):
        assert must in names


def test_library_exports_every_declared_symbol(built_lib):
    lib = L.lib()
    missing = [n for n in sorted(declared_symbols()) if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header(built_lib):
    assert declared_symbols() <= set(L.SIGNATURES), declared_symbols() - set(L.SIGNATURES)


def test_only_declared_symbols_are_exported(built_lib):
    import subprocess
    out = subprocess.run(["nm", "-D", "--defined-only", built_lib], capture_output=True, text=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if " T " in l and l.split()[-1].startswith("sr_")}
    assert exported == declared_symbols(), exported ^ declared_symbols()


def test_shader_registry(built_lib):
    lib = L.lib()
    i = C.c_int()
    for name, stage in [("mvp_pos_nrm", A.SR_STAGE_VERTEX), ("mvp_pos_nrm_uv", A.SR_STAGE_VERTEX),
                        ("clip_rgba8", A.SR_STAGE_VERTEX), ("clip", A.SR_STAGE_GEOMETRY),
                        ("blinn_phong_dir", A.SR_STAGE_FRAGMENT), ("textured_blinn_phong", A.SR_STAGE_FRAGMENT),
                        ("over", A.SR_STAGE_BLEND), ("replace", A.SR_STAGE_BLEND)]:
        assert lib.sr_shader_lookup(name.encode(), stage, C.byref(i)) == A.SR_OK
    assert lib.sr_shader_lookup(b"no_such_shader", A.SR_STAGE_FRAGMENT, C.byref(i)) == A.SR_ENOTFOUND
    assert lib.sr_shader_lookup(b"over", A.SR_STAGE_VERTEX, C.byref(i)) == A.SR_ENOTFOUND


def test_status_strings_and_version(built_lib):
    lib = L.lib()
    assert lib.sr_status_string(A.SR_ENAN) == b"SR_ENAN"
    assert lib.sr_version().startswith(b"softrender-gb300")


def test_draw_defaults(built_lib):
    d = A.SrDraw()
    L.lib().sr_draw_init(C.byref(d))
    assert (d.tile_w, d.tile_h) == (128, 128)          # DEFAULT_TILE_SIZE (fragment.rs:29)
    assert d.prim == A.SR_PRIM_TRIANGLE and d.blend == 0 and d.cull == A.SR_CULL_NONE


def test_invalid_arguments_rejected_on_host(built_lib):
    lib = L.lib()
    h = C.c_void_p()
    bad = A.SrFbDesc(0, 10, A.SR_COLOR_RGBA8, 1, 0)         # mod.rs:129: non-zero width
    assert lib.sr_pipeline_create(C.byref(bad), None, 0, C.byref(h)) == A.SR_EINVAL
    bad = A.SrFbDesc(10, 0, A.SR_COLOR_RGBA8, 1, 0)
    assert lib.sr_pipeline_create(C.byref(bad), None, 0, C.byref(h)) == A.SR_EINVAL
    assert lib.sr_render(None, None) == A.SR_EINVAL
    assert lib.sr_shader_lookup(None, 0, C.byref(C.c_int())) == A.SR_EINVAL
    # indices out of range are rejected before any device work
    import numpy as np
    plane = np.zeros(3, dtype=np.float32)
    idx = np.array([0, 1, 5], dtype=np.uint32)
    arr = (C.c_void_p * 1)(plane.ctypes.data)
    assert lib.sr_mesh_upload(arr, 1, 3, idx.ctypes.data, 3, C.byref(h)) == A.SR_EINVAL
    # more vertices than u32 vertex references leave room for (checked before any copy)
    assert lib.sr_mesh_upload(None, 0, (1 << 31) + 1, None, 0, C.byref(h)) == A.SR_EINVAL
    assert h.value is None


# ---------------------------------------------------------------- the Rust binding shown to integrators
_C2RUST = {"uint32_t": "u32", "int32_t": "i32", "uint64_t": "u64", "uint8_t": "u8", "float": "f32",
           "double": "f64", "size_t": "usize", "int": "c_int", "char": "c_char", "void": "c_void"}


def _rust_type(c_decl):
    """The Rust spelling of a C type: `const float* const*` -> `*const *const f32`.
    A `const` before a `*` qualifies what that `*` points to."""
    toks = re.findall(r"\w+|\*", c_decl)
    base, pointee_const, levels = None, False, []
    for t in toks:
        if t == "const":
            pointee_const = True
        elif t == "*":
            levels.append(pointee_const)
            pointee_const = False
        else:
            base = t
    ty = _C2RUST.get(base, base)
    for c in levels:
        ty = ("*const " if c else "*mut ") + ty
    return ty


def _header_text():
    txt = open(os.path.join(ROOT, "include", "sr.h")).read()
    return re.sub(r"/\*.*?\*/", "", txt, flags=re.S)


def _rust_block():
    """The declarations of the Rust -sys crate (ffi/softrender-cuda-sys)."""
    return open(os.path.join(ROOT, "ffi", "softrender-cuda-sys", "src", "lib.rs")).read()


def test_rust_binding_functions_match_header():
    hdr, rust = _header_text(), _rust_block()
    want = {}
    for ret, name, args in re.findall(r"SR_API\s+([\w\s\*]+?)\b(sr_\w+)\s*\(([^)]*)\)\s*;", hdr):
        params = [] if args.strip() in ("", "void") else args.split(",")
        # drop the parameter name, keep its type
        types = [_rust_type(re.sub(r"\b\w+\s*$", "", p)) for p in params]
        r = _rust_type(ret).strip()
        want[name] = (types, None if r == "c_void" else r)
    got = {}
    for name, args, ret in re.findall(r"pub fn (sr_\w+)\(([^)]*)\)\s*(?:->\s*([^;]+))?;", rust):
        types = [" ".join(a.split(":", 1)[1].split()) for a in args.split(",") if a.strip()]
        got[name] = (types, ret.strip() if ret else None)
    assert set(got) == set(want), set(got) ^ set(want)
    bad = {n: (want[n], got[n]) for n in want if want[n] != got[n]}
    assert not bad, bad


def test_rust_binding_structs_match_header():
    hdr, rust = _header_text(), _rust_block()
    rust_structs = {n: [(f, " ".join(t.split())) for f, t in re.findall(r"pub (\w+): ([^,]+)", body)]
                    for n, body in re.findall(r"pub struct (sr_\w+) \{(.*?)\}", rust, flags=re.S)}
    checked = 0
    for body, name in re.findall(r"typedef struct \w+ \{(.*?)\} (sr_\w+);", hdr, flags=re.S):
        fields = []
        for decl in (d.strip() for d in body.split(";")):
            if not decl:
                continue
            m = re.match(r"((?:const\s+)?\w+\s*\**)\s*(.*)$", decl, flags=re.S)
            for item in m.group(2).split(","):
                item = item.strip()
                arr = re.match(r"(\w+)\[(\d+)\]", item)
                ty = _rust_type(m.group(1))
                fields.append((arr.group(1), f"[{ty}; {arr.group(2)}]") if arr else (item, ty))
        assert name in rust_structs, name
        assert rust_structs[name] == fields, (name, rust_structs[name], fields)
        checked += 1
    assert checked >= 8


def test_ctypes_struct_layouts_match_header(tmp_path):
    """Every ctypes structure of softrender._abi has the size, and each of its
    fields the offset, that a C++ compiler gives the struct of include/sr.h /
    include/sr_shaders.h of the same name (a mismatch would corrupt every call
    that passes the struct).  Host compiler only, no GPU."""
    import shutil
    import subprocess
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    classes = {"sr_uniforms": A.SrUniforms, "sr_fb_desc": A.SrFbDesc, "sr_viewport": A.SrViewport,
               "sr_draw": A.SrDraw, "sr_stats": A.SrStats, "sr_batch_item": A.SrBatchItem,
               "sr_server_config": A.SrServerConfig, "sr_request": A.SrRequest,
               "sr_server_stats": A.SrServerStats}
    lines = ["#include <cstddef>", "#include <cstdio>", '#include "sr.h"', '#include "sr_shaders.h"',
             "int main() {"]
    want = []
    for cname, cls in classes.items():
        lines.append(f'    std::printf("{cname} %zu\\n", sizeof({cname}));')
        want.append(f"{cname} {C.sizeof(cls)}")
        for fname, _ in cls._fields_:
            lines.append(f'    std::printf("{cname}.{fname} %zu\\n", offsetof({cname}, {fname}));')
            want.append(f"{cname}.{fname} {getattr(cls, fname).offset}")
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.cpp"
    src.write_text("\n".join(lines) + "\n")
    exe = str(tmp_path / "layout")
    subprocess.check_call(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), str(src), "-o", exe])
    got = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    assert [g for g in got if g] == want


def test_header_is_plain_c_and_links(built_lib, tmp_path):
    """include/sr.h is a C header (the C ABI a Rust `-sys` crate, cgo or any
    C caller binds): a C99 program compiles against it with -pedantic
    -Werror, links against the library and calls its host-only entry points."""
    import shutil
    import subprocess
    if not shutil.which("gcc"):
        pytest.skip("gcc not available")
    src = tmp_path / "c_abi.c"
    src.write_text(
        '#include <stdio.h>\n#include "sr.h"\n'
        "int main(void) {\n"
        "    sr_draw d;\n"
        "    sr_draw_init(&d);\n"
        '    printf("%s|%u|%u|%s\\n", sr_version(), d.tile_w, d.tile_h, sr_status_string(SR_ENAN));\n'
        "    return 0;\n"
        "}\n")
    exe = str(tmp_path / "c_abi")
    libdir = os.path.dirname(built_lib)
    subprocess.check_call(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic",
                           "-I", os.path.join(ROOT, "include"), str(src), "-o", exe,
                           "-L", libdir, "-lsoftrender_gb300", "-Wl,-rpath," + libdir])
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.strip()
    version, tw, th, name = out.split("|")
    assert version.startswith("softrender-gb300") and (tw, th) == ("128", "128") and name == "SR_ENAN"
