"""The Rust binding written out in INTEGRATION.md agrees with include/quaru_gpu.h: every declared
function exists with the same number of parameters, the #[repr(C)] structs list the header's fields
in the header's order, and the constants have the header's values."""
from __future__ import annotations

import re
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def _header() -> str:
    text = (ROOT / "include" / "quaru_gpu.h").read_text()
    return re.sub(r"/\*.*?\*/", " ", text, flags=re.S)


def _rust_blocks() -> str:
    doc = (ROOT / "INTEGRATION.md").read_text()
    blocks = re.findall(r"```rust\n(.*?)```", doc, flags=re.S)
    assert blocks, "INTEGRATION.md holds no Rust block"
    return "\n".join(re.sub(r"//[^\n]*", "", b) for b in blocks)


def _nparams(args: str) -> int:
    args = args.strip()
    return 0 if args in ("", "void") else args.count(",") + 1


def _header_functions() -> dict:
    return {name: _nparams(args) for name, args in re.findall(r"\b(qs_\w+)\s*\(([^;{()]*)\)\s*;", _header())}


def test_rust_extern_functions_match_the_header():
    rust = _rust_blocks()
    externs = re.findall(r"extern \"C\" \{(.*?)\n\}", rust, flags=re.S)
    assert externs
    decls = re.findall(r"pub fn (qs_\w+)\(([^)]*)\)", "\n".join(externs), flags=re.S)
    assert len(decls) >= 15
    header = _header_functions()
    for name, args in decls:
        assert name in header, f"{name} is not declared in quaru_gpu.h"
        assert _nparams(args) == header[name], f"{name}: {_nparams(args)} parameters, header {header[name]}"


def test_rust_structs_match_the_header():
    rust = _rust_blocks()
    header = _header()
    structs = re.findall(r"#\[repr\(C\)\]\s*pub struct (qs_\w+) \{(.*?)\}", rust, flags=re.S)
    assert structs
    for name, body in structs:
        rust_fields = re.findall(r"pub (\w+):", body)
        if not rust_fields:  # opaque handle
            assert re.search(rf"typedef struct {name} {name};", header), name
            continue
        m = re.search(rf"typedef struct {name} \{{(.*?)\}} {name};", header, flags=re.S)
        assert m, f"{name} is not a struct of quaru_gpu.h"
        c_fields = [re.findall(r"(\w+)\s*$", f.strip())[0] for f in m.group(1).split(";") if f.strip()]
        assert rust_fields == c_fields, name


def test_rust_constants_match_the_header():
    rust = _rust_blocks()
    defines = dict(re.findall(r"#define (QS_\w+) (-?\d+)", _header()))
    consts = re.findall(r"pub const (QS_\w+): \w+ = (-?\d+);", rust)
    assert consts
    for name, value in consts:
        assert defines.get(name) == value, name
