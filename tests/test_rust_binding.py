"""The Rust binding (rust/quantr-gpu/src/ffi.rs) against the C ABI (include/qgpu.h), on the host:
no Rust toolchain exists here, so the declarations are parsed and compared instead of compiled.

* every function of qgpu.h is declared in the extern block and nothing else is, with the same
  parameter count and, parameter by parameter, the same pointer-ness and scalar width;
* the #[repr(C)] structs have the C structs' fields in the same order with the same offsets and
  size (C layout rules, which repr(C) follows), and QgpuOp matches the ctypes record (80 bytes);
* the status, precision, mode and gate-kind constants equal the header's values."""
import re
from pathlib import Path

from quantr_gb300 import _native

ROOT = Path(__file__).resolve().parent.parent
HDR = (ROOT / "include" / "qgpu.h").read_text()
FFI = (ROOT / "rust" / "quantr-gpu" / "src" / "ffi.rs").read_text()

C_SCALARS = {"int": (4, True), "int32_t": (4, True), "uint32_t": (4, True), "size_t": (8, True),
             "uint64_t": (8, True), "int64_t": (8, True), "double": (8, False), "char": (1, True),
             "uint8_t": (1, True), "void": (0, True)}
R_SCALARS = {"c_int": (4, True), "i32": (4, True), "u32": (4, True), "usize": (8, True),
             "u64": (8, True), "i64": (8, True), "f64": (8, False), "c_char": (1, True),
             "u8": (1, True), "c_void": (0, True)}


def _strip_comments(s):
    return re.sub(r"/\*.*?\*/", "", re.sub(r"//[^\n]*", "", s), flags=re.S)


def c_functions():
    out = {}
    for ret, name, args in re.findall(r"^\s*((?:const\s+)?[a-z_0-9]+\s*\*?)\s*(qgpu_\w+)\s*\(([^)]*)\);",
                                      _strip_comments(HDR), re.M):
        params = [] if args.strip() == "void" else [a.strip() for a in args.split(",")]
        out[name] = (ret.replace(" ", ""), params)
    return out


def c_param(p):
    ptr = p.count("*")
    base = re.sub(r"\b(const|struct)\b", "", p.replace("*", " ")).split()[0]
    if base.startswith("qgpu_"):
        return ("opaque" if base == "qgpu_handle" else base, ptr)
    return (C_SCALARS[base], ptr)


def rust_functions():
    block = _strip_comments(FFI[FFI.index('extern "C" {'):])
    out = {}
    for name, args, ret in re.findall(r"pub fn (qgpu_\w+)\s*\(([^)]*)\)\s*(?:->\s*([^;]+))?;", block, re.S):
        params = [a.split(":", 1)[1].strip() for a in args.split(",") if a.strip()]
        out[name] = ((ret or "").strip(), params)
    return out


def r_param(p):
    ptr = p.count("*mut") + p.count("*const")
    base = p.replace("*mut", "").replace("*const", "").strip()
    if base.startswith("Qgpu"):
        return ({"QgpuHandle": "opaque", "QgpuOp": "qgpu_op", "QgpuBatchItem": "qgpu_batch_item"}[base], ptr)
    return (R_SCALARS[base], ptr)


def test_every_entry_point_is_declared_with_matching_parameters():
    cf, rf = c_functions(), rust_functions()
    assert len(cf) >= 27 and set(cf) == set(rf), set(cf) ^ set(rf)
    for name, (_, cparams) in cf.items():
        rparams = rf[name][1]
        assert len(cparams) == len(rparams), name
        for cp, rp in zip(cparams, rparams):
            assert c_param(cp) == r_param(rp), (name, cp, rp)


def _c_struct(name):
    body = re.search(r"typedef struct " + name + r"\s*\{(.*?)\}\s*" + name + ";", _strip_comments(HDR), re.S).group(1)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        m = re.match(r"([a-z_0-9]+)\s+(\w+)(?:\[(\w+)\])?", decl)
        typ, fname, arr = m.groups()
        count = 1 if arr is None else (10 if arr == "QGPU_MAX_OP_WIRES" else int(arr))
        fields.append((fname, C_SCALARS[typ][0], count))
    return fields


def _rust_struct(name):
    body = re.search(r"pub struct " + name + r"\s*\{(.*?)\}", _strip_comments(FFI), re.S).group(1)
    fields = []
    for decl in body.split(","):
        decl = decl.strip()
        if not decl:
            continue
        fname, typ = [x.strip() for x in decl.replace("pub ", "").split(":")]
        m = re.match(r"\[(\w+);\s*(\w+)\]", typ)
        if m:
            fields.append((fname, R_SCALARS[m.group(1)][0], 10 if m.group(2) == "QGPU_MAX_OP_WIRES" else int(m.group(2))))
        else:
            fields.append((fname, R_SCALARS[typ][0], 1))
    return fields


def _layout(fields):
    off, out, align = 0, [], 1
    for fname, size, count in fields:
        off = (off + size - 1) // size * size
        out.append((fname, off))
        off += size * count
        align = max(align, size)
    return out, (off + align - 1) // align * align


def test_repr_c_structs_match_the_header():
    for c_name, r_name in (("qgpu_op", "QgpuOp"), ("qgpu_batch_item", "QgpuBatchItem")):
        assert _layout(_c_struct(c_name)) == _layout(_rust_struct(r_name)), c_name
    offs, size = _layout(_rust_struct("QgpuOp"))
    assert size == 80
    for fname, off in offs:
        assert getattr(_native.QgpuOp, fname).offset == off, fname


def test_constants_match_the_header():
    consts = dict((k, int(v)) for k, v in re.findall(r"pub const (QGPU_\w+): [\w:]+ = (-?\d+);", FFI))
    for k, v in re.findall(r"#define (QGPU_\w+)\s+(-?\d+)", HDR):
        assert consts[k] == int(v), k
    kinds = re.search(r"enum qgpu_gate_kind \{(.*?)\};", HDR, re.S).group(1)
    names = [n.strip() for n in re.sub(r"=\s*0", "", kinds).replace("\n", " ").split(",") if n.strip()]
    for i, n in enumerate(names):
        assert consts[n] == i, n
