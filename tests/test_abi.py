"""The C ABI boundary (no GPU): the library loads, exports every symbol that
include/phgb300.h declares, and every declaration names the reference function
it replaces or says it has no counterpart."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "phgb300.h"


def _declared():
    text = HEADER.read_text()
    return re.findall(r"^PH_API\s+[\w\s\*]+?\b(ph_\w+)\s*\(", text, flags=re.M)


def test_header_declares_entry_points():
    names = _declared()
    assert len(names) >= 20
    for must in ("ph_reconst_xyproj", "ph_reconst_vol", "ph_phase_retrieval", "ph_ccl", "ph_ccl_roots",
                 "ph_transfer", "ph_transfer_sqrt", "ph_asm_prop", "ph_reconst_vol_padded", "ph_pad2d"):
        assert must in names


def test_library_loads_and_exports_every_symbol(ph):
    from ph_gb300 import _lib
    lib = _lib.lib()
    assert lib.ph_version() >= 100
    for name in _declared():
        assert hasattr(lib, name), f"{name} declared in phgb300.h but not exported"
        assert name in _lib.SIGNATURES, f"{name} has no ctypes signature"
    assert set(_lib.SIGNATURES) == set(_declared())


def test_every_declaration_cites_reference():
    text = HEADER.read_text()
    blocks = re.split(r"\n(?=/\*)", text)
    for name in _declared():
        if name in ("ph_create", "ph_destroy", "ph_last_error", "ph_version", "ph_set_option",
                    "ph_scratch_bytes", "ph_reserve", "ph_kernel_launches", "ph_profile_report",
                    "ph_noalloc_last_error"):
            continue
        block = next(b for b in blocks if re.search(rf"\b{name}\s*\(", b))
        low = block.lower()
        assert re.search(r"\.jl:\d+", block) or "no reference counterpart" in low or "no counterpart" in low, name


def test_null_context_is_rejected(ph):
    from ph_gb300 import _lib
    lib = _lib.lib()
    assert lib.ph_reconst_xyproj(None, None, None, None, None, None, 8, 8, 1, None) == _lib.PH_ERR_INVALID
    assert lib.ph_set_option(None, 1, 1) == _lib.PH_ERR_INVALID
    assert lib.ph_last_error(None) == b"null context"


def test_create_without_gpu_fails_cleanly(ph):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from ph_gb300 import _lib
    h = ctypes.c_void_p()
    assert _lib.lib().ph_create(0, 0, ctypes.byref(h)) == _lib.PH_ERR_CUDA
    assert not h.value


@pytest.mark.timeout(60)
def test_default_context_without_gpu_raises(ph):
    """The first context creation loads the library and fails cleanly (no deadlock) without a GPU."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from ph_gb300 import _lib
    with pytest.raises(_lib.PhError, match="ph_create"):
        _lib.default_context(0)


def test_host_mirror_validates_before_launch(ph):
    """Size and dtype checks happen on the host with the reference's messages."""
    import torch
    a = torch.zeros((4, 4), dtype=torch.complex64)
    b = torch.zeros((8, 8), dtype=torch.complex64)
    with pytest.raises(AssertionError, match="All arrays must have the same size. Got \\(4, 4\\), \\(8, 8\\)"):
        ph.cu_get_reconst_xyprojection(ph.CuWavefront(a), ph.CuTransfer(b), ph.CuTransfer(a), 2)
    with pytest.raises(TypeError):
        ph.cu_get_reconst_xyprojection(ph.CuWavefront(a.real.contiguous()), ph.CuTransfer(a), ph.CuTransfer(a), 2)
    with pytest.raises(AssertionError, match="2\\*size"):
        ph.cu_get_reconst_vol_and_xyprojection_padded(ph.CuWavefront(a), ph.CuTransfer(a), ph.CuTransfer(a), 2)


def _split_top(s: str) -> list:
    """Top-level comma split of a parenthesis-free-at-top string."""
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "({[":
            depth += 1
        elif ch in ")}]":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur.strip())
    return out


def _close(s: str, i: int) -> int:
    """Index of the parenthesis closing the one at s[i]."""
    depth = 0
    for k in range(i, len(s)):
        depth += s[k] == "("
        depth -= s[k] == ")"
        if depth == 0:
            return k
    raise ValueError("unbalanced")


def test_julia_ccalls_match_header_arity():
    """Every ccall of the Julia binding passes as many argument types as the C
    declaration has parameters (the binding cannot run without Julia)."""
    hdr = (ROOT / "include" / "phgb300.h").read_text()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)   # declarations only
    arity, c_params = {}, {}
    for m in re.finditer(r"\b(ph_[a-z0-9_]+)\s*\(", hdr):
        start = m.end() - 1
        params = hdr[start + 1:_close(hdr, start)].strip()
        if params and params != "void" and not params.startswith("*"):
            c_params[m.group(1)] = _split_top(params)
            arity[m.group(1)] = len(c_params[m.group(1)])
        elif params in ("", "void"):
            c_params[m.group(1)] = []
            arity[m.group(1)] = 0
    jl = (ROOT / "particleholography.jl_gb300" / "julia" / "ParticleHolographyGB300.jl").read_text()
    checked = 0
    for m in re.finditer(r"ccall\(\(:(ph_[a-z0-9_]+), libphgb300\),", jl):
        name = m.group(1)
        rest = jl[m.end():]
        ret = _split_top(rest[:rest.index("(")] + "x")[0]   # the return type, up to the type tuple
        i = rest.index("(")
        types = _split_top(rest[i + 1:_close(rest, i)])
        assert name in arity, name
        assert len(types) == arity[name], (name, len(types), arity[name], ret)
        for jt, ct in zip(types, c_params[name]):
            assert _kind_jl(jt) == _kind_c(ct), (name, jt, ct)
        checked += 1
    assert checked >= 20


def _kind_c(param: str) -> str:
    p = param.replace("const ", "").strip()
    if "*" in p:
        return "ptr"
    t = p.split()[0]
    return {"int32_t": "i32", "int64_t": "i64", "double": "f64", "float": "f32", "size_t": "size",
            "uint32_t": "u32"}.get(t, t)


def _kind_jl(t: str) -> str:
    t = t.strip()
    if t.startswith(("Ptr{", "CuPtr{", "Ref{", "Cstring")):
        return "ptr"
    return {"Int32": "i32", "Int64": "i64", "Float64": "f64", "Float32": "f32", "Csize_t": "size",
            "UInt32": "u32"}.get(t, t)
