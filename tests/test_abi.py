"""The C ABI library builds for sm_103a, loads, and exports every symbol include/gdt_gb300.h declares
(no compute calls: this runs without a GPU)."""
import os
import re

from conftest import ROOT, import_gdt


def declared_symbols():
    with open(os.path.join(ROOT, "include", "gdt_gb300.h")) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gdt_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "gdt_solve" in syms and "gdt_assemble_cg_diffusion" in syms and "gdt_fv_timestep" in syms


def test_library_exports_every_declared_symbol():
    gdt = import_gdt()
    gdt._build.build()
    L = gdt._capi.load()
    for name in declared_symbols():
        assert hasattr(L, name), name
    # every declared symbol also has a ctypes signature
    assert set(declared_symbols()) <= set(gdt._capi.symbols())


def test_library_is_sm103a_and_in_tree():
    gdt = import_gdt()
    path = gdt._build.build()
    assert path.startswith(os.path.join(ROOT, "dune-gdt_gb300"))
    assert "arch=compute_103a,code=sm_103a" in " ".join(gdt._build.ARCH)
