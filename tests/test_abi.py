"""The C-ABI library builds, loads and exports every symbol include/bsa_gpu.h declares
(no compute call: this runs without a GPU)."""
import ctypes
import subprocess

from bsalib_gb300 import api


def test_header_declares_the_reference_surfaces():
    syms = api.header_symbols()
    for s in ("bsa_Init", "bsa_Run", "bsa_Finalise", "bsaclInit", "bsaclInitDeviceMemory", "bsaclRun",
              "bsaclFinalise", "bsa_gpu_clsBispectra", "bsa_gpu_mshBispectra"):
        assert s in syms


def test_library_exports_every_declared_symbol(bsalib):
    missing = [s for s in api.header_symbols() if not hasattr(bsalib, s)]
    assert not missing, missing


def test_exports_are_plain_c(bsalib):
    out = subprocess.run(["nm", "-D", "--defined-only", api.LIB_PATH], capture_output=True, text=True).stdout
    names = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    for s in api.header_symbols():
        assert s in names, s          # unmangled, i.e. extern "C"


def test_library_is_sm103a_only(bsalib):
    from bsalib_gb300 import build
    assert "arch=compute_103a,code=sm_103a" in " ".join(build.ARCH)


def test_batch_host_checks(bsalib):
    # host-side checks of the batched sweep, before any device work
    assert bsalib.bsa_gpu_batchClear() == 0
    nm, nf = ctypes.c_int(0), ctypes.c_int(0)
    assert bsalib.bsa_gpu_batchCase(-1, ctypes.byref(nm), ctypes.byref(nf)) == -1
    assert bsalib.bsa_gpu_batchCase(0, ctypes.byref(nm), ctypes.byref(nf)) == -1
    assert bsalib.bsa_gpu_batchRun(None, None, None, None, None) == -2
    assert b"empty batch" in bsalib.bsa_lastError()


def test_struct_layouts_match_the_header(tmp_path):
    # sizes and field offsets of the header's structs, from a C program compiled against it,
    # against the ctypes mirrors the binding passes through the C-ABI
    import os
    fields = {
        "bsa_zone": (api.Zone, [f[0] for f in api.Zone._fields_]),
        "bsa_triangle": (api.Triangle, [f[0] for f in api.Triangle._fields_]),
        "bsa_gpu_stats": (api.Stats, [f[0] for f in api.Stats._fields_]),
    }
    lines = ["#include <stddef.h>", "#include <stdio.h>", f'#include "{os.path.abspath(api.HEADER)}"', "int main(void) {"]
    for st, (_, names) in fields.items():
        lines.append(f'    printf("{st} size %zu\\n", sizeof({st}));')
        for n in names:
            lines.append(f'    printf("{st} {n} %zu\\n", offsetof({st}, {n}));')
    lines += ["    return 0;", "}"]
    src, exe = tmp_path / "layout.c", tmp_path / "layout"
    src.write_text("\n".join(lines) + "\n")
    subprocess.run(["gcc", "-std=c11", "-o", str(exe), str(src)], check=True)
    got = {}
    for ln in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        st, what, val = ln.split()
        got[(st, what)] = int(val)
    for st, (cls, names) in fields.items():
        assert got[(st, "size")] == ctypes.sizeof(cls), st
        for n in names:
            assert got[(st, n)] == getattr(cls, n).offset, (st, n)
