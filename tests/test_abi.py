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
