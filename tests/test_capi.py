"""The C-ABI library builds for sm_103a, loads, and exports every function that
include/clowns_gpu.h declares (no GPU needed: no compute calls)."""
import subprocess


def test_library_builds_and_exports_all_declared_symbols(pkg):
    lib_path = pkg.build()
    L = pkg.lib()
    declared = pkg.declared_symbols()
    assert len(declared) >= 10
    missing = [s for s in declared if not hasattr(L, s)]
    assert not missing, missing
    nm = subprocess.run(["nm", "-D", "--defined-only", str(lib_path)], capture_output=True, text=True).stdout
    exported = {ln.split()[-1] for ln in nm.splitlines() if " T " in ln}
    assert set(declared) <= exported


def test_library_is_sm103a(pkg):
    lib_path = pkg.build()
    out = subprocess.run(["/usr/local/cuda/bin/cuobjdump", "--list-elf", str(lib_path)],
                         capture_output=True, text=True).stdout
    assert "sm_103a" in out


def test_version_and_error_string(pkg):
    L = pkg.lib()
    assert L.clowns_version() >= 10000
    assert isinstance(pkg.last_error(), str)
