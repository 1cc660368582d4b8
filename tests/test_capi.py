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


def test_will_dropin_rejects_bad_arguments_without_a_gpu(pkg):
    """PCGPME_WILL's drop-in validates its arguments before any device work: a
    zero order, a leading dimension below n, NL other than 4 or 6, or ITER < 1
    return CLOWNS_ERR_ARG (the reference has no error argument; B is left as it
    was) with a message; the workspace query answers 0 for invalid sizes."""
    import ctypes as C
    import numpy as np
    L = pkg.lib()
    n = 8
    al = np.zeros((4, n))
    ll = np.zeros((4, n), dtype=np.int32)
    d = np.ones(n)
    b = np.arange(n, dtype=np.float64)
    b0 = b.copy()

    def call(nl, na, nn, it):
        c = [C.c_int(v) for v in (nl, na, nn, 64, it)]
        e, p = C.c_double(1e-10), C.c_double(5.0)
        return L.pcgpme_will_gpu(al.ctypes.data, C.addressof(c[0]), C.addressof(c[1]), ll.ctypes.data,
                                 d.ctypes.data, C.addressof(c[2]), C.addressof(c[3]), b.ctypes.data,
                                 C.addressof(e), C.addressof(p), C.addressof(c[4]))

    for args in [(4, n, 0, 10), (4, n - 1, n, 10), (5, n, n, 10), (4, n, n, 0)]:
        rc = call(*args)
        assert rc == -2, (args, rc)             # CLOWNS_ERR_ARG
        assert "pcgpme_will" in pkg.last_error()
        assert np.array_equal(b, b0)
    assert L.clowns_pcgpme_will_workspace_bytes(0, 4) == 0
    assert L.clowns_pcgpme_will_workspace_bytes(100, 5) == 0
    assert L.clowns_pcgpme_will_workspace_bytes(100, 4) > 0
